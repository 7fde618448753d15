"""Host-side admission rules and the pending watchdog of the serving loop
(pycpet_gb300.serving): requests that can never run are refused with a
reason, and requests waiting too long are cancelled.  No GPU needed."""
import numpy as np

from pycpet_gb300.serving import Request, expire_pending, validate_request

FRAMES = {0: None, 1: None}
BIG = 1 << 40


def test_valid_requests_pass():
    pts = np.zeros((5, 3))
    for kind in ("point_field", "volume", "volume_esp"):
        assert validate_request(Request(kind, 0, points=pts), FRAMES, BIG) is None
    r = Request("topo", 1, starts=np.zeros((4, 3)), n_iter=[10, 20, 30, 0])
    assert validate_request(r, FRAMES, BIG) is None


def test_refusals():
    pts = np.zeros((5, 3))
    cases = [
        (Request("magnet", 0, points=pts), "unknown request kind"),
        (Request("volume", 7, points=pts), "not resident"),
        (Request("volume", 0, points=np.zeros((0, 3))), "at least one point"),
        (Request("volume", 0, points=np.array([[0.0, np.nan, 0.0]])), "finite"),
        (Request("point_field", 0, points=None), "needs points"),
        (Request("topo", 0, starts=np.array([[np.inf, 0, 0]]), n_iter=5), "finite"),
        (Request("topo", 0, starts=np.zeros((0, 3)), n_iter=5), "at least one start"),
        (Request("topo", 0, starts=np.zeros((2, 3)), n_iter=[1, 2, 3]), "step caps"),
        (Request("topo", 0, starts=np.zeros((2, 3)), n_iter=-1), "step caps"),
        (Request("topo", 0, starts=np.zeros((2, 3)), n_iter=(1 << 24) + 1), "step caps"),
        (Request("topo", 0, starts=np.zeros((2, 3)), n_iter=5, step=float("nan")), "step must be finite"),
        (Request("topo", 0, starts=np.zeros((2, 3)), n_iter=5, half_dims=(1, -1, 1)), "half_dims"),
    ]
    for req, words in cases:
        why = validate_request(req, FRAMES, BIG)
        assert why is not None and words in why, (req.kind, why)


def test_budget_refusal():
    r = Request("volume", 0, points=np.zeros((1000, 3)))
    assert validate_request(r, FRAMES, r.bytes_needed()) is None
    why = validate_request(r, FRAMES, r.bytes_needed() - 1)
    assert why is not None and "budget" in why


def test_pending_deadline():
    reqs = [Request("volume", 0, arrival=t, points=np.zeros((1, 3))) for t in (0.0, 1.0, 2.0, 3.0)]
    kept, expired = expire_pending(reqs, now=3.5, deadline_s=2.0)
    assert [r.arrival for r in expired] == [0.0, 1.0]
    assert [r.arrival for r in kept] == [2.0, 3.0]
    kept, expired = expire_pending(reqs, now=100.0, deadline_s=None)
    assert len(kept) == 4 and not expired
