"""The C-ABI library builds, loads and exports every symbol include/cpetgb.h
declares; the Python binding declares every one of them; without a GPU the
library refuses work instead of falling back to the CPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def header_symbols():
    with open(os.path.join(ROOT, "include", "cpetgb.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"^\s*int\s+(cpetgb_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def built():
    from pycpet_gb300 import build

    return build.build_library()


def test_library_exports_header_symbols(built):
    syms = header_symbols()
    assert len(syms) >= 17
    L = ctypes.CDLL(built)
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_binding_covers_header(built):
    from pycpet_gb300 import _lib

    assert set(header_symbols()) == set(_lib.SIGNATURES)
    L = _lib.lib()
    assert L.cpetgb_version() >= 10000
    assert L.cpetgb_get_default_precision() == _lib.FP32C
    assert L.cpetgb_set_default_precision(7) == _lib.EINVAL
    assert "precision" in _lib.last_error()


def test_no_cpu_fallback(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    from pycpet_gb300 import CpetgbError, field_grid

    with pytest.raises(CpetgbError) as e:
        field_grid(np.zeros((4, 3)), np.ones((2, 3)), np.ones(2))
    assert e.value.code == -5  # CPETGB_ENODEV


def test_argument_validation_before_device(built):
    """Shape errors are reported as EINVAL before any device work."""
    from pycpet_gb300 import _lib

    L = _lib.lib()
    assert L.cpetgb_field_grid(3, 0, 1, 1, None, None, None, 1, None, None) == _lib.EINVAL
    assert L.cpetgb_topo_hist2d(0, 1, None, 0, 20, None, None, None, None) == _lib.EINVAL


def test_argument_validation_new_entry_points(built):
    """The clustering, writer, preparation and dipole entry points refuse bad
    arguments with a status and a message, before any device work."""
    import ctypes

    import numpy as np
    from pycpet_gb300 import _lib

    L = _lib.lib()
    h = np.zeros((2, 3))
    out = np.zeros((2, 2))
    assert L.cpetgb_chi2_distance_matrix(7, 0, 2, 3, h.ctypes.data, out.ctypes.data, None) == _lib.EINVAL
    assert L.cpetgb_field_distance_matrix(1, 0, -1, 3, h.ctypes.data, out.ctypes.data, None) == _lib.EINVAL
    assert L.cpetgb_chi2_distance_matrix(1, 0, 2, 3, None, out.ctypes.data, None) == _lib.EINVAL
    off = np.array([0, 1], np.int64)
    rng = np.array([0.0, 1.0, 0.0, 1.0])
    vals = np.zeros((1, 2))
    cnt = np.zeros(4, np.uint64)
    assert L.cpetgb_topo_hist2d_sets(0, 1, off.ctypes.data, vals.ctypes.data, 0, 4, rng.ctypes.data,
                                     cnt.ctypes.data, None, None) == _lib.EINVAL
    bad = np.array([0.0, np.nan, 0.0, 1.0])
    assert L.cpetgb_topo_hist2d_sets(0, 1, off.ctypes.data, vals.ctypes.data, 2, 2, bad.ctypes.data,
                                     cnt.ctypes.data, None, None) == _lib.ERANGE
    length = ctypes.c_int64(0)
    v = np.zeros((2, 3), np.float32)
    assert L.cpetgb_format_fixed3(0, 2, 0, v.ctypes.data, None, 0, ctypes.byref(length), None) == _lib.EINVAL
    x, q, c = np.zeros((4, 3)), np.zeros(4), np.zeros(3)
    n_out = ctypes.c_int(0)
    assert L.cpetgb_prepare_frame(0, 4, x.ctypes.data, q.ctypes.data, None, None, c.ctypes.data, None, 2.0,
                                  None, None, x.ctypes.data, q.ctypes.data, ctypes.byref(n_out), None) == _lib.EINVAL
    assert "resid" in _lib.last_error()
    assert L.cpetgb_topo_dipole_lines(5, 0, 1, 1, x.ctypes.data, None, 0.1, c.ctypes.data, x.ctypes.data,
                                      x.ctypes.data, out.ctypes.data, None, None, None) == _lib.EINVAL
    assert L.cpetgb_engine_set_ctas_per_sm(None, 2) == _lib.EINVAL
    assert L.cpetgb_format_sci18(0, 2, 0, v.ctypes.data, None, 0, ctypes.byref(length), None) == _lib.EINVAL
    assert L.cpetgb_format_sci18(5, 2, 3, v.ctypes.data, None, 0, ctypes.byref(length), None) == _lib.EINVAL


def test_settings_and_checks_validate_arguments(built):
    """Process-wide settings and the wait-limit check refuse bad values before
    any device work; the per-call precision variants refuse bad precisions."""
    import numpy as np
    from pycpet_gb300 import _lib

    L = _lib.lib()
    old = L.cpetgb_field_refinement()
    assert 0.0 <= old <= 1.0
    for bad in (-0.5, 1.5, float("nan"), float("inf")):
        assert L.cpetgb_set_field_refinement(bad) == _lib.EINVAL
        assert "refinement" in _lib.last_error()
    assert L.cpetgb_field_refinement() == old
    assert L.cpetgb_set_field_refinement(0.25) == _lib.OK and L.cpetgb_field_refinement() == 0.25
    assert L.cpetgb_set_field_refinement(old) == _lib.OK
    for bad in (0.0, -1.0, 2.5, float("nan")):
        assert L.cpetgb_check_wait_limit(bad) == _lib.EINVAL
    x0 = np.zeros((1, 3), np.float32)
    E = np.zeros((1, 3), np.float32)
    assert L.cpetgb_compute_looped_field_p(7, 1, 1, x0.ctypes.data, x0.ctypes.data, x0.ctypes.data,
                                           E.ctypes.data) == _lib.EINVAL


def test_tuning_table_round_trip(built):
    """The autotuner table is host state: keys, bounds and removal."""
    from pycpet_gb300 import _lib

    L = _lib.lib()
    assert L.cpetgb_tune_variants(0) == 14 and L.cpetgb_tune_variants(1) == 2
    k_small = L.cpetgb_tune_key(0, 1, 0, 1e5)
    k_big = L.cpetgb_tune_key(0, 1, 0, 1e10)
    assert k_small >= 0 and k_big > k_small
    assert L.cpetgb_tune_get(k_big) == -1
    assert L.cpetgb_tune_set(k_big, 4) == 0 and L.cpetgb_tune_get(k_big) == 4
    assert L.cpetgb_tune_set(k_big, 14) == _lib.EINVAL      # no such variant
    assert L.cpetgb_tune_set(k_big, -1) == 0 and L.cpetgb_tune_get(k_big) == -1
    kt = L.cpetgb_tune_key(1, 1, 1, 1e5)
    assert L.cpetgb_tune_set(kt, 2) == _lib.EINVAL and L.cpetgb_tune_set(kt, 1) == 0
    assert L.cpetgb_tune_set(kt, -1) == 0
    assert L.cpetgb_tune_key(7, 1, 0, 1.0) == _lib.EINVAL


def test_shipped_tuning_table_is_valid(built):
    """Every entry of the shipped GB300 table names an existing variant of a
    valid key (grid keys: op 0; streamline keys: op 1)."""
    import json
    import os

    from conftest import ROOT
    from pycpet_gb300 import _lib

    L = _lib.lib()
    with open(os.path.join(ROOT, "pycpet_gb300", "tuned", "nvidia_gb300.json")) as fh:
        table = json.load(fh)["table"]
    assert table
    for k, v in table.items():
        op = int(k) >> 12
        assert op in (0, 1)
        assert 0 <= v < L.cpetgb_tune_variants(op), (k, v)
        before = L.cpetgb_tune_get(int(k))  # restored: the table is process state
        assert L.cpetgb_tune_set(int(k), v) == 0
        assert L.cpetgb_tune_get(int(k)) == v
        assert L.cpetgb_tune_set(int(k), before) == 0
