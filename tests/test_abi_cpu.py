"""C-ABI library checks that need no GPU: it loads, exports every symbol
that include/sm2d.h declares, and its host tables (grids, R-LUT) are
bit-exact with the reference's host code (fixtures in tests/golden/)."""
import os
import re

import numpy as np
import pytest

import sm_2d_gb300 as sm
from golden_cases import DEFAULT_GROUPS, host_tables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sm2d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sm2d_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = sm.lib()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_grids_match_reference_tables():
    T = host_tables()
    e, r = sm.energy_grid_piecewise(DEFAULT_GROUPS)
    assert np.array_equal(e, np.float32(T["piecewise_default"]["edges"]))
    e, r = sm.energy_grid_log(0.1, 250.0, 256)
    assert np.array_equal(e, np.float32(T["log_0.1_250_256"]["edges"]))
    assert np.array_equal(r, np.float32(T["log_0.1_250_256"]["rep"]))
    lut = sm.range_lut(r)
    for k in ("R", "S", "logE", "logR", "logS"):
        assert np.array_equal(lut[k], np.float32(T["log_0.1_250_256"][k])), k
    th, _ = sm.angular_grid(np.float32(-np.pi / 2), np.float32(np.pi / 2), 512)
    assert np.array_equal(th, np.float32(T["theta_pi2_512"]["edges"]))


def test_fermi_eyges_matches_oracle(oracle_mod):
    for args in [(150.0, 400, 0.5, 3.8), (70.0, 120, 0.5, 0.0), (230.0, 600, 0.5, 5.0)]:
        got = sm.fermi_eyges(*args)
        want = oracle_mod.fe_precompute(*args)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_host_table_argument_errors():
    with pytest.raises(sm.Sm2dError):
        sm.energy_grid_log(0.0, 1.0, 4)
    with pytest.raises(sm.Sm2dError):
        sm.angular_grid(1.0, 0.0, 4)


def test_bucket_layout_size():
    # DeviceOutflowBucket: 32 ids, 32 counts, 32 x L floats, 3 moments
    assert sm.lib().sm2d_bucket_bytes(256) == 32972
    assert sm.lib().sm2d_bucket_bytes(128) == 16588


def _k5_args(nt_local, n_e_local, n_e, local_bins, n_cells=16):
    import ctypes as C
    P = C.c_void_p
    return ([P(16)] * 18 + [C.c_float(0), C.c_float(0), C.c_double(0), C.c_double(0), C.c_float(0),
                            C.c_double(0), C.c_int(1), P(16), C.c_int(n_e), C.c_int(nt_local), C.c_int(n_e_local),
                            C.c_int(local_bins), P(16), C.c_int(n_cells), P(None)])


@pytest.mark.parametrize("entry", ["sm2d_k5_conservation_audit", "sm2d_k5_conservation_audit_static"])
def test_k5_entries_refuse_bad_layouts(entry):
    """Both K5 entries refuse a local-bin count other than 128/256 and
    non-positive layout counts before touching the device (the kernel divides
    by nt_local and N_E_local and reads local_bins values per slot)."""
    fn = getattr(sm.lib(), entry)
    assert fn(*_k5_args(4, 2, 1029, 100)) == -6     # SM2D_ERR_LAYOUT
    assert fn(*_k5_args(0, 2, 1029, 256)) == -1     # SM2D_ERR_ARG
    assert fn(*_k5_args(4, 0, 1029, 256)) == -1
    assert fn(*_k5_args(4, 2, 0, 256)) == -1
    assert fn(*_k5_args(3, 2, 1029, 256)) == -1     # 256 local bins are not a whole number of (3 x 2) groups
