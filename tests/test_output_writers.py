"""Depth-dose metrics and output files against the reference's own writers
(save_dose_2d / save_pdd, run_simulation.cpp:31-114; get_depth_dose /
find_bragg_peak_z, deterministic_beam.cpp:207-236; bragg_peak.cpp), whose
outputs on seeded synthetic dose grids are stored in tests/golden/writers/
(made by tests/golden/make_golden.py).  Host code: no GPU."""
import json
import os

import numpy as np
import pytest

import sm_2d_gb300 as sm

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "writers")
CASES = sorted(os.listdir(GOLD))


def _load(case):
    raw = open(os.path.join(GOLD, case, "dose.bin"), "rb").read()
    nx, nz = np.frombuffer(raw[:8], np.int32)
    dx, dz = np.frombuffer(raw[8:16], np.float32)
    dose = np.frombuffer(raw[16:], np.float64).reshape(nz, nx)
    return dose, float(dx), float(dz)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("normalize", [False, True])
def test_files_are_byte_identical(case, normalize, tmp_path):
    dose, dx, dz = _load(case)
    suffix = "_norm" if normalize else ""
    sm.write_dose_2d(str(tmp_path / "d.txt"), dose, dx, dz, normalize)
    sm.write_pdd(str(tmp_path / "p.txt"), dose, dz, normalize)
    assert (tmp_path / "d.txt").read_bytes() == open(os.path.join(GOLD, case, f"dose_2d{suffix}.txt"), "rb").read()
    assert (tmp_path / "p.txt").read_bytes() == open(os.path.join(GOLD, case, f"pdd{suffix}.txt"), "rb").read()


@pytest.mark.parametrize("case", CASES)
def test_metrics_match(case):
    dose, dx, dz = _load(case)
    want = json.load(open(os.path.join(GOLD, case, "metrics.json")))
    assert sm.bragg_peak_row(dose) == want["bragg_peak_row"]
    got = sm.bragg_metrics(dose, dz)
    for k in sm.runtime.BRAGG_KEYS:
        assert np.float32(got[k]) == np.float32(want[k]), (k, got[k], want[k])
    pdd = sm.depth_dose(dose)
    ref = [sum(row[i] for i in range(dose.shape[1])) for row in dose]   # sequential, as the reference sums
    assert np.array_equal(pdd, np.array(ref), equal_nan=True)


def test_nan_cells_print_as_zero():
    dose, dx, dz = _load("nan_cell")
    assert np.isnan(dose).sum() == 1
    text = open(os.path.join(GOLD, "nan_cell", "dose_2d.txt")).read()
    assert "nan" not in text.lower()


def test_bad_arguments_are_refused(tmp_path):
    with pytest.raises(sm.Sm2dError):
        sm.write_pdd(str(tmp_path / "missing_dir" / "p.txt"), np.ones((3, 2)), 0.5)
    with pytest.raises(ValueError):
        sm.depth_dose(np.ones(4))
