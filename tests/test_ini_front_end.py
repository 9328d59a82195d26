"""The INI front end (sm2d_load_ini, sm2d_run_simulation, the run_simulation
command): the reference's configuration files parse into the problem and
beam its runner builds (config_loader.hpp:98-413, gpu_transport_runner.cpp:
28-105), pinned on the reference's own case files (tests/golden/
one_step_case_*/case.ini) against its grid tables; the parsing rules,
defaults and errors; and, on a GPU, the run_simulation command against the
same spot run through the Transport API."""
import os
import subprocess

import numpy as np
import pytest

import sm_2d_gb300 as sm
from sm_2d_gb300 import runtime as rt
from golden_cases import GOLDEN, host_tables, load_case

LIB_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "sm_2d_gb300", "_lib")


@pytest.mark.parametrize("case", "ABCD")
def test_reference_case_files(case):
    cfg, beam, run = rt.load_ini(os.path.join(GOLDEN, f"one_step_case_{case}", "case.ini"))
    want = load_case(case)
    wc, wb = want["cfg"], want["beam"]
    for k in ("Nx", "Nz", "dx", "dz", "x_min", "z_min", "E_fine_on", "E_fine_off", "weight_active_min",
              "step_coarse", "sigma_x_initial", "E0"):
        assert np.float32(getattr(cfg, k)) == np.float32(wc[k]), (k, getattr(cfg, k), wc[k])
    assert np.array_equal(cfg.theta_edges, want["theta_edges"])
    assert np.array_equal(cfg.E_edges, np.asarray(host_tables()["piecewise_default"]["edges"], np.float32))
    assert cfg.layout == dict(nt_local=4, ne_local=2, nx_sub=8, nz_sub=4)
    got_b = dict(x0=beam.x0, z0=beam.z0, theta0=beam.theta0, E0=beam.E0, W=beam.W_total, sigma_x=beam.sigma_x,
                 sigma_theta=beam.sigma_theta, sigma_E=beam.sigma_E, n_samples=beam.n_samples, seed=beam.seed)
    for k, v in wb.items():
        assert np.float32(got_b[k]) == np.float32(v), (k, got_b[k], v)
    assert run["max_iterations"] == 1 and not run["save_2d"] and not run["save_pdd"]


def _write(tmp_path, text):
    p = tmp_path / "sim.ini"
    p.write_text(text)
    return str(p)


def test_parsing_rules_and_defaults(tmp_path):
    path = _write(tmp_path, """
stray = 1            ; a key before any section
# a comment
[energy]
mean_MeV = "70.5"
mean_MeV = 71.0
 [ grid ]
Nx=30
Nz = 40
dx_mm = 0.25mm
[transport]
E_trigger = 12.0
energy_groups = 1:10:0.5, 10:100:1
N_theta = 24
[output]
output_dir = 'out dir'
normalize_dose = Yes
save_pdd = off
""")
    cfg, beam, run = rt.load_ini(path)
    assert beam.E0 == np.float32(71.0) and cfg.E0 == np.float32(71.0)   # the later key wins
    assert (cfg.Nx, cfg.Nz) == (30, 40) and cfg.dx == np.float32(0.25) and cfg.dz == np.float32(1.0)
    assert cfg.x_min == np.float32(-(30 * np.float32(0.25)) / 2)
    # legacy trigger: E_fine_on follows it, E_fine_off = max(11, on)
    assert cfg.E_fine_on == np.float32(12.0) and cfg.E_fine_off == np.float32(12.0)
    edges, _ = sm.energy_grid_piecewise([(1.0, 10.0, 0.5), (10.0, 100.0, 1.0)])
    assert np.array_equal(cfg.E_edges, edges)
    th, _ = sm.angular_grid(-0.35, 0.35, 24)
    assert np.array_equal(cfg.theta_edges, th)
    assert run["max_iterations"] == 100                      # max_iterations 0 -> grid.max_steps
    assert run["output_dir"] == "out dir" and run["normalize_dose"] and not run["save_pdd"] and run["save_2d"]
    assert beam.n_samples == 1000 and beam.seed == 42 and beam.W_total == np.float32(1.0)


def test_malformed_energy_groups_keep_the_default(tmp_path):
    cfg, _, _ = rt.load_ini(_write(tmp_path, "[transport]\nenergy_groups = 1:10, 10:100:1\n"))
    assert len(cfg.E_edges) - 1 == 1029


@pytest.mark.parametrize("text,msg", [
    ("[energy]\nmean_MeV = -1\n", "mean_E0 must be positive"),
    ("[transport]\nN_theta_local = 3\n", "not compiled"),
    ("[transport]\nenergy_groups = 1:10:0.5, 5:20:1\n", "non-overlapping"),
    ("[grid]\ndz_mm = 0\n", "grid spacing"),
    ("[transport]\nE_fine_on = 20\nE_fine_off = 15\n", "E_fine_off must be >="),
])
def test_invalid_files_are_refused(tmp_path, text, msg):
    with pytest.raises(sm.Sm2dError, match=msg):
        rt.load_ini(_write(tmp_path, text))


def test_missing_file_is_refused(tmp_path):
    with pytest.raises(sm.Sm2dError, match="Failed to load configuration file"):
        rt.load_ini(str(tmp_path / "nope.ini"))


@pytest.mark.gpu
def test_run_simulation_command_equals_the_transport_api(tmp_path):
    path = _write(tmp_path, """[energy]
mean_MeV = 40.0
sigma_MeV = 0.4
[spatial]
sigma_x_mm = 1.5
[angular]
sigma_theta_rad = 0.002
[sampling]
n_samples = 300
random_seed = 7
[grid]
Nx = 40
Nz = 70
dx_mm = 0.5
dz_mm = 0.5
max_steps = 3000
[output]
output_dir = res
normalize_dose = true
""")
    exe = os.path.join(LIB_DIR, "run_simulation")
    r = subprocess.run([exe, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cfg, beam, run = rt.load_ini(path)
    with sm.Transport(cfg) as t:
        t.inject(beam.x0, beam.z0, beam.theta0, beam.E0, beam.W_total, beam.sigma_x, beam.sigma_theta,
                 beam.sigma_E, beam.n_samples, beam.seed)
        t.run(run["max_iterations"])
        dose = t.dose()
    rows = [l.split("\t") for l in (tmp_path / "res" / "dose_2d.txt").read_text().splitlines()
            if l and not l.startswith("#")]
    got = np.array([float(x[2]) for x in rows]).reshape(cfg.Nz, cfg.Nx)
    assert np.abs(got - dose).max() <= 5e-5 + 1e-5 * dose.max()     # printed with 4 decimals
    pdd = (tmp_path / "res" / "pdd.txt").read_text().splitlines()
    assert pdd[0] == "# Depth-Dose Distribution (PDD)" and pdd[1] == "# Depth(mm) Dose(Gy) Dose_norm"
    peak = sm.bragg_peak_row(dose)
    assert pdd[2].startswith(f"# Bragg Peak at: {peak * 0.5:g} mm")
    bad = subprocess.run([exe, str(tmp_path / "missing.ini")], capture_output=True, text=True, timeout=120)
    assert bad.returncode == 1 and "Failed to load configuration file" in bad.stderr
