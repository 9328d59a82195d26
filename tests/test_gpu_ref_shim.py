"""The C++ drop-in layer (libsm2d_ref.so) on the GPU: the reference's
run_k1k6_pipeline_transport wrapper (gpu_transport_wrapper.hpp:78-92), its
pipeline entry on DevicePsiC buffers with the K1K6PipelineState
(k1k6_pipeline.cuh:296-416), init_device_lut and the stage entries, called by
a C++ program built here against include/sm2d_ref_types.hpp
(tests/shim_driver.cpp) as the reference's runner and tests call them.

Bars: the wrapper's edep equals the C ABI's post-convolved dose of the same
beam; the pipeline entry leaves in the state the C ABI's tallies and audit
record of the same phase space, with the final phase space in the buffer the
reference's pointer swaps end on; run_k1_active_mask equals the engine's K1
mask bit for bit; the stand-alone K2 reports that it has no separate form.
Deposits are summed with atomics, so doses agree to 1e-5 of their maximum."""
import os
import subprocess

import numpy as np
import pytest

import sm_2d_gb300 as sm
from sm_2d_gb300 import build as B

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BEAM = dict(x0=0.0, z0=0.0, theta0=0.0, E0=40.0, W=1.0, sigma_x=1.5, sigma_theta=0.002, sigma_E=0.4, n_samples=400,
            seed=11)
NX, NZ, MAXIT = 40, 80, 1000


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    B.build()
    cuda = B._cuda_home()
    exe = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    inc = [os.path.join(cuda, "include"), os.path.join(cuda, "targets", "sbsa-linux", "include"),
           os.path.join(cuda, "targets", "x86_64-linux", "include"), os.path.join(ROOT, "include")]
    libs = [os.path.join(cuda, "lib64"), os.path.join(cuda, "targets", "sbsa-linux", "lib"),
            os.path.join(cuda, "targets", "x86_64-linux", "lib")]
    cmd = (["g++", "-std=c++17", "-O1"] + ["-I" + p for p in inc] + [os.path.join(ROOT, "tests", "shim_driver.cpp"),
           "-o", exe, "-L" + B.OUT, "-lsm2d_ref", "-lsm2d_ref_host", "-lsm2d"] + ["-L" + p for p in libs] +
           ["-lcudart", "-Wl,-rpath," + B.OUT, "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    subprocess.run(cmd, check=True)
    return exe


def _run(driver, mode, tmp_path):
    out = tmp_path / f"{mode}.bin"
    r = subprocess.run([driver, mode, str(out)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (mode, r.returncode, r.stderr[-2000:])
    return np.fromfile(out, np.float64), r.stderr


def _engine():
    cfg = sm.Config.reference_runner(NX, NZ, 0.5, 0.5, sigma_x_initial=1.5, E0=40.0)
    cfg.max_iterations = MAXIT
    return sm.Transport(cfg)


def test_wrapper_equals_the_c_abi(driver, tmp_path):
    edep, _ = _run(driver, "wrapper", tmp_path)
    edep = edep.reshape(NZ, NX)
    with _engine() as t:
        t.inject(**BEAM)
        t.run(MAXIT)
        dose = t.dose()
    assert dose.max() > 0
    assert np.abs(edep - dose).max() <= 1e-5 * dose.max()
    assert sm.bragg_peak_row(edep) == sm.bragg_peak_row(dose)


def test_pipeline_on_device_buffers_fills_the_state(driver, tmp_path):
    out, _ = _run(driver, "pipeline", tmp_path)
    Nc = NX * NZ
    edep, tail = out[:Nc], out[Nc:]
    (W_in, W_out, W_cut, W_nuc, W_bnd, E_in, E_out, E_dep, E_cut, E_nuc, E_bnd, W_pass, E_pass, drop_w, drop_e,
     resid, w_psi_in, w_psi_out) = tail
    with _engine() as t:
        t.inject(**BEAM)
        n = t.run(MAXIT)
        tal = t.tallies()
        a = t.audit()
        sc = t.scalars()
    assert np.abs(edep - tal["edep"]).max() <= 1e-5 * tal["edep"].max()
    for got, key in ((W_in, "W_in_total"), (W_out, "W_out_total"), (W_cut, "W_cutoff_total"),
                     (W_nuc, "W_nuclear_total"), (W_bnd, "W_boundary_total"), (E_in, "E_in_total"),
                     (E_out, "E_out_total"), (E_dep, "E_dep_total"), (E_cut, "E_cutoff_total"),
                     (E_nuc, "E_nuclear_total"), (E_bnd, "E_boundary_total")):
        assert abs(got - a[key]) <= 1e-9 + 1e-5 * abs(a[key]), (key, got, a[key])
    assert (int(W_pass), int(E_pass)) == (a["W_pass"], a["E_pass"])
    assert abs(drop_w - sc["transport_dropped_weight"]) <= 1e-9 + 1e-5 * abs(sc["transport_dropped_weight"])
    assert abs(drop_e - sc["transport_dropped_energy"]) <= 1e-9 + 1e-5 * abs(sc["transport_dropped_energy"])
    # the final phase space is in one buffer (its weight is the last audit's
    # psi_out weight), the other one is clear
    assert min(w_psi_in, w_psi_out) == 0.0
    assert abs(max(w_psi_in, w_psi_out) - a["W_out_total"]) <= 1e-5 * a["W_out_total"] + 1e-12, (n, w_psi_in, w_psi_out)


def test_stage_entries(driver, tmp_path):
    out, err = _run(driver, "stages", tmp_path)
    mask, k2 = out[:-1].astype(np.uint8), out[-1]
    with _engine() as t:
        t.inject(**BEAM)
        t.step()
        want = t.mask()
    assert np.array_equal(mask, want)
    assert k2 == 0.0
    assert "one deterministic pass" in err
