"""The expectation form on the GPU against the CPU oracle of the same form:
K2/K3 emit the expected result of re-binning their MCS angle and straggling
loss (sm2d_redist.h) instead of one hashed draw of each.  Bars as for the
sampled form: lists, masks and the block id of every slot bit-exact for the
first iterations (the children's claim keys give the oracle's sequential
claim order), the same iteration count, audit records equal within float
summation noise, dose within 1e-4 of its maximum, the same Bragg-peak row."""
import numpy as np
import pytest

import bench
import sm_2d_gb300 as sm
from sm_2d_gb300.runtime import Beam
from test_gpu_configs import _audit_close, _full_run, _oracle, _oracle_dose, _step_exact

pytestmark = pytest.mark.gpu


def _cfg(Nx, Nz, E0, sx, lanes=1):
    cfg = sm.Config.reference_runner(Nx, Nz, 0.5, 0.5, sigma_x_initial=sx, E0=E0, energy_split=1).production()
    cfg.expectation = 1
    cfg.max_iterations = bench.MAX_IT
    cfg.lanes = lanes
    return cfg


def test_small_beam_slot_exact_then_full_run(oracle_mod):
    cfg = _cfg(48, 60, 40.0, 1.5)
    beam = dict(x0=0.0, z0=0.0, theta0=0.0, E0=40.0, W=1.0, sigma_x=1.5, sigma_theta=0.002, sigma_E=0.4,
                n_samples=400, seed=11)
    o = _oracle(oracle_mod, cfg, beam)
    with sm.Transport(cfg) as t:
        t.inject(**beam)
        _step_exact(t, o, 15, "expect-small")
        _full_run(t, o, cfg, 1e-4, "expect-small", oracle_mod)


def test_production_beam_full_run(oracle_mod):
    """150 MeV, sigma_x 3.8 mm, 200 x 400 cells: 20 iterations slot-exact,
    then the full run."""
    cfg = _cfg(200, 400, 150.0, 3.8)
    beam = dict(bench.BEAM)
    o = _oracle(oracle_mod, cfg, beam)
    with sm.Transport(cfg) as t:
        t.inject(**beam)
        _step_exact(t, o, 20, "expect-C2")
        _full_run(t, o, cfg, 1e-4, "expect-C2", oracle_mod)


def test_plan_spots_equal_oracle_single_spots(oracle_mod):
    """Four spots of the 512-spot plan on two lanes (refilled on the device)
    against the oracle transporting each spot alone."""
    spots = [s for i, s in enumerate(bench.plan_spots("plan512", 0, 512)) if i in bench.plan_sample("plan512", 512, 4)]
    cfg = _cfg(200, 400, 150.0, 3.8, lanes=2)
    orcs = [_oracle(oracle_mod, cfg, b, E0=b["E0"], sigma_x=b["sigma_x"]) for b in spots]
    oracle_mod.run_many(orcs, bench.MAX_IT, 4)
    beams = [Beam(b["x0"], b["z0"], b["theta0"], b["E0"], b["W"], b["sigma_x"], b["sigma_theta"], b["sigma_E"],
                  b["n_samples"], b["seed"]) for b in spots]
    with sm.Transport(cfg) as t:
        dose, res = t.batch_run(beams, bench.MAX_IT)
    for i, (b, o, r) in enumerate(zip(spots, orcs, res)):
        tag = (i, b["E0"])
        assert r["finished"] == 1 and r["iterations"] == int(o.scalars()["iterations"]), tag
        _audit_close(r["last"], o.audit(), tag)
        ref = _oracle_dose(oracle_mod, o, cfg)
        assert float(np.abs(dose[i] - ref).max() / ref.max()) <= 1e-4, tag
        assert sm.bragg_peak_row(dose[i]) == sm.bragg_peak_row(ref), tag
