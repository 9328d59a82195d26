"""The precision form on the GPU against the oracle of the same form: the K5
audit books each iteration's cutoff, nuclear and boundary weight from the
iteration's own per-cell increments, and the R-LUT is inverted in double below
10 MeV.  Bars as for the other forms: the block id of every slot bit-exact for
the first iterations, audit records equal within float-summation noise, the
same iteration count, dose within 1e-4 of its maximum; and the weight audit
passes every iteration, where the reference's differencing of float
cumulative tallies fails on a spot that stops inside the domain."""
import numpy as np
import pytest

import bench
import sm_2d_gb300 as sm
from test_gpu_configs import _full_run, _oracle, _step_exact

pytestmark = pytest.mark.gpu

BEAM70 = dict(x0=0.0, z0=0.0, theta0=0.0, E0=70.0, W=1.0, sigma_x=4.1, sigma_theta=0.002, sigma_E=0.7,
              n_samples=1000, seed=7)


def _cfg(precision):
    cfg = bench.make_config("reference", "plan512", "precision" if precision else "sampled")
    cfg.E0, cfg.sigma_x_initial = BEAM70["E0"], BEAM70["sigma_x"]
    return cfg


def test_precision_form_matches_oracle_and_passes_every_weight_audit(oracle_mod):
    cfg = _cfg(True)
    o = _oracle(oracle_mod, cfg, BEAM70)
    with sm.Transport(cfg) as t:
        t.inject(**BEAM70)
        _step_exact(t, o, 20, "precision")
        _full_run(t, o, cfg, 1e-4, "precision", oracle_mod)
        hist = t.audit_history()
    assert len(hist) > 50 and all(h["W_pass"] for h in hist), [h["W_error"] for h in hist if not h["W_pass"]]
    # the same spot with the reference's audit arithmetic fails some iterations
    ref = _cfg(False)
    with sm.Transport(ref) as t:
        t.inject(**BEAM70)
        t.run(bench.MAX_IT)
        fails = sum(1 for h in t.audit_history() if not h["W_pass"])
    assert fails > 0


def test_precision_form_through_the_slab_phantom(oracle_mod):
    cfg = bench.make_config("reference", "c3", "precision")
    beam = dict(bench.C3_BEAM, seed=bench.spot_seeds(0, 1)[0])
    o = _oracle(oracle_mod, cfg, beam)
    with sm.Transport(cfg) as t:
        t.inject(**beam)
        _step_exact(t, o, 10, "precision-C3")
        _full_run(t, o, cfg, 1e-4, "precision-C3", oracle_mod)
        hist = t.audit_history()
    assert all(h["W_pass"] for h in hist)
