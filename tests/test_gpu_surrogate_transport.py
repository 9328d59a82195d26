"""The learned surrogate inside the transport (expectation form): K3 bins whose
energy window has four uniformly spaced centres take their children's weights
from the network's 8 theta x 4 E table instead of the closed forms of
sm2d_redist.h (the per-bin redistribution of k3_finetransport.cu:263-366).

* With the method's own tables on the table path (method_tables), the GPU
  equals the oracle's table path slot for slot: lists, masks and the block id
  of every slot bit-exact for the first iterations, the same iteration count,
  dose within 1e-4 of its maximum, the same Bragg-peak row.
* With a network whose every region falls back (tolerance 0 on an untrained
  network), the run equals the expectation form without the surrogate.
* With the trained network: the oracle running the same network (the C
  restatement of its arithmetic, sums in double) gives the same iteration
  count and dose within 1e-3 of its maximum; every row's weights sum to 1, so
  weight is conserved to 1e-6 of the injected weight over the run and energy
  to 1e-6 of the injected energy; the dose error against the FP64 oracle of
  the closed forms is stated and bounded (the network's angular weights for
  steps of 1-3 angle bins move the Bragg peak by a fraction of a row on the
  40 MeV beam: about 9 % of the peak cell dose, 4 % in depth dose).
"""
import numpy as np
import pytest

import bench
import sm_2d_gb300 as sm
from oracle import surrogate as so
from test_gpu_configs import _full_run, _oracle_dose, _step_exact

pytestmark = pytest.mark.gpu

BEAM40 = dict(x0=0.0, z0=0.0, theta0=0.0, E0=40.0, W=1.0, sigma_x=1.5, sigma_theta=0.002, sigma_E=0.4,
              n_samples=400, seed=11)


def _cfg(Nx, Nz, E0, sx):
    cfg = sm.Config.reference_runner(Nx, Nz, 0.5, 0.5, sigma_x_initial=sx, E0=E0, energy_split=1).production()
    cfg.expectation = 1
    cfg.max_iterations = bench.MAX_IT
    return cfg


def test_method_tables_equal_oracle_table_path(oracle_mod):
    cfg = _cfg(48, 60, 40.0, 1.5)
    o = oracle_mod.Oracle(dict(cfg.oracle_config(), surrogate_tables=1), cfg.theta_edges, cfg.E_edges)
    o.inject(**BEAM40)
    with sm.Surrogate() as surr, sm.Transport(cfg) as t:
        t.set_surrogate(surr, method_tables=True)
        t.inject(**BEAM40)
        _step_exact(t, o, 15, "method-tables")
        _full_run(t, o, cfg, 1e-4, "method-tables", oracle_mod)
        st = t.surrogate_stats()
    assert st["rows"] > 1000 and st["fallback_rows"] == 0 and st["overflow_bins"] == 0, st


def test_all_rows_falling_back_equal_the_closed_forms():
    cfg = _cfg(48, 60, 40.0, 1.5)
    with sm.Surrogate() as u, sm.Transport(cfg) as a, sm.Transport(cfg) as b:
        u.set_params(so.init_params())   # untrained: its error is above zero in every region
        u.calibrate(u.features(1 << 20, 7))
        b.set_surrogate(u, tol=0.0)
        a.inject(**BEAM40)
        b.inject(**BEAM40)
        for it in range(12):
            a.step()
            b.step()
            assert np.array_equal(a.psi_in(values=False)[0], b.psi_in(values=False)[0]), it
        na, nb = a.run(bench.MAX_IT), b.run(bench.MAX_IT)
        assert na == nb
        da, db = a.dose(), b.dose()
        st = b.surrogate_stats()
    assert np.abs(da - db).max() <= 1e-5 * da.max()
    assert st["rows"] > 1000 and st["fallback_rows"] == st["rows"], st


@pytest.fixture(scope="module")
def trained():
    s = sm.Surrogate()
    s.set_params(so.init_params())
    f = s.features(1 << 21, 101)
    s.train(f, s.plain(f), steps=6000)
    s.region_err = s.calibrate(s.features(1 << 20, 102))
    yield s
    s.close()


@pytest.mark.parametrize("E0,sx", [(40.0, 1.5), (70.0, 3.0)])
def test_trained_network_in_the_transport(trained, oracle_mod, E0, sx):
    Nz = 60 if E0 < 50 else 100
    cfg = _cfg(48, Nz, E0, sx)
    beam = dict(BEAM40, E0=E0, sigma_x=sx, sigma_E=0.01 * E0)
    with sm.Transport(cfg) as a, sm.Transport(cfg) as b:
        b.set_surrogate(trained, tol=0.005)
        a.inject(**beam)
        b.inject(**beam)
        na, nb = a.run(bench.MAX_IT), b.run(bench.MAX_IT)
        hist = b.audit_history()
        da, db = a.dose(), b.dose()
        sc = b.scalars()
        tal = b.tallies()
        st = b.surrogate_stats()
    assert 0 < nb < bench.MAX_IT and abs(nb - na) <= 2, (na, nb)
    assert st["rows"] > 1000 and st["fallback_rows"] < st["rows"] and st["overflow_bins"] == 0, st
    # every row sums to 1: the weight audit fails on rounding at most rarely,
    # and the run's weight balance closes
    fails = sum(1 for h in hist if not h["W_pass"])
    assert fails <= 0.02 * len(hist) and max(h["W_error"] for h in hist) < 1e-5, fails
    wsum = (tal["w_cut"].astype(np.float64).sum() + tal["w_nuc"].astype(np.float64).sum()
            + tal["w_bnd"].astype(np.float64).sum() + sc["transport_dropped_weight"])
    w_in = sc["source_injected_weight"] - sc["source_out_of_grid_weight"] - sc["source_slot_dropped_weight"]
    assert abs(wsum - w_in) <= 1e-6 * sc["source_injected_weight"], (wsum, w_in)
    # energy: deposits, cutoff, nuclear and boundary losses and drops add up to
    # the injected energy (less what the source could not represent)
    total = (tal["edep"].sum() + tal["e_cut"].sum() + tal["e_nuc"].sum() + tal["e_bnd"].sum()
             + sc["transport_dropped_energy"] + sc["audit_residual_energy"])
    bal = total - sc["source_injected_energy"] + sc["source_representation_loss_energy"]
    assert abs(bal) <= 1e-6 * sc["source_injected_energy"], bal
    # against the closed forms on the GPU and the FP64 oracle of the form
    err_closed = float(np.abs(db - da).max() / da.max())
    o64 = oracle_mod.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges, fp64=True)
    o64.inject(**beam)
    o64.run(bench.MAX_IT)
    ref64 = _oracle_dose(oracle_mod, o64, cfg)
    err64 = float(np.abs(db - ref64).max() / ref64.max())
    err64_closed = float(np.abs(da - ref64).max() / ref64.max())
    pdd_err = float(np.abs(db.sum(1) - ref64.sum(1)).max() / ref64.sum(1).max())
    # the oracle with the same network and calibration
    on = oracle_mod.Oracle(dict(cfg.oracle_config(), surrogate_tables=2), cfg.theta_edges, cfg.E_edges)
    on.set_surrogate(trained.params(), trained.region_err, 0.005)
    on.inject(**beam)
    n_on = on.run(bench.MAX_IT)
    ref_net = _oracle_dose(oracle_mod, on, cfg)
    err_net = float(np.abs(db - ref_net).max() / ref_net.max())
    rows_on, fb_on = on.surrogate_counts()
    print(f"surrogate transport E0={E0}: rows {st['rows']}, fallback {st['fallback_rows'] / st['rows']:.3f} "
          f"(oracle {rows_on}, {fb_on / max(rows_on, 1):.3f}), dose vs oracle with the network {err_net:.2e}, "
          f"vs closed forms {err_closed:.2e}, vs FP64 {err64:.2e} (closed forms {err64_closed:.2e}), "
          f"PDD vs FP64 {pdd_err:.2e}")
    assert n_on == nb and err_net <= 1e-3, (n_on, nb, err_net)
    assert abs(sm.bragg_peak_row(db) - sm.bragg_peak_row(ref64)) <= 1
    assert pdd_err <= 0.05 and err64 <= 0.12, (pdd_err, err64)
