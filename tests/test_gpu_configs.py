"""GPU against the CPU oracle on the workloads the benchmark runs, at their full
sizes: the 70 MeV pencil on the 256 log-E / 512 theta / 128-local-bin grid
(80 x 120 cells), the 150 MeV production beam on 200 x 400 cells (reference
grids and log grid), spots of the 512-spot plan spanning 70-230 MeV through the
batch entry, and the 230 MeV beam through the 300 x 600 slab phantom.

Bars: the block id of every slot bit-exact for the first iterations (the
deterministic claim order equals the oracle's sequential claims, so this is a
check of every binning decision); the same iteration count; every audit record
equal within float-summation noise; dose within 1e-5 (single spots on the log
grid) or 1e-4 (everything else) of its maximum; the same Bragg-peak row.  The
oracle follows k1k6_pipeline.cu:1606-2038 (the loop) and k5_audit.cu:139-166
(the pass flags).
"""
import numpy as np
import pytest

import bench
import sm_2d_gb300 as sm
from sm_2d_gb300.runtime import Beam

pytestmark = pytest.mark.gpu


def _audit_close(g, o, tag):
    for k, v in o.items():
        if k.endswith("_total"):
            assert abs(g[k] - v) <= 1e-9 + 1e-5 * abs(v), (tag, k, g[k], v)
    assert g["processed_cells"] == o["processed_cells"], tag


def _oracle(orc, cfg, beam, E0=None, sigma_x=None):
    oc = cfg.oracle_config()
    if E0 is not None:
        oc.update(E0=E0, sigma_x_initial=sigma_x)
    o = orc.Oracle(oc, cfg.theta_edges, cfg.E_edges)
    if cfg.density_z is not None:
        o.set_density(cfg.density_z)
    o.inject(**beam)
    return o


def _oracle_dose(orc, o, cfg):
    return orc.postprocess(o.tallies()["edep"], o.fe()[2], o.cfg["sigma_x_initial"], cfg.Nx, cfg.Nz, cfg.dx)


def _step_exact(t, o, n_it, tag):
    """n_it iterations on both sides: lists, masks and the block id of every
    slot bit-exact, audit records equal."""
    for it in range(n_it):
        t.step()
        assert o.step(), (tag, it)
        ga, gc = t.lists()
        oa, oc = o.lists()
        assert np.array_equal(ga, oa) and np.array_equal(gc, oc), (tag, it)
        assert np.array_equal(t.mask(), o.mask()), (tag, it)
        gb, _ = t.psi_in(values=False)
        ob, _ = o.psi_in(values=False)
        assert np.array_equal(gb, ob), (tag, it, int((gb != ob).sum()))
        _audit_close(t.audit(), o.audit(), (tag, it))


def _full_run(t, o, cfg, tol, tag, orc, max_it=bench.MAX_IT):
    n_o = o.run(max_it)
    n_g = t.run(max_it)
    assert n_g == n_o, (tag, n_g, n_o)
    _audit_close(t.audit(), o.audit(), tag)
    e_g, e_o = t.tallies()["edep"], o.tallies()["edep"]
    err = float(np.abs(e_g - e_o).max() / e_o.max())
    assert err <= tol, (tag, err)
    dose, ref = t.dose(), _oracle_dose(orc, o, cfg)
    derr = float(np.abs(dose - ref).max() / ref.max())
    assert derr <= tol, (tag, derr)
    assert sm.bragg_peak_row(dose) == sm.bragg_peak_row(ref), tag
    sc = t.scalars()
    assert sc["claim_table_overflows"] == 0 and sc["claim_misses"] == 0 and sc["bin_list_overflows"] == 0
    return err


C1_BEAM = dict(x0=0.0, z0=0.0, theta0=0.0, E0=70.0, W=1.0, sigma_x=0.0, sigma_theta=0.0, sigma_E=0.0,
               n_samples=1, seed=42)


def _c1_config():
    return sm.Config.log_grid(80, 120, 0.5, 0.5, N_E=256, E_min=0.1, E_max=250.0, N_theta=512,
                              theta_max=np.pi / 2, layout=sm.LAYOUT_B128, E_fine_on=10.0, E_fine_off=11.0,
                              sigma_x_initial=0.0, E0=70.0, energy_split=1).production()


def test_c1_pencil_log_grid(oracle_mod):
    """70 MeV pencil, 80 x 120 cells, 256 log-E / 512 theta bins, 8x4x4x1
    local bins, energy split: 20 iterations slot-exact, then the full run."""
    cfg = _c1_config()
    o = _oracle(oracle_mod, cfg, C1_BEAM)
    with sm.Transport(cfg) as t:
        t.inject(**C1_BEAM)
        _step_exact(t, o, 20, "C1")
        err = _full_run(t, o, cfg, 1e-5, "C1", oracle_mod)
    assert err <= 1e-5


@pytest.mark.parametrize("grid", ["reference", "log"])
def test_c2_production_beam(grid, oracle_mod):
    """150 MeV, sigma_x 3.8 mm, sigma_E 1 %, 1000 LCG samples, 200 x 400 cells:
    30 iterations slot-exact, then the full run."""
    cfg = bench.make_config(grid, "c2")
    beam = dict(bench.BEAM)
    o = _oracle(oracle_mod, cfg, beam)
    with sm.Transport(cfg) as t:
        t.inject(**beam)
        _step_exact(t, o, 30, ("C2", grid))
        _full_run(t, o, cfg, 1e-4, ("C2", grid), oracle_mod)


def _plan_sample(k=8):
    """k spots of the 512-spot plan spread over its energies, the highest
    (a spot that leaves the 200 mm domain distally) and the lowest included:
    the benchmark's accuracy sample."""
    spots = bench.plan_spots("plan512", 0, 512)
    return [spots[i] for i in bench.plan_sample("plan512", 512, k)]


def test_plan_spots_equal_oracle_single_spots(oracle_mod):
    """Eight spots of the plan (70-230 MeV), transported by the batch entry on
    three lanes (refilled on the device), against the oracle transporting each
    spot alone with the Fermi-Eyges tables of its own energy and width."""
    spots = _plan_sample(8)
    energies = [b["E0"] for b in spots]
    assert min(energies) <= 72.0 and max(energies) >= 226.0
    cfg = bench.make_config("reference", "plan512")
    cfg.lanes = 3
    orcs = [_oracle(oracle_mod, cfg, b, E0=b["E0"], sigma_x=b["sigma_x"]) for b in spots]
    oracle_mod.run_many(orcs, bench.MAX_IT, 8)
    beams = [Beam(b["x0"], b["z0"], b["theta0"], b["E0"], b["W"], b["sigma_x"], b["sigma_theta"], b["sigma_E"],
                  b["n_samples"], b["seed"]) for b in spots]
    with sm.Transport(cfg) as t:
        dose, res = t.batch_run(beams, bench.MAX_IT)
    exits = 0
    for i, (b, o, r) in enumerate(zip(spots, orcs, res)):
        sc = o.scalars()
        tag = (i, b["E0"])
        assert r["finished"] == 1 and r["iterations"] == int(sc["iterations"]), (tag, r["iterations"], sc)
        _audit_close(r["last"], o.audit(), tag)
        assert abs(r["injected_energy"] - sc["source_injected_energy"]) <= 1e-9 * sc["source_injected_energy"]
        assert abs(r["transport_dropped_energy"] - sc["transport_dropped_energy"]) <= 1e-6 + 1e-5 * abs(
            sc["transport_dropped_energy"])
        ref = _oracle_dose(oracle_mod, o, cfg)
        derr = float(np.abs(dose[i] - ref).max() / ref.max())
        assert derr <= 1e-4, (tag, derr)
        assert sm.bragg_peak_row(dose[i]) == sm.bragg_peak_row(ref), tag
        exits += o.audit()["E_boundary_total"] > 0.05 * sc["source_injected_energy"]
    assert exits >= 1   # the 230 MeV spot leaves the domain through its distal face


def test_c3_slab_phantom(oracle_mod):
    """230 MeV, sigma_x 5 mm, through the seeded slab phantom on 300 x 600
    cells: 20 iterations slot-exact, then the full run (the beam leaves the
    domain distally)."""
    cfg = bench.make_config("reference", "c3")
    beam = dict(bench.C3_BEAM, seed=bench.spot_seeds(0, 1)[0])
    o = _oracle(oracle_mod, cfg, beam)
    with sm.Transport(cfg) as t:
        t.inject(**beam)
        _step_exact(t, o, 20, "C3")
        _full_run(t, o, cfg, 1e-4, "C3", oracle_mod)
