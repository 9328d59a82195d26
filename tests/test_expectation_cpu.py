"""The expectation form on the CPU oracle: its redistribution masses against
numerical integration of the quantities they stand for, and the method on the
reference runner's grids -- conservation, the FP32 build against the FP64
build, and the Bragg peak of a 40 MeV beam against the continuous-slowing-down
range of the R-LUT.  The sampled form's per-bin hashed draws make its FP32
and FP64 results drift apart (a last-bit difference moves a component to
another angle bin, and the seeds of everything after it change); the
expectation form has no draws, so the two builds agree to float rounding."""
import numpy as np
import pytest

import sm_2d_gb300 as sm
from oracle import oracle as orc

SQRT2 = np.sqrt(2.0)


def _phi_cdf(x):
    from math import erf
    return 0.5 * (1.0 + np.vectorize(erf)(x / SQRT2))


def theta_masses_numeric(s):
    """E over u ~ N(0, s^2) of the reference's 2-bin re-binning: (1 - r^2) to
    round(u), r^2 to the neighbour towards u; distances folded at 7."""
    u = np.linspace(-14 * s - 1, 14 * s + 1, 2_000_001)
    p = np.exp(-0.5 * (u / s) ** 2)
    n = np.round(u)
    r = u - n
    M = np.zeros(8)
    for idx, ww in ((n, 1 - r ** 2), (n + np.sign(r), r ** 2)):
        np.add.at(M, np.minimum(np.abs(idx).astype(int), 7), ww * p)
    return M / M.sum()


def energy_masses_numeric(Em, sE, cen):
    """E over E' ~ N(Em, sE^2) of the mean-preserving split between the two
    centres around E'; E' beyond the first / last centre folds there."""
    x = np.linspace(Em - 9 * sE, Em + 9 * sE, 2_000_001)
    p = np.exp(-0.5 * ((x - Em) / sE) ** 2)
    M = np.zeros(len(cen))
    M[0] += p[x >= cen[0]].sum()
    M[-1] += p[x <= cen[-1]].sum()
    for e in range(len(cen) - 1):
        m = (x < cen[e]) & (x > cen[e + 1])
        f = (x[m] - cen[e + 1]) / (cen[e] - cen[e + 1])
        M[e] += (f * p[m]).sum()
        M[e + 1] += ((1 - f) * p[m]).sum()
    return M / M.sum()


@pytest.mark.parametrize("s", [0.05, 0.3, 0.7, 1.0, 2.0, 3.5])
def test_theta_masses_match_integration(s):
    want = theta_masses_numeric(s)
    for fp64, tol in ((True, 1e-5), (False, 3e-5)):   # the integration grid resolves to about 3e-6
        Mt, _ = orc.redist_masses(s, 10.0, 0.0, [10.0], fp64=fp64)
        np.testing.assert_allclose(Mt, want, atol=tol)
        assert abs(Mt.sum() - 1.0) < (1e-12 if fp64 else 2e-7)
    # small spreads: the neighbours take s^2 together, as the frac^2 split's
    # variance-preserving share
    Mt, _ = orc.redist_masses(0.05, 10.0, 0.0, [10.0], fp64=True)
    assert abs(Mt[1] - 0.05 ** 2) < 1e-9


@pytest.mark.parametrize("Em,sE", [(9.8, 0.1), (9.55, 0.3), (9.95, 0.02), (9.2, 0.05), (9.75, 0.6)])
def test_energy_masses_match_integration(Em, sE):
    cen = [10.0, 9.7, 9.4, 9.1]
    want = energy_masses_numeric(Em, sE, cen)
    for fp64, tol in ((True, 1e-5), (False, 3e-5)):
        _, Me = orc.redist_masses(0.0, Em, sE, cen, fp64=fp64)
        np.testing.assert_allclose(Me, want, atol=tol)
        assert abs(Me.sum() - 1.0) < (1e-12 if fp64 else 2e-7)
    # no spread: the energy split of Em itself (mean preserving)
    _, Me = orc.redist_masses(0.0, 9.58, 0.0, cen, fp64=True)
    assert np.nonzero(Me)[0].tolist() == [1, 2]
    assert abs((Me * np.array(cen)).sum() - 9.58) < 1e-12


def _run(fp64, E0=40.0, Nx=40, Nz=80, expect=1, tables=0):
    cfg = sm.Config.reference_runner(Nx, Nz, 0.5, 0.5, sigma_x_initial=1.5, E0=E0, energy_split=1).production()
    cfg.expectation = expect
    o = orc.Oracle(dict(cfg.oracle_config(), surrogate_tables=tables), cfg.theta_edges, cfg.E_edges, fp64=fp64)
    o.inject(x0=0.0, z0=0.0, theta0=0.0, E0=E0, W=1.0, sigma_x=1.5, sigma_theta=0.002, sigma_E=0.01 * E0,
             n_samples=400, seed=11)
    fails = 0
    n = 0
    e_err = 0.0
    while n < 3000 and o.step():
        n += 1
        a = o.audit()
        fails += a["W_pass"] == 0
        e_err = max(e_err, a["E_error"])
    tal, sc = o.tallies(), o.scalars()
    dose = orc.postprocess(tal["edep"], o.fe()[2], 1.5, Nx, Nz, cfg.dx)
    total = (tal["edep"].sum() + tal["e_cut"].sum() + tal["e_nuc"].sum() + tal["e_bnd"].sum()
             + sc["transport_dropped_energy"] + sc["audit_residual_energy"])
    return dict(n=n, dose=dose, fails=fails, e_err=e_err, balance=total - sc["source_injected_energy"]
                + sc["source_representation_loss_energy"], cfg=cfg)


def test_expectation_form_fp32_matches_fp64():
    a, b = _run(False), _run(True)
    assert a["n"] == b["n"]
    err = np.abs(a["dose"] - b["dose"]).max() / b["dose"].max()
    pdd = np.abs(a["dose"].sum(1) - b["dose"].sum(1)).max() / b["dose"].sum(1).max()
    assert err < 1e-3 and pdd < 1e-4, (err, pdd)
    for r in (a, b):
        assert abs(r["balance"]) < 1e-6
        assert r["fails"] == 0   # weight audit (1e-6) passes every iteration
        # the energy audit carries the reference's accounting of a step's
        # nuclear loss: the deposit dE w counts the removed weight's share
        # dE w_rem that the nuclear channel books again with E w_rem, a
        # relative 1e-5..1e-4 on these beams (the sampled form alike)
        assert r["e_err"] < 1e-4


def test_expectation_form_bragg_peak_at_the_csda_range():
    """40 MeV in water: the CSDA range of the R-LUT is 14.9 mm; the Bragg peak
    lies within a millimetre before it, and no dose lies 2 mm beyond it."""
    r = _run(False)
    pdd = r["dose"].sum(1)
    z = (np.arange(pdd.size) + 0.5) * 0.5
    lut = sm.range_lut(sm.energy_grid_piecewise(sm.runtime.DEFAULT_ENERGY_GROUPS)[1])
    rep = sm.energy_grid_piecewise(sm.runtime.DEFAULT_ENERGY_GROUPS)[1]
    R40 = float(np.interp(40.0, rep, lut["R"]))
    assert 14.0 < R40 < 16.0
    zp = z[pdd.argmax()]
    assert R40 - 1.0 <= zp <= R40 + 0.25, (zp, R40)
    assert pdd[z > R40 + 2.0].sum() < 1e-3 * pdd.sum()


def test_expectation_needs_the_energy_split():
    cfg = sm.Config.reference_runner(8, 8, 0.5, 0.5)
    cfg.expectation = 1
    with pytest.raises(sm.Sm2dError, match="energy split"):
        sm.Transport(cfg)


def test_table_path_with_the_method_tables_equals_the_closed_forms():
    """K3 components whose energy window has uniformly spaced centres take
    their children's weights from a 32-entry table (the learned surrogate's
    path); given the plain table of their features, the run equals the closed
    forms up to float rounding (the table's energy masses are evaluated in
    units of the centre spacing)."""
    a, b = _run(False), _run(False, tables=1)
    assert a["n"] == b["n"]
    assert np.abs(a["dose"] - b["dose"]).max() / a["dose"].max() < 1e-5
    assert abs(b["balance"]) < 1e-6 and b["fails"] == 0
