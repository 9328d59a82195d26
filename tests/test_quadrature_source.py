"""The quadrature source: inject_source_kernel called with its spreads
(k1k6_pipeline.cu:300-427).  The cells within +-4 sigma_x of x0 (clamped to
the grid) take the Gaussian weight of their centres over the float sum of
those weights; with sigma_theta > 1e-4 each of the 7 angle nodes
theta0 + a_k sigma_theta carries w_k of it; without spreads the kernel is the
pencil.  On the CPU the oracle's source is checked against that arithmetic;
on a GPU sm2d_inject_quadrature gives the oracle's phase space (block ids
bit-exact) and the transport from it follows the oracle step by step and
over a whole run."""
import numpy as np
import pytest

import sm_2d_gb300 as sm

GH_A = np.array([-2.65, -1.67, -0.82, 0.0, 0.82, 1.67, 2.65], np.float32)
GH_W = np.array([0.0105, 0.0769, 0.2448, 0.3357, 0.2448, 0.0769, 0.0105], np.float32)


def _cfg(Nx=48, Nz=60, E0=50.0, N_theta=36):
    cfg = sm.Config.reference_runner(Nx, Nz, 0.5, 0.5, N_theta=N_theta, sigma_x_initial=2.0, E0=E0).production()
    return cfg


def _oracle(oracle_mod, cfg):
    return oracle_mod.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges)


def _cell_range(cfg, x0, sx):
    f = np.float32
    lo, hi = f(x0) - f(4.0) * f(sx), f(x0) + f(4.0) * f(sx)
    ix0 = int((lo - f(cfg.x_min)) / f(cfg.dx))
    ix1 = int((hi - f(cfg.x_min)) / f(cfg.dx)) + 1
    return max(ix0, 0), min(ix1, cfg.Nx)


def _expected_cell_weights(cfg, x0, sx):
    ix0, ix1 = _cell_range(cfg, x0, sx)
    xc = cfg.x_min + (np.arange(ix0, ix1) + 0.5) * cfg.dx
    g = np.exp(-0.5 * (xc - x0) ** 2 / sx ** 2) * cfg.dx
    return ix0, ix1, g / g.sum()


def _cell_weights(bid, val, cfg, L):
    v = val.reshape(cfg.Nz * cfg.Nx, 32, L).astype(np.float64)
    return v.sum(axis=(1, 2)).reshape(cfg.Nz, cfg.Nx)


@pytest.mark.parametrize("x0,sx,sth,W", [(0.3, 2.0, 0.003, 2.0),     # angles and cells
                                         (-11.3, 2.0, 0.003, 1.0),   # the range clamped at the grid edge
                                         (1.1, 1.5, 0.0, 1.0)])      # cells only
def test_oracle_source_follows_the_kernel(oracle_mod, x0, sx, sth, W):
    cfg = _cfg()
    o = _oracle(oracle_mod, cfg)
    o.inject_quadrature(x0, 0.0, 0.0, sth, 50.0, W, sx)
    bid, val = o.psi_in()
    cw = _cell_weights(bid, val, cfg, o.L)
    ix0, ix1, wx = _expected_cell_weights(cfg, x0, sx)
    ang = float(GH_W.astype(np.float64).sum()) if sth > 1e-4 else 1.0
    assert np.flatnonzero(cw.sum(axis=1)).tolist() == [0]          # the source row z0 = 0
    row = cw[0]
    assert np.flatnonzero(row > 0).tolist() == [ix for ix in range(ix0, ix1) if wx[ix - ix0] * W > 0]
    assert np.allclose(row[ix0:ix1], W * ang * wx, rtol=1e-5, atol=1e-12)
    # normalised over the cells in the grid, whatever the clamp cut off
    assert abs(row.sum() - W * ang) <= 1e-5 * W
    sc = o.scalars()
    assert sc["source_injected_weight"] == pytest.approx(W) and sc["source_injected_energy"] == pytest.approx(50.0 * W)


def test_oracle_angle_nodes_carry_their_weights(oracle_mod):
    """On 360 theta bins of +-0.35 rad every node theta0 + a_k sigma_theta
    (sigma_theta 20 mrad) falls into a bin of its own, which holds w_k W."""
    cfg = _cfg(N_theta=360)
    o = _oracle(oracle_mod, cfg)
    o.inject_quadrature(0.0, 0.0, 0.01, 0.02, 50.0, 1.0, 1.0)
    bid, val = o.psi_in()
    L, nt = o.L, cfg.layout["nt_local"]
    v = val.reshape(-1, 32, L)
    b = bid.reshape(-1, 32)
    per_bin = {}
    for c, s in zip(*np.nonzero(b != 0xFFFFFFFF)):
        for l in np.flatnonzero(v[c, s] > 0):
            tb = int(b[c, s] & 0xFFF) * nt + int(l) % nt
            per_bin[tb] = per_bin.get(tb, 0.0) + float(v[c, s, l])
    edges = cfg.theta_edges
    want = {}
    for a, w in zip(GH_A, GH_W):
        th = np.float32(np.float32(0.01) + a * np.float32(0.02))
        cont = (th - edges[0]) / ((edges[-1] - edges[0]) / np.float32(360))
        tb = int(cont) + (1 if cont - int(cont) >= 0.5 else 0)
        want[tb] = want.get(tb, 0.0) + float(w)
    assert sorted(per_bin) == sorted(want)
    for tb, w in want.items():
        assert per_bin[tb] == pytest.approx(w, rel=1e-5)


def test_oracle_source_without_spreads_is_the_pencil(oracle_mod):
    cfg = _cfg()
    a, b = _oracle(oracle_mod, cfg), _oracle(oracle_mod, cfg)
    a.inject_quadrature(0.7, 0.3, 0.01, 5e-5, 50.0, 1.0, 0.005)
    b.inject(0.7, 0.3, 0.01, 50.0, 1.0)
    for x, y in zip(a.psi_in(), b.psi_in()):
        assert np.array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("x0,sx,sth", [(0.3, 2.0, 0.003), (-11.3, 2.0, 0.003), (1.1, 1.5, 0.0), (0.25, 0.005, 0.003)])
def test_engine_source_and_transport_match_oracle(oracle_mod, x0, sx, sth):
    from test_gpu_parity import _assert_audit_matches, _assert_slot_sets, _slot_weights
    cfg = _cfg()
    o = _oracle(oracle_mod, cfg)
    o.inject_quadrature(x0, 0.0, 0.0, sth, 50.0, 1.0, sx)
    with sm.Transport(cfg) as t:
        t.inject_quadrature(x0, 0.0, 0.0, sth, 50.0, 1.0, sx)
        gb, gv = t.psi_in()
        ob, ov = o.psi_in()
        assert np.array_equal(gb, ob)
        assert np.allclose(gv, ov, rtol=1e-6, atol=1e-12)
        sc, osc = t.scalars(), o.scalars()
        for k in ("source_injected_weight", "source_injected_energy"):
            assert sc[k] == pytest.approx(osc[k], rel=1e-6, abs=1e-9), k
        # injected minus represented energy: float sums of the same bins in
        # another order, so within 1e-7 of the injected energy
        k = "source_representation_loss_energy"
        assert abs(sc[k] - osc[k]) <= 1e-7 * osc["source_injected_energy"], (sc[k], osc[k])
        for it in range(15):
            t.step()
            o.step()
            assert np.array_equal(t.mask(), o.mask()), it
            gb, gv = t.psi_in()
            ob, ov = o.psi_in()
            assert np.array_equal(gb, ob), (it, int((gb != ob).sum()))
            _assert_slot_sets(_slot_weights(gb, gv, t.L), _slot_weights(ob, ov, o.L), it)
            _assert_audit_matches(t.audit(), o.audit(), it)
        n_o = 15
        while n_o < 3000 and o.step():
            n_o += 1
        n_g = 15 + t.run(3000)
        dose = t.dose()
    assert n_g == n_o
    ot = o.tallies()
    ref = oracle_mod.postprocess(ot["edep"], o.fe()[2], cfg.sigma_x_initial, cfg.Nx, cfg.Nz, cfg.dx)
    assert np.abs(dose - ref).max() <= 1e-4 * ref.max()


@pytest.mark.gpu
def test_engine_source_edges():
    cfg = _cfg()
    with sm.Transport(cfg) as t:
        # without spreads: the pencil, as sm2d_inject places it
        t.inject_quadrature(0.7, 0.3, 0.01, 5e-5, 50.0, 1.0, 0.005)
        q = t.psi_in()
        t.reset()
        t.inject(0.7, 0.3, 0.01, 50.0, 1.0)
        p = t.psi_in()
        assert np.array_equal(q[0], p[0]) and np.array_equal(q[1], p[1])
        t.reset()
        # angle nodes need a positive sigma_x (the cell weights divide by it)
        with pytest.raises(sm.Sm2dError, match="sigma_x"):
            t.inject_quadrature(0.0, 0.0, 0.0, 0.003, 50.0, 1.0, 0.0)
        # into an occupied phase space: refused
        t.inject_quadrature(0.0, 0.0, 0.0, 0.003, 50.0, 1.0, 2.0)
        with pytest.raises(sm.Sm2dError, match="not empty"):
            t.inject_quadrature(0.0, 0.0, 0.0, 0.003, 50.0, 1.0, 2.0)
        # a beam whose cells all lie outside the grid injects nothing
        t.reset()
        t.inject_quadrature(500.0, 0.0, 0.0, 0.003, 50.0, 1.0, 2.0)
        assert not t.psi_in()[1].any()
