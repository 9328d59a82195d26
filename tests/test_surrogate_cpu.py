"""CPU checks of the redistribution surrogate's oracle: the method's tables
(C restatement of K3's per-bin physics) and the network's float64/bf16
restatement, its gradient against finite differences, and the host helpers."""
import numpy as np
import pytest

import sm_2d_gb300 as sm
from oracle import oracle as orc
from oracle import surrogate as so


def table_oracle():
    cfg = sm.Config.log_grid(4, 4, 0.5, 0.5, N_E=256, E_min=0.1, E_max=250.0, N_theta=512)
    return orc.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges)


def sample_features(n, seed):
    r = np.random.default_rng(seed)
    return np.stack([np.exp(r.uniform(np.log(0.1), np.log(250.0), n)), r.uniform(-0.3, 0.3, n),
                     r.uniform(0.05, 2.0, n), r.uniform(0.2, 2.0, n)], axis=1).astype(np.float32)


def test_tables_are_distributions():
    o = table_oracle()
    t = o.redistribution_table(sample_features(4000, 1))
    assert t.shape == (4000, 32)
    assert (t >= 0).all()
    np.testing.assert_allclose(t.sum(axis=1), 1.0, atol=2e-6)


def test_table_physics_limits():
    o = table_oracle()
    # 150 MeV over 0.1 mm of water: energy loss far below a bin, so all weight in
    # E bin 0; sigma_theta well below a bin, so the two bins around the incoming
    # direction (3 and 4) share it equally
    t = o.redistribution_table(np.array([[150.0, 0.1, 0.1, 1.0]], np.float32))[0].reshape(4, 8)
    assert t[1:].sum() < 1e-6
    assert abs(t[0, 3] - 0.5) < 1e-3 and abs(t[0, 4] - 0.5) < 1e-3
    # 1 MeV over 2 mm: the mean energy falls to the LUT floor (R(1 MeV) is about
    # 0.02 mm), so most weight is in the lowest E bin; the straggling sigma of
    # the step (Bohr, several MeV at this beta) puts the rest in the top bin,
    # and the angle spreads into the end bins
    t = o.redistribution_table(np.array([[1.0, 0.0, 2.0, 1.0]], np.float32))[0].reshape(4, 8)
    assert t[3].sum() > 0.5 and t[1:3].sum() < 0.02
    assert t[3, 0] > 0.05 and t[3, 7] > 0.05
    # the incoming angle does not enter the relative bins
    a = o.redistribution_table(np.array([[20.0, -0.2, 1.0, 1.5], [20.0, 0.25, 1.0, 1.5]], np.float32))
    np.testing.assert_array_equal(a[0], a[1])


def test_fp32_table_matches_fp64_method():
    cfg = sm.Config.log_grid(4, 4, 0.5, 0.5, N_E=256, E_min=0.1, E_max=250.0, N_theta=512)
    o32 = orc.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges)
    o64 = orc.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges, fp64=True)
    f = sample_features(3000, 2)
    d = np.abs(o32.redistribution_table(f) - o64.redistribution_table(f))
    assert d.max() < 2e-3, d.max()
    assert d.mean() < 1e-5


def test_gradient_matches_finite_differences():
    r = np.random.default_rng(3)
    f = sample_features(64, 4)
    y = r.dirichlet(np.ones(32), 64)
    p = so.init_params().astype(np.float64)
    p[so.O_B1:] = r.normal(0, 0.1, so.N_PARAMS - so.O_B1)
    g = so.grad_exact(p, f, y)
    idx = np.concatenate([r.choice(np.arange(so.O_W1, so.O_W2).reshape(-1, 16)[:, :4].ravel(), 8),
                          r.choice(np.arange(so.O_W2, so.O_W3), 8), r.choice(np.arange(so.O_W3, so.O_B1), 8),
                          r.choice(np.arange(so.O_B1, so.N_PARAMS), 8)])
    h = 1e-4   # smaller steps lose digits to cancellation in the float64 loss
    for k in idx:
        a, b = p.copy(), p.copy()
        a[k] += h
        b[k] -= h
        fd = (so.loss_exact(a, f, y) - so.loss_exact(b, f, y)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(g[k]), (k, fd, g[k])


def test_bf16_restatement_close_to_exact_gradient():
    r = np.random.default_rng(5)
    o = table_oracle()
    f = sample_features(512, 6)
    y = o.redistribution_table(f)
    p = so.init_params()
    loss, g = so.loss_and_grad(p, f, y)
    ge = so.grad_exact(p, f, y)
    assert abs(loss - so.loss_exact(p, f, y)) < 2e-2 * abs(loss)
    for lo, hi in [(so.O_W2, so.O_W3), (so.O_W3, so.O_B1), (so.O_B2, so.O_B3), (so.O_B3, so.N_PARAMS)]:
        rel = np.linalg.norm(g[lo:hi] - ge[lo:hi]) / np.linalg.norm(ge[lo:hi])
        assert rel < 0.1, (lo, rel)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], np.float32)
    b = so.bf16(x)
    assert b[0] == 1.0 and b[1] == 1.0 and b[2] == np.float32(1.0 + 2 ** -6) and b[3] == -2.5
    assert abs(b[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_surrogate_geometry_exported():
    g = sm.Surrogate.geometry()
    assert abs(g["dtheta"] - np.pi / 512) < 1e-7
    assert abs(g["dlnE"] - np.log(2500.0) / 256) < 1e-7
    assert g["step_min"] == pytest.approx(0.05) and g["step_max"] == pytest.approx(2.0)


def test_adam_restatement_first_step():
    p = so.init_params()
    r = np.random.default_rng(7)
    g = (r.choice([-1.0, 1.0], so.N_PARAMS) * r.uniform(1e-3, 2e-3, so.N_PARAMS)).astype(np.float32)
    q, m, v = so.adam(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3)
    # the first bias-corrected Adam step moves each parameter by lr against its gradient's sign
    np.testing.assert_allclose(q - p, -1e-3 * np.sign(g), rtol=1e-3, atol=1e-9)


def test_surrogate_entries_refuse_bad_arguments_without_a_gpu():
    # argument checks come before any CUDA call, so they answer on a host without a GPU
    import ctypes as C
    from sm_2d_gb300 import surrogate as sg
    L = sg._lib()
    h = C.c_void_p()
    assert L.sm2d_mlp_create(0, None, C.byref(h)) == -1 and not h.value
    assert L.sm2d_mlp_create((1 << 30) + 1, None, C.byref(h)) == -1 and not h.value   # above the row limit
    assert L.sm2d_redistribution_features(0, 1, None, None) == -1
    assert L.sm2d_redistribution_table(None, None, 10, None) == -1
    assert L.sm2d_mlp_forward(None, None, 10, None) == -1
    assert L.sm2d_mlp_sync(None) == -1
    assert L.sm2d_mlp_destroy(None) == -1
    assert b"null" in L.sm2d_last_error()


def test_bf16_input_pairs_carry_sixteen_bits():
    # each scaled input reaches the first GEMM as bf16(u) and bf16(128 (u - bf16(u))):
    # together they restore u to about 2^-16 of its range
    f = sample_features(20000, 8)
    x = so.features(f)
    u = np.stack([2.0 * (np.log(f[:, 0].astype(np.float64)) - so.LN_EMIN) / (so.LN_EMAX - so.LN_EMIN) - 1.0,
                  f[:, 1] / so.TH_MAX, 2.0 * (f[:, 2] - so.DS_MIN) / (so.DS_MAX - so.DS_MIN) - 1.0,
                  2.0 * (f[:, 3] - so.RHO_MIN) / (so.RHO_MAX - so.RHO_MIN) - 1.0], axis=1)
    rebuilt = x[:, :4].astype(np.float64) + x[:, 4:8].astype(np.float64) / 128.0
    assert np.abs(rebuilt - u).max() < 2.0 ** -15
    assert np.abs(x[:, :4] - u).max() > 2.0 ** -10     # bf16 alone would lose them
    assert (x[:, 8:] == 0).all()


def test_first_layer_sees_inputs_to_sixteen_bits():
    """With the remainder columns tied to bf16(W1[:, i]) / 128, the first
    GEMM forms bf16(W1) u with u to about 2^-16, and an input moved by less
    than a bf16 step moves the hidden pre-activations by about W1 times that
    step, not by the sawtooth of an independent remainder weight."""
    r = np.random.default_rng(9)
    p = so.init_params()
    W1 = so.unpack(p)[0]
    assert (W1[:, 4:8] == 0).all()          # the tied parameters stay zero
    f = sample_features(4000, 10)
    u = np.stack([2.0 * (np.log(f[:, 0].astype(np.float64)) - so.LN_EMIN) / (so.LN_EMAX - so.LN_EMIN) - 1.0,
                  f[:, 1] / so.TH_MAX, 2.0 * (f[:, 2] - so.DS_MIN) / (so.DS_MAX - so.DS_MIN) - 1.0,
                  2.0 * (f[:, 3] - so.RHO_MIN) / (so.RHO_MAX - so.RHO_MIN) - 1.0], axis=1)
    wimg = so.w1_image(W1).astype(np.float64)
    pre = so.features(f).astype(np.float64) @ wimg.T
    exact = u @ so.bf16(W1[:, :4]).astype(np.float64).T
    scale = np.abs(so.bf16(W1[:, :4])).sum(axis=1).max()
    assert np.abs(pre - exact).max() < scale * 2.0 ** -15
    # a theta moved by 1/4 of a bf16 step of its scaled value
    g = f.copy()
    g[:, 1] = (f[:, 1].astype(np.float64) + 0.25 * 2.0 ** -9 * so.TH_MAX).astype(np.float32)
    d = so.features(g).astype(np.float64) @ wimg.T - pre
    step = (g[:, 1].astype(np.float64) - f[:, 1]) / so.TH_MAX
    want = step[:, None] * so.bf16(W1[:, 1]).astype(np.float64)[None, :]
    assert np.abs(d - want).max() < scale * 2.0 ** -14
    del r


def test_tied_gradient_is_the_sum_of_both_columns():
    r = np.random.default_rng(11)
    f = sample_features(256, 12)
    y = r.dirichlet(np.ones(32), 256)
    p = so.init_params()
    _, g = so.loss_and_grad(p, f, y)
    g1 = g[so.O_W1:so.O_W2].reshape(so.HID, so.IN)
    assert (g1[:, 4:8] == 0).all()
    # finite differences of the bf16 restatement through a weight of column 0:
    # moving W1[o, 0] moves both image columns 0 and 4
    o = int(np.argmax(np.abs(g1[:, 0])))
    k = so.O_W1 + o * so.IN
    h = 2.0 ** -4 * max(abs(float(p[k])), 0.05)
    a, b = p.copy(), p.copy()
    a[k] += h
    b[k] -= h
    la, _ = so.loss_and_grad(a, f, y)
    lb, _ = so.loss_and_grad(b, f, y)
    fd = (la - lb) / (2 * h)
    assert abs(fd - g1[o, 0]) <= 0.05 * abs(g1[o, 0]) + 1e-6, (fd, g1[o, 0])
