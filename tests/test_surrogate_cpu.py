"""CPU checks of the redistribution surrogate's oracle: the method's tables
(the expectation form's closed forms, sm2d_redist.h, restated in the C
oracle) and the network's float64/bf16 restatement, its gradient against
finite differences, and the host helpers."""
import numpy as np
import pytest

import sm_2d_gb300 as sm
from oracle import oracle as orc
from oracle import surrogate as so


def sample_features(n, seed):
    """(s, u, r, cap) rows of the training distribution."""
    r = np.random.default_rng(seed)
    return np.stack([8.0 * r.uniform(0, 1, n) ** 2, r.uniform(0, 1, n), 4.0 * r.uniform(0, 1, n) ** 2,
                     (r.uniform(0, 1, n) < 0.5).astype(np.float64)], axis=1).astype(np.float32)


def test_tables_are_distributions():
    t = orc.redistribution_table(sample_features(4000, 1))
    assert t.shape == (4000, 32)
    assert (t >= 0).all()
    np.testing.assert_allclose(t.sum(axis=1), 1.0, atol=2e-6)


def test_table_limits():
    # no spreads: the angle stays, the energy splits between the centres
    # around the mean (window capped at the incoming bin: centres 1, 0, -1, -2)
    t = orc.redistribution_table(np.array([[0.0, 0.5, 0.0, 1.0]], np.float32))[0].reshape(4, 8)
    assert t[:, 1:].sum() == 0.0
    np.testing.assert_allclose(t[:, 0], [0.5, 0.5, 0.0, 0.0], atol=1e-7)
    # window not capped (centres 2, 1, 0, -1): u = 0.25 gives 0.25 to e = 1
    t = orc.redistribution_table(np.array([[0.0, 0.25, 0.0, 0.0]], np.float32))[0].reshape(4, 8)
    np.testing.assert_allclose(t[:, 0], [0.0, 0.25, 0.75, 0.0], atol=1e-7)
    # the energy split keeps the mean; straggling spreads it
    for u, r in [(0.3, 0.2), (0.7, 0.5)]:
        t = orc.redistribution_table(np.array([[1.0, u, r, 0.0]], np.float32), fp64=True)[0].reshape(4, 8)
        me = t.sum(axis=1)
        assert abs((me * np.array([2.0, 1.0, 0.0, -1.0])).sum() - u) < 5e-3
    # a small angle spread sends s^2 to the neighbours, a large one spreads far
    t = orc.redistribution_table(np.array([[0.1, 0.5, 0.0, 1.0]], np.float32), fp64=True)[0].reshape(4, 8)
    assert abs(t[:, 1].sum() - 0.01) < 1e-6
    t = orc.redistribution_table(np.array([[4.0, 0.5, 0.0, 1.0]], np.float32))[0].reshape(4, 8)
    assert t[:, 4:].sum() > 0.3


def test_fp32_table_matches_fp64_method():
    f = sample_features(3000, 2)
    d = np.abs(orc.redistribution_table(f) - orc.redistribution_table(f, fp64=True))
    # the angular masses are differences of normal CDF values: in float they
    # cancel to a few 1e-5 absolute (1e-6 on average) at the widest spreads
    assert d.max() < 5e-5
    assert d.mean() < 1e-6


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
    f = sample_features(512, 6)
    y = orc.redistribution_table(f)
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
    assert g["s_max"] == 8.0 and g["r_max"] == 4.0 and g["u_max"] == 1.0 and g["cap_max"] == 1.0
    assert g["regions_s"] * g["regions_u"] * g["regions_r"] * g["regions_cap"] == 4096


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
    u = so.scaled(f)
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
    u = so.scaled(f)
    wimg = so.w1_image(W1).astype(np.float64)
    pre = so.features(f).astype(np.float64) @ wimg.T
    exact = u @ so.bf16(W1[:, :4]).astype(np.float64).T
    scale = np.abs(so.bf16(W1[:, :4])).sum(axis=1).max()
    assert np.abs(pre - exact).max() < scale * 2.0 ** -15
    # u moved by 1/4 of a bf16 step of its scaled value 2 u - 1
    g = f.copy()
    g[:, 1] = (f[:, 1].astype(np.float64) + 0.25 * 2.0 ** -10).astype(np.float32)
    d = so.features(g).astype(np.float64) @ wimg.T - pre
    step = 2.0 * (g[:, 1].astype(np.float64) - f[:, 1])
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
