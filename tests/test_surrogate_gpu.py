"""The learned redistribution surrogate on the GPU, through the C ABI.

* the method's tables (sm2d_redistribution_table, the expectation form's
  closed forms on the device) equal the C oracle's float tables;
* the tcgen05 forward pass equals the oracle's restatement (bf16 operands,
  wide accumulation) on the same weights, and every row sums to 1;
* the gradients of the fused training kernel equal the oracle's gradients,
  and one Adam step equals the oracle's Adam step;
* training on the method's tables lowers the loss, and the trained network is
  closer to the method than the untrained one; with the calibrated per-region
  fallback, rows that keep the network's output are within the tolerance and
  the other rows are the method's rows exactly.
"""
import numpy as np
import pytest

import sm_2d_gb300 as sm
from oracle import surrogate as so

pytestmark = pytest.mark.gpu

# forward tables: the hidden activations are rounded to bf16 on both sides, but
# from sums accumulated in different orders (fp32 tensor core, float64 here);
# a sum within that difference of a bf16 rounding boundary rounds the other
# way and moves its row by 1e-5..1e-4 (about 2 % of rows), exceptionally by a
# few 1e-3; a weight within that difference of the 2^-12 floor is zero on one
# side only (a move of 2.4e-4).  Bounds: the median row, the share of rows
# above 1e-3, the worst row.
FWD_MEDIAN, FWD_ROW_ATOL, FWD_MAX_SHARE, FWD_ATOL = 1e-6, 1e-3, 0.01, 1e-2
GRAD_RTOL = 2e-2    # relative L2 error of each parameter block's gradient


@pytest.fixture(scope="module")
def surr():
    s = sm.Surrogate()
    yield s
    s.close()


def test_plain_table_matches_oracle(surr, oracle_mod):
    f = surr.features(20000, 11)
    t = surr.plain(f).cpu().numpy()
    ref = oracle_mod.redistribution_table(f.cpu().numpy())
    assert np.abs(t - ref).max() == 0.0   # the same float arithmetic (sm2d_redist.h) on both sides
    assert (t >= 0).all()
    np.testing.assert_allclose(t.sum(axis=1), 1.0, atol=2e-6)


def test_feature_distribution(surr):
    f = surr.features(200000, 3).cpu().numpy()
    assert f[:, 0].min() >= 0.0 and f[:, 0].max() <= 8.0 and abs(np.sqrt(f[:, 0] / 8.0).mean() - 0.5) < 0.01
    assert f[:, 1].min() >= 0.0 and f[:, 1].max() < 1.0 and abs(f[:, 1].mean() - 0.5) < 0.01
    assert f[:, 2].min() >= 0.0 and f[:, 2].max() <= 4.0
    assert set(np.unique(f[:, 3])) == {0.0, 1.0} and abs(f[:, 3].mean() - 0.5) < 0.01


def test_forward_matches_oracle(surr):
    p = so.init_params()
    p[so.O_B1:] = np.random.default_rng(1).normal(0, 0.05, so.N_PARAMS - so.O_B1).astype(np.float32)
    surr.set_params(p)
    f = surr.features(3000, 21)   # not a multiple of the 128-row tile
    t = surr.forward(f).cpu().numpy()
    ref = so.table(p, f.cpu().numpy())
    d = np.abs(t - ref).max(axis=1)
    assert np.median(d) <= FWD_MEDIAN, np.median(d)
    assert np.mean(d > FWD_ROW_ATOL) < FWD_MAX_SHARE and d.max() <= FWD_ATOL, (np.mean(d > FWD_ROW_ATOL), d.max())
    np.testing.assert_allclose(t.sum(axis=1), 1.0, atol=1e-6)


def test_gradients_match_oracle(surr):
    p = so.init_params()
    surr.set_params(p)
    f = surr.features(1000, 31)
    y = surr.plain(f)
    loss, g = surr.gradients(f, y)
    ref_loss, ref = so.loss_and_grad(p, f.cpu().numpy(), y.cpu().numpy())
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    blocks = {"W1": (so.O_W1, so.O_W2), "W2": (so.O_W2, so.O_W3), "W3": (so.O_W3, so.O_B1),
              "b1": (so.O_B1, so.O_B2), "b2": (so.O_B2, so.O_B3), "b3": (so.O_B3, so.N_PARAMS)}
    for name, (lo, hi) in blocks.items():
        rel = np.linalg.norm(g[lo:hi] - ref[lo:hi]) / max(np.linalg.norm(ref[lo:hi]), 1e-30)
        assert rel <= GRAD_RTOL, (name, rel)


def test_adam_step_matches_oracle(surr):
    p = so.init_params()
    surr.set_params(p)
    f = surr.features(surr.batch, 41)
    y = surr.plain(f)
    _, g = surr.gradients(f, y)
    surr.train(f, y, steps=1, lr0=1e-3, lr_min=1e-3)
    q = surr.params()
    ref, _, _ = so.adam(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3)
    np.testing.assert_allclose(q, ref, rtol=1e-5, atol=1e-7)


def test_training_gains_over_untrained_and_fallback_bounds_error(surr):
    surr.set_params(so.init_params())
    f = surr.features(1 << 21, 51)
    y = surr.plain(f)
    fv = surr.features(1 << 16, 52)
    yv = surr.plain(fv).cpu().numpy()
    err0 = np.abs(surr.forward(fv).cpu().numpy() - yv).mean()
    hist = surr.train(f, y, steps=6000, lr0=2e-3, lr_min=2e-5)
    assert np.isfinite(hist).all()
    assert hist[-200:].mean() < hist[:20].mean()
    err1 = np.abs(surr.forward(fv).cpu().numpy() - yv).mean()
    assert err1 < 0.2 * err0, (err0, err1)
    # calibration on its own set, then fallback on a fresh one
    fc = surr.features(1 << 20, 53)
    surr.calibrate(fc)
    tol = 0.01
    fn = surr.features(1 << 16, 54)
    out, fb = surr.redistribute(fn, tol)
    out, fb = out.cpu().numpy(), fb.cpu().numpy().astype(bool)
    ref = surr.plain(fn).cpu().numpy()
    np.testing.assert_allclose(out.sum(axis=1), 1.0, atol=1e-6)
    np.testing.assert_array_equal(out[fb], ref[fb])
    row_err = np.abs(out - ref).max(axis=1)
    assert fb.mean() < 1.0
    print(f"surrogate: mean |err| untrained {err0:.3g}, trained {err1:.3g}; fallback {fb.mean():.3f} of rows; "
          f"row max error q99 {np.quantile(row_err[~fb], 0.99):.3g}, max {row_err.max():.3g}")
    assert np.quantile(row_err[~fb], 0.99) <= tol and row_err.max() <= 5 * tol
