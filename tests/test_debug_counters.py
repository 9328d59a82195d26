"""Drop counters of k2/k3/k4_get_debug_counters (sm2d_get_debug_counters):
output-slot, bucket and prune drops per stage, whose weights and energies add
up to the transport-drop channel.  On the CPU the oracle's per-iteration
channels, summed over a run, add up to its transport drops; on a GPU the
engine's counters equal the oracle's channels stage by stage and kind by
kind, in both emission modes, and reset per stage."""
import numpy as np
import pytest

import sm_2d_gb300 as sm

KINDS = ("slot", "bucket", "pruned")


def _problem(use_buckets=0):
    """A 40 MeV beam in 40 x 70 cells with the production seeds and floor
    cutoff but without the stopping rule, and prune thresholds high enough
    that K2 and K3 prune (1e-5 and 1e-6 of a unit weight): the run ends when
    no cell is listed, so no remainder is booked into the transport drops."""
    cfg = sm.Config.reference_runner(40, 70, 0.5, 0.5, sigma_x_initial=1.5, E0=40.0).production()
    cfg.stop_weight_fraction = 0.0
    cfg.prune_coarse, cfg.prune_fine = 1e-5, 1e-6
    cfg.use_buckets = use_buckets
    beam = dict(x0=0.0, z0=0.0, theta0=0.0, E0=40.0, W=1.0, sigma_x=1.5, sigma_theta=0.002, sigma_E=0.4,
                n_samples=300, seed=11)
    return cfg, beam


def _oracle_run(oracle_mod, cfg, beam):
    o = oracle_mod.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges)
    o.inject(**beam)
    n = 0
    while n < 3000 and o.step():
        n += 1
    assert n < 3000
    return o, n


def test_oracle_channels_add_up_to_the_transport_drops(oracle_mod):
    cfg, beam = _problem()
    o, _ = _oracle_run(oracle_mod, cfg, beam)
    ch = o.drop_channels()
    sc = o.scalars()
    assert sum(w for w, _ in ch.values()) == pytest.approx(sc["transport_dropped_weight"], rel=1e-12, abs=1e-15)
    assert sum(e for _, e in ch.values()) == pytest.approx(sc["transport_dropped_energy"], rel=1e-12, abs=1e-15)
    # the thresholds make both transports prune; K4 has output-slot drops only
    assert ch[(2, "pruned")][0] > 0 and ch[(3, "pruned")][0] > 0
    assert ch[(4, "bucket")] == (0.0, 0.0) and ch[(4, "pruned")] == (0.0, 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("use_buckets", [0, 1])
def test_engine_counters_equal_oracle_channels(oracle_mod, use_buckets):
    cfg, beam = _problem(use_buckets)
    o, n_o = _oracle_run(oracle_mod, cfg, beam)
    och = o.drop_channels()
    with sm.Transport(cfg) as t:
        t.inject(**beam)
        assert t.run(3000) == n_o
        got = {s: t.debug_counters(s) for s in (2, 3, 4)}
        sc = t.scalars()
        t.reset_debug_counters(3)
        after = {s: t.debug_counters(s) for s in (2, 3, 4)}
        with pytest.raises(sm.Sm2dError, match="stage"):
            t.debug_counters(5)
    tot_w = sum(got[s][k][1] for s in got for k in KINDS)
    tot_e = sum(got[s][k][2] for s in got for k in KINDS)
    assert tot_w == pytest.approx(sc["transport_dropped_weight"], rel=1e-6, abs=1e-12)
    assert tot_e == pytest.approx(sc["transport_dropped_energy"], rel=1e-6, abs=1e-10)
    for s in (2, 3, 4):
        for k in KINDS:
            n, w, e = got[s][k]
            ow, oe = och[(s, k)]
            assert abs(w - ow) <= 1e-6 * max(ow, 1e-9), (s, k, w, ow)
            assert abs(e - oe) <= 1e-6 * max(oe, 1e-9), (s, k, e, oe)
            assert (n > 0) == (w > 0), (s, k, n, w)
    assert after[3] == {k: (0, 0.0, 0.0) for k in KINDS}
    assert after[2] == got[2] and after[4] == got[4]
