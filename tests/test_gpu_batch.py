"""Batched spots.  A plan (sm2d_batch_run: lanes in flight, a finished lane
refilled with the plan's next spot inside the device loop) and a wave
(sm2d_batch_inject + run) transport every spot as a single-lane engine
transports it alone (inject + run), as the reference runner transports one
spot per call with the Fermi-Eyges tables of that spot's energy and width
(gpu_transport_wrapper.cu:273-276): same iteration count and audit record,
dose within 1e-5 of its maximum."""
import numpy as np
import pytest

import sm_2d_gb300 as sm
from sm_2d_gb300.runtime import Beam

pytestmark = pytest.mark.gpu


def _cfg(lanes, E0=40.0, sigma_x=1.5):
    cfg = sm.Config.reference_runner(40, 70, 0.5, 0.5, sigma_x_initial=sigma_x, E0=E0).production()
    cfg.lanes = lanes
    return cfg


def _beams():
    # uneven spots: energies (so iteration counts), widths, positions and
    # sample seeds differ
    out = []
    for i, (E0, x0, sx) in enumerate([(40.0, 0.0, 1.5), (30.0, -2.0, 1.0), (35.0, 1.5, 2.0), (40.0, 3.0, 1.0),
                                      (25.0, 0.5, 1.5), (20.0, -1.0, 1.2), (32.0, 2.0, 1.8)]):
        out.append(Beam(x0, 0.0, 0.0, E0, 1.0, sx, 0.002, 0.01 * E0, 300, 11 + i))
    return out


def _single(b, max_it=3000):
    with sm.Transport(_cfg(1, b.E0, b.sigma_x)) as one:
        one.inject(b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples, b.seed)
        n = one.run(max_it)
        wfail = sum(1 for h in one.audit_history() if not h["W_pass"])
        return dict(n=n, dose=one.dose(), sc=one.scalars(), au=one.audit(), wfail=wfail)


@pytest.fixture(scope="module")
def singles():
    return [_single(b) for b in _beams()]


def _check_spot(i, r, dose, ref):
    assert r["finished"] == 1 and r["iterations"] == ref["n"], (i, r["iterations"], ref["n"])
    assert abs(r["weight_audit_failures"] - ref["wfail"]) <= 1, (i, r["weight_audit_failures"], ref["wfail"])
    sc, au = ref["sc"], ref["au"]
    assert abs(r["injected_energy"] - sc["source_injected_energy"]) <= 1e-9 * sc["source_injected_energy"]
    assert abs(r["transport_dropped_energy"] - sc["transport_dropped_energy"]) <= 1e-6
    for k in ("W_in_total", "W_out_total", "E_in_total", "E_dep_total", "E_nuclear_total"):
        assert abs(r["last"][k] - au[k]) <= 1e-9 + 1e-5 * abs(au[k]), (i, k)
    m = ref["dose"].max()
    err = np.abs(dose - ref["dose"]).max()
    assert err <= 1e-5 * m, (i, float(err / m))


def test_plan_equals_single_spots(singles):
    beams = _beams()
    with sm.Transport(_cfg(3)) as many:   # 7 spots on 3 lanes: lanes refilled as their spots finish
        assert many.lanes == 3
        dose, res = many.batch_run(beams, 3000)
        passes, refills, _ = many.plan_stats()
        # a single spot afterwards is back on the problem's tables
        b = beams[0]
        many.reset()
        many.inject(b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples, b.seed)
        assert many.run(3000) == singles[0]["n"]
        single_again = many.dose()
    for i in range(len(beams)):
        _check_spot(i, res[i], dose[i], singles[i])
    # the first fill and at least one refill per finishing round; fewer
    # passes than waves of 3 would need
    n_it = [s["n"] for s in singles]
    assert refills >= 3
    waves = sum(max(n_it[k:k + 3]) + 1 for k in range(0, len(n_it), 3))
    assert passes < waves, (passes, waves)
    assert np.abs(single_again - singles[0]["dose"]).max() <= 1e-5 * singles[0]["dose"].max()


def test_wave_equals_single_spots(singles):
    beams = _beams()[:3]
    with sm.Transport(_cfg(4)) as many:   # 3 spots on 4 lanes: one lane stays empty
        many.batch_inject(beams)
        many.run(3000)
        res = many.batch_results(4)
        dose = many.batch_dose(4)
    for i in range(3):
        _check_spot(i, res[i], dose[i], singles[i])
    assert res[3]["iterations"] == 0 and not dose[3].any()


def test_plan_iteration_limit():
    """A spot cut at max_iterations: unfinished, its in-flight weight and
    energy booked as a transport drop (the terminal residual)."""
    beams = _beams()[:4]
    lim = 25
    with sm.Transport(_cfg(2)) as many:
        _, res = many.batch_run(beams, lim, dose=False)
    for i, b in enumerate(beams):
        ref = _single(b, lim)
        r = res[i]
        assert r["finished"] == 0 and r["iterations"] == lim == ref["n"], (i, r)
        want_w = ref["sc"]["transport_dropped_weight"] + ref["au"]["W_out_total"]
        want_e = ref["sc"]["transport_dropped_energy"] + ref["au"]["E_out_total"]
        assert abs(r["transport_dropped_weight"] - want_w) <= 1e-5 * want_w, (i, r["transport_dropped_weight"], want_w)
        assert abs(r["transport_dropped_energy"] - want_e) <= 1e-5 * want_e


def test_plan_repeats():
    """The same plan twice on one engine: same iteration counts, and dose
    equal up to the order of float atomic additions (1e-6 of its maximum)."""
    beams = _beams()
    with sm.Transport(_cfg(3)) as many:
        d1, r1 = many.batch_run(beams, 3000)
        many.plan_load(beams, 3000)
        many.plan_run_async()
        d2, r2 = many.plan_results()
    assert [r["iterations"] for r in r1] == [r["iterations"] for r in r2]
    assert np.abs(d1 - d2).max() <= 1e-6 * d1.max()


def test_value_pages_hold_the_plan_and_a_short_region_stops_it():
    """Each lane's claimed slots take value pages from the lane's region.  The
    plan's peak stays inside the default region; a region cut to exactly that
    peak gives the same spots; a region smaller than the peak stops the run
    with SM2D_ERR_ALLOC (cells past the region write to the overflow pages)
    instead of writing over another lane's pages, and the engine runs again
    after a reset."""
    beams = _beams()
    with sm.Transport(_cfg(3)) as many:
        d1, r1 = many.batch_run(beams, 3000)
        per_lane, peak = many.page_stats()
    assert per_lane == min(40 * 70 * 32, (8 << 20) // 256) and 0 < peak <= per_lane, (per_lane, peak)
    cfg = _cfg(3)
    cfg.slot_pages_per_lane = peak
    with sm.Transport(cfg) as tight:
        d2, r2 = tight.batch_run(beams, 3000)
        assert tight.page_stats() == (peak, peak)
    assert [r["iterations"] for r in r1] == [r["iterations"] for r in r2]
    assert np.abs(d1 - d2).max() <= 1e-6 * d1.max()
    cfg.slot_pages_per_lane = max(1, peak // 4)
    with sm.Transport(cfg) as short:
        with pytest.raises(sm.Sm2dError, match="value pages"):
            short.batch_run(beams, 3000)
        short.reset()
        b = Beam(0.0, 0.0, 0.0, 20.0, 1.0, 0.3, 0.0, 0.0, 1, 1)   # a pencil: a few pages
        short.inject(b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples, b.seed)
        assert short.run(3000) > 0 and short.dose().max() > 0


def test_lanes_in_flight_change_speed_not_results():
    """A plan that keeps fewer lanes in flight (the others stay empty) and the
    tuner's choice give the same spots as a plan on every lane: same
    iteration counts, dose equal up to the order of float atomic additions."""
    beams = _beams()
    with sm.Transport(_cfg(4)) as many:
        d_all, r_all = many.batch_run(beams, 3000)
        assert many.lanes_in_flight() == 4
        many.set_lanes_in_flight(2)
        assert many.lanes_in_flight() == 2
        d_two, r_two = many.batch_run(beams, 3000)
        passes_two, _, _ = many.plan_stats()
        many.plan_load(beams, 3000)
        n, ms = many.tune_lanes_in_flight()
        assert n in (1, 2, 3, 4) and ms > 0 and many.lanes_in_flight() == n
        many.plan_run_async()
        d_t, r_t = many.plan_results()
    for d, r in ((d_two, r_two), (d_t, r_t)):
        assert [x["iterations"] for x in r] == [x["iterations"] for x in r_all]
        assert all(x["finished"] for x in r)
        assert np.abs(d - d_all).max() <= 1e-6 * d_all.max()
    # two lanes take longer to work through seven spots than four do
    assert passes_two > max(x["iterations"] for x in r_all)


def test_plan_on_the_engine_lane_limit():
    """600 small uneven spots on 512 lanes, the engine's limit: the first fill
    takes 512 spots, the refills the other 88 (finished-lane lists over 16
    warp steps, per-lane sums staged for 512 lanes).  Spots taken from the
    start, the middle and the refills equal the same spots run alone."""
    rng = np.random.default_rng(77)
    beams = [Beam(float(rng.uniform(-3.0, 3.0)), 0.0, 0.0, float(rng.choice([20.0, 25.0, 30.0, 35.0])), 1.0,
                  float(rng.uniform(0.8, 2.0)), 0.002, 0.3, 100, 1000 + i) for i in range(600)]
    with sm.Transport(_cfg(512)) as many:
        assert many.lanes == 512
        dose, res = many.batch_run(beams, 3000)
        passes, refills, _ = many.plan_stats()
    assert all(r["finished"] for r in res) and refills >= 2
    assert passes < max(r["iterations"] for r in res) * 2
    for i in (0, 257, 511, 512, 599):
        ref = _single(beams[i])
        assert res[i]["iterations"] == ref["n"], (i, res[i]["iterations"], ref["n"])
        m = ref["dose"].max()
        assert np.abs(dose[i] - ref["dose"]).max() <= 1e-5 * m, i


def test_batch_run_into_pinned_host_maps():
    """Dose maps asked into pinned host memory are written there by the device
    as each spot completes (no copy at the end); they equal the maps copied
    into pageable memory, up to the order of float atomic additions."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from sm_2d_gb300.runtime import SpotResult
    beams = _beams()
    n = len(beams)
    with sm.Transport(_cfg(3)) as many:
        d_pageable, r_pageable = many.batch_run(beams, 3000)
        pinned = torch.full((n, 70, 40), -1.0, dtype=torch.float64).pin_memory()
        arr = (Beam * n)(*beams)
        res = (SpotResult * n)()
        rc = many._lib.sm2d_batch_run(many.h, C.cast(arr, C.c_void_p), n, 3000, C.c_void_p(pinned.data_ptr()),
                                      C.cast(res, C.c_void_p))
        assert rc == 0, many._lib.sm2d_last_error()
    d_pinned = pinned.numpy()
    assert [res[i].as_dict()["iterations"] for i in range(n)] == [r["iterations"] for r in r_pageable]
    assert (d_pinned >= 0.0).all()   # every map written
    assert np.abs(d_pinned - d_pageable).max() <= 1e-6 * d_pageable.max()


def test_batch_refuses_bad_beams():
    with sm.Transport(_cfg(2)) as t:
        bad = [Beam(0.0, 0.0, 0.0, 40.0, 1.0, 1.5, 0.002, 0.4, 0, 1)]   # Gaussian without samples
        with pytest.raises(sm.Sm2dError):
            t.batch_run(bad, 100)


def test_plan_edges(singles):
    """An empty plan, fewer spots than lanes, dose asked of a plan loaded
    without dose maps, and a larger plan after a smaller one (its buffers
    grow)."""
    beams = _beams()
    with sm.Transport(_cfg(4)) as many:
        many.plan_load([], 3000)
        many.plan_run_async()
        d, r = many.plan_results()
        assert d.shape == (0, 70, 40) and r == []
        dose, res = many.batch_run(beams[:2], 3000)          # 2 spots on 4 lanes
        for i in range(2):
            _check_spot(i, res[i], dose[i], singles[i])
        many.plan_load(beams[:3], 3000, dose=False)
        many.plan_run_async()
        with pytest.raises(sm.Sm2dError, match="without dose"):
            many.plan_results(dose=True)
        _, res = many.plan_results(dose=False)
        assert [r["iterations"] for r in res] == [s["n"] for s in singles[:3]]
        dose, res = many.batch_run(beams, 3000)              # 7 spots: the plan buffers grow
        for i in range(len(beams)):
            _check_spot(i, res[i], dose[i], singles[i])


def test_plan_in_bucket_mode_equals_direct_mode(singles):
    """The reference's bucket structure (DeviceOutflowBucket + K4) gives the
    same spots as the fused direct scatter, refills included."""
    beams = _beams()
    cfg = _cfg(3)
    cfg.use_buckets = 1
    with sm.Transport(cfg) as many:
        dose, res = many.batch_run(beams, 3000)
    for i in range(len(beams)):
        _check_spot(i, res[i], dose[i], singles[i])


def test_launch_shape_changes_speed_not_results():
    """The kernels stride over their work and the claims follow keys, so a
    plan transported with another launch shape (blocks per SM of each pass
    kernel) gives the same spots to float-summation noise; the autotuner
    returns a shape within the candidates and keeps it."""
    cfg = sm.Config.reference_runner(40, 60, 0.5, 0.5, sigma_x_initial=1.5, E0=30.0).production()
    cfg.lanes = 3
    beams = [Beam(0.0, 0.0, 0.0, 20.0 + 3.0 * i, 1.0, 1.0 + 0.2 * i, 0.002, 0.2, 200, 40 + i) for i in range(5)]
    with sm.Transport(cfg) as t:
        d0, r0 = t.batch_run(beams, 2000)
        t.set_launch_shape([2, 2, 1, 1])
        assert t.launch_shape() == [2, 2, 1, 1]
        d1, r1 = t.batch_run(beams, 2000)
        t.plan_load(beams, 2000)
        shape, ms = t.autotune()
        assert ms > 0 and t.launch_shape() == shape and 1 <= shape[0] <= 16 and 1 <= shape[1] <= 8
        d2, r2 = t.batch_run(beams, 2000)
    for d in (d1, d2):
        assert np.abs(d - d0).max() <= 1e-5 * d0.max()
    assert [r["iterations"] for r in r1] == [r["iterations"] for r in r0] == [r["iterations"] for r in r2]
