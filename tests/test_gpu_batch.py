"""Batched spots (sm2d_batch_run): every spot of a batch -- lanes
transported together, in waves -- equals the same spot transported alone
on a single-lane engine (inject + run), as the reference runner transports
one spot per call with the Fermi-Eyges tables of that spot's energy and
width (gpu_transport_wrapper.cu:273-276): same iteration count and audit
record, dose within 1e-5 of its maximum."""
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
    # uneven spots: energies, widths, positions and sample seeds differ
    out = []
    for i, (E0, x0, sx) in enumerate([(40.0, 0.0, 1.5), (30.0, -2.0, 1.0), (35.0, 1.5, 2.0), (40.0, 3.0, 1.0),
                                      (25.0, 0.5, 1.5)]):
        out.append(Beam(x0, 0.0, 0.0, E0, 1.0, sx, 0.002, 0.01 * E0, 300, 11 + i))
    return out


def test_batch_equals_single_spots():
    beams = _beams()
    ref_dose, ref_res = [], []
    for b in beams:
        with sm.Transport(_cfg(1, b.E0, b.sigma_x)) as one:
            one.inject(b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples,
                       b.seed)
            n = one.run(3000)
            ref_dose.append(one.dose())
            wfail = sum(1 for h in one.audit_history() if not h["W_pass"])
            ref_res.append((n, one.scalars(), one.audit(), wfail))
    with sm.Transport(_cfg(3)) as many:   # 5 spots on 3 lanes: two waves, the second one partial
        assert many.lanes == 3
        dose, res = many.batch_run(beams, 3000)
        # a single spot afterwards is back on the problem's tables (lane 0
        # last held those of beams[3], 1.0 mm wide)
        b = beams[0]
        many.reset()
        many.inject(b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples, b.seed)
        assert many.run(3000) == ref_res[0][0]
        single_again = many.dose()
    for i, b in enumerate(beams):
        n, sc, au, wfail = ref_res[i]
        r = res[i]
        assert r["finished"] == 1 and r["iterations"] == n, (i, r["iterations"], n)
        assert abs(r["weight_audit_failures"] - wfail) <= 1, (i, r["weight_audit_failures"], wfail)
        assert abs(r["injected_energy"] - sc["source_injected_energy"]) <= 1e-9 * sc["source_injected_energy"]
        assert abs(r["transport_dropped_energy"] - sc["transport_dropped_energy"]) <= 1e-6
        for k in ("W_in_total", "W_out_total", "E_in_total", "E_dep_total", "E_nuclear_total"):
            assert abs(r["last"][k] - au[k]) <= 1e-9 + 1e-5 * abs(au[k]), (i, k)
        m = ref_dose[i].max()
        assert np.abs(dose[i] - ref_dose[i]).max() <= 1e-5 * m, (i, float(np.abs(dose[i] - ref_dose[i]).max() / m))
    assert np.abs(single_again - ref_dose[0]).max() <= 1e-5 * ref_dose[0].max()


def test_batch_refuses_bad_beams():
    with sm.Transport(_cfg(2)) as t:
        bad = [Beam(0.0, 0.0, 0.0, 40.0, 1.0, 1.5, 0.002, 0.4, 0, 1)]   # Gaussian without samples
        with pytest.raises(sm.Sm2dError):
            t.batch_run(bad, 100)
