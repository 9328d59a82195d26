"""The precision form on the CPU oracle (no GPU): on a 70 MeV spot that stops
inside its 200 x 400 domain, the reference's audit (K5 books each iteration's
absorbed weight as the difference of two float cumulative tallies) fails
iterations late in the spot, when the cumulative absorbed weight dwarfs the
in-flight weight; booking the iteration's own increments passes every
iteration.  The double R-LUT inversion below 10 MeV moves the dose by less
than 1e-6 of its maximum."""
import numpy as np

import bench
from oracle import oracle as orc

BEAM70 = dict(x0=0.0, z0=0.0, theta0=0.0, E0=70.0, W=1.0, sigma_x=4.1, sigma_theta=0.002, sigma_E=0.7,
              n_samples=1000, seed=7)


def _run(precision):
    ocfg, th, ee, rho = bench.oracle_problem("reference", "plan512", "precision" if precision else "sampled")
    o = orc.Oracle(dict(ocfg, E0=BEAM70["E0"], sigma_x_initial=BEAM70["sigma_x"]), th, ee)
    o.inject(**BEAM70)
    fails, worst, n = 0, 0.0, 0
    while n < bench.MAX_IT and o.step():
        n += 1
        a = o.audit()
        fails += a["W_pass"] == 0
        worst = max(worst, a["W_error"])
    return n, fails, worst, o.tallies()["edep"]


def test_precision_form_audit_passes_where_the_reference_audit_fails(oracle_mod):
    n0, f0, w0, e0 = _run(False)
    n1, f1, w1, e1 = _run(True)
    assert n0 == n1
    assert f0 > 0 and w0 > 1e-6
    assert f1 == 0 and w1 < 1e-6
    assert np.abs(e1 - e0).max() <= 1e-6 * e0.max()
