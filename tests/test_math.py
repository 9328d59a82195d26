"""The transport's elementary functions (sm2d_math.h): accuracy of the host
build against double-precision libm, and (on a GPU) bit-identity of the CUDA
build with the host build, which is what lets the kernels and the oracle take
identical binning decisions."""
import math

import numpy as np
import pytest

RANGES = {
    "exp": [(-100.0, 88.0), (-8.0, 7.0), (-0.01, 0.01)],
    "log": [("exp", -80.0, 80.0), (0.5, 2.0), (1e-3, 400.0)],
    "sin": [(-7.0, 7.0), (-1.6, 1.6)],
    "cos": [(-7.0, 7.0), (-1.6, 1.6)],
    "erf": [(-5.0, 5.0), (-1e-3, 1e-3), (0.9, 4.1)],
}
REF = {"exp": math.exp, "log": math.log, "sin": math.sin, "cos": math.cos, "erf": math.erf}
MAX_ULP = {"exp": 1.5, "log": 2.0, "sin": 2.0, "cos": 2.0, "erf": 1.5}


def samples(name, n, seed=7):
    rng = np.random.default_rng(seed)
    parts = []
    for r in RANGES[name]:
        if r[0] == "exp":
            parts.append(np.exp(rng.uniform(r[1], r[2], n)))
        else:
            parts.append(rng.uniform(r[0], r[1], n))
    return np.concatenate(parts).astype(np.float32)


def ulp_error(got, x, ref):
    want = np.array([ref(float(v)) for v in x])
    u = np.spacing(np.abs(want.astype(np.float32))).astype(np.float64)
    u[u == 0] = np.float64(np.spacing(np.float32(0)))
    return np.abs(got.astype(np.float64) - want) / u


@pytest.mark.parametrize("name", sorted(REF))
def test_host_build_accuracy(name, oracle_mod):
    x = samples(name, 20000)
    err = ulp_error(oracle_mod.math_eval(name, x), x, REF[name])
    assert err.max() <= MAX_ULP[name], (name, float(err.max()), float(x[err.argmax()]))


def test_special_values(oracle_mod):
    m = oracle_mod.math_eval
    assert m("exp", [0.0])[0] == 1.0 and m("exp", [-200.0])[0] == 0.0 and np.isinf(m("exp", [100.0])[0])
    assert m("log", [1.0])[0] == 0.0 and np.isneginf(m("log", [0.0])[0]) and np.isnan(m("log", [-1.0])[0])
    assert m("sin", [0.0])[0] == 0.0 and m("cos", [0.0])[0] == 1.0
    assert m("erf", [0.0])[0] == 0.0 and m("erf", [6.0])[0] == 1.0 and m("erf", [-6.0])[0] == -1.0
    x = np.linspace(-5, 5, 1001, dtype=np.float32)
    assert np.array_equal(m("erf", -x), -m("erf", x))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(REF))
def test_cuda_build_is_bit_identical(name, oracle_mod):
    import sm_2d_gb300.runtime as rt
    x = np.concatenate([samples(name, 200000, seed=11),
                        np.float32([0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 3.14159274, 1.57079637])])
    if name == "log":
        x = np.abs(x) + np.float32(1e-30)
    got = rt.math_eval(name, x)
    want = oracle_mod.math_eval(name, x)
    same = (got.view(np.uint32) == want.view(np.uint32))
    assert same.all(), (name, int((~same).sum()), float(x[~same][0]))
