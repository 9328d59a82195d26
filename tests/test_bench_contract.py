"""bench.py's output contract on the CPU: the reference arm (the oracle port
on the host cores) prints one JSON line with the keys the driver reads, and
the lane count follows the device memory the engine would take."""
import json
import os
import subprocess
import sys

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--small", "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 1
    assert d["unit"] == "spots/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["vs_baseline"] is None and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "spots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


@pytest.mark.parametrize("workload", ["plan512", "c2", "c3"])
def test_lanes_follow_free_memory(workload):
    cfg = bench.make_config("reference", workload)
    per = bench.lane_bytes(cfg)
    nc = cfg.Nx * cfg.Nz
    dense = nc * 32 * 1028                     # every slot of every cell with its 256 values
    pages = min(nc * 32, 32768) * 1024         # the lane's value pages
    assert pages + nc * 4096 < per < dense / 2  # pages and psi_out claim rows, far below a dense phase space
    assert bench.auto_lanes(cfg, 0) == 1       # always at least one lane
    assert bench.auto_lanes(cfg, 10 ** 15) == 512
    free = 280 * 2 ** 30
    n = bench.auto_lanes(cfg, free)
    assert n * per <= 0.85 * free < (n + 1) * per or n == 512


@pytest.mark.parametrize("grid,workload", [("reference", "plan512"), ("log", "plan512"), ("reference", "c3")])
def test_reference_arm_problem_equals_the_gpu_arm_problem(grid, workload):
    """The reference arm builds its oracle problem from the oracle's own grid
    tables; it must be the problem the GPU arm transports."""
    cfg = bench.make_config(grid, workload)
    ocfg, th, ee, rho = bench.oracle_problem(grid, workload)
    want = cfg.oracle_config()
    assert set(want) <= set(ocfg)
    for k, v in want.items():
        assert ocfg[k] == pytest.approx(v, rel=0, abs=0), k
    assert (th == cfg.theta_edges).all() and (ee == cfg.E_edges).all()
    assert (rho is None) == (cfg.density_z is None)
    if rho is not None:
        assert (rho == cfg.density_z).all()


def test_reference_arm_does_not_load_the_gpu_library():
    code = ("import sys, bench; bench.cpu_spots_per_s('reference', 'plan512', 1, 1); "
            "assert 'sm_2d_gb300' not in sys.modules, sorted(m for m in sys.modules if 'sm_2d' in m)")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
