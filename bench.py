#!/usr/bin/env python
"""Benchmark: spots/s of the SM_2D K1..K6 transport step on one GB300.

Workload (the production single-beam case): a 150 MeV Gaussian proton beam
(sigma_x 3.8 mm, sigma_theta 2 mrad, sigma_E 1 % of E0, 1000 LCG samples,
seed 42) into homogeneous water, 200 x 400 cells of 0.5 mm (100 x 200 mm),
full coarse/fine pipeline with the conservation audit every iteration, FP32
phase space.  Phase-space grids are the ones the reference code builds and
runs: 36 angular bins on +-0.35 rad, the default piecewise 1029-bin energy
grid, 256 local bins (4 theta x 2 E x 8 x_sub x 4 z_sub).  `--grid log` runs
the 256 log-E / 512 theta / 128-local-bin variant with the energy-split
method instead.  A step is one wave: `lanes` spots of that beam (sample seeds
differ per spot) transported together to completion (until the in-flight
weight of each falls below 1e-6 of its injected weight).

Arms: default = libsm2d.so on the GPU; `--impl reference` = the reference's
algorithm on the host cores (the CPU restatement in oracle/, all threads, one
spot per thread), since the reference has no CPU transport of its own.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "spots/s on 1 GB300, surrogate+batched vs plain K1–K6, at ≤1% dose error"
BEAM = dict(x0=0.0, z0=0.0, theta0=0.0, E0=150.0, W=1.0, sigma_x=3.8, sigma_theta=0.002, sigma_E=1.5,
            n_samples=1000, seed=42)
MAX_IT = 4000


SMALL = False   # --small: 100 x 200 cells and an 80 MeV beam, for profiler captures


def make_config(grid: str):
    import sm_2d_gb300 as sm
    if SMALL:
        cfg = sm.Config.reference_runner(100, 200, 0.5, 0.5, N_theta=36, sigma_x_initial=BEAM["sigma_x"],
                                         E0=BEAM["E0"])
        cfg.max_iterations = MAX_IT
        return cfg.production()
    if grid == "log":
        cfg = sm.Config.log_grid(200, 400, 0.5, 0.5, N_E=256, E_min=0.1, E_max=250.0, N_theta=512,
                                 theta_max=np.pi / 2, layout=sm.LAYOUT_B128, E_fine_on=10.0, E_fine_off=11.0,
                                 sigma_x_initial=BEAM["sigma_x"], E0=BEAM["E0"], energy_split=1)
    else:
        cfg = sm.Config.reference_runner(200, 400, 0.5, 0.5, N_theta=36, sigma_x_initial=BEAM["sigma_x"],
                                         E0=BEAM["E0"])
    cfg.max_iterations = MAX_IT
    return cfg.production()


def spot_seeds(rank, lanes):
    """Sample seeds of one wave on `rank`: disjoint across ranks (replicas by
    spot), consecutive within a wave."""
    return [BEAM["seed"] + 100003 * rank + i for i in range(lanes)]


def max_over_ranks(x, dist, device):
    """The largest of a per-rank value (timings take the slowest rank)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def lane_bytes(cfg):
    """Device bytes one lane of the engine holds (sm2d_create's allocation)."""
    nc = cfg.Nx * cfg.Nz
    L = cfg.layout["nt_local"] * cfg.layout["ne_local"] * cfg.layout["nx_sub"] * cfg.layout["nz_sub"]
    psi = nc * 32 * (4 + 4 * L)
    per_cell = nc * (2 * 8 + 44 + 44 + 8 + 1 + 4 + 8)
    rows = nc * 2048 + (nc // 8) * 4 * (2048 + 128 + 4)
    bins = nc * L // 4 * 16
    return psi + per_cell + rows + bins


def auto_lanes(cfg, free_bytes, cap=64):
    """Lanes filling at most 60 % of the free device memory (at most `cap`)."""
    return int(max(1, min(cap, 0.6 * free_bytes // lane_bytes(cfg))))


def workload_desc(grid, L):
    if SMALL:
        return ("profiling case: 80 MeV Gaussian beam (sigma_x 3.8 mm, sigma_theta 2 mrad, sigma_E 0.8 MeV, "
                "1000 samples) in water 100x200 cells @0.5 mm; reference grids; full K1-K6 + audit per iteration")
    if grid == "log":
        ph = "256 log E bins 0.1-250 MeV, 512 theta bins +-pi/2, 128 local bins (8x4x4x1), energy-split method"
    else:
        ph = "reference grids: 1029 piecewise E bins, 36 theta bins +-0.35 rad, 256 local bins (4x2x8x4)"
    return ("150 MeV Gaussian beam (sigma_x 3.8 mm, sigma_theta 2 mrad, sigma_E 1.5 MeV, 1000 samples) "
            f"in water 200x400 cells @0.5 mm; {ph}; full K1-K6 + audit per iteration; until in-flight "
            f"weight < 1e-6 W0")


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm_ = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm_)) if sm_ else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------- CPU arm
def cpu_spots_per_s(grid: str, n_threads: int, n_spots: int):
    """Transport n_spots independent copies of the workload on the CPU oracle,
    n_threads at a time; returns (spots/s, wall seconds)."""
    from oracle import oracle as orc
    cfg = make_config(grid)
    oc = cfg.oracle_config()
    oracles = []
    for i in range(n_spots):
        o = orc.Oracle(oc, cfg.theta_edges, cfg.E_edges)
        b = dict(BEAM)
        o.inject(**b)
        oracles.append(o)
    t0 = time.perf_counter()
    orc.run_many(oracles, MAX_IT, n_threads)
    dt = time.perf_counter() - t0
    for o in oracles:
        o.close()
    return n_spots / dt, dt


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n_threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_spots_per_s(args.grid, n_threads, n_threads)
    vals, walls = [], []
    for _ in range(args.steps):
        v, dt = cpu_spots_per_s(args.grid, n_threads, n_threads)
        vals.append(v)
        walls.append(dt)
    value = float(len(vals) * n_threads / sum(walls))
    cfg = make_config(args.grid)
    sample = f"{n_threads} spots per step (one per host thread), full transport of each"
    line = {"metric": METRIC, "value": value, "unit": "spots/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(walls)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_desc(args.grid, cfg.layout), "grid": args.grid},
            "cpu_baseline": {"value": value, "unit": "spots/s", "cores": n_threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "spots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU arm
def run_gpu_arm(args):
    import torch
    import sm_2d_gb300 as sm
    from sm_2d_gb300.runtime import Beam

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.all_reduce(torch.zeros(1, device="cuda"))
            torch.cuda.synchronize()

    cfg = make_config(args.grid)
    cfg.lanes = args.lanes if args.lanes > 0 else auto_lanes(cfg, torch.cuda.mem_get_info()[0])
    t = sm.Transport(cfg)
    B = t.lanes
    ext = torch.cuda.ExternalStream(t.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    # one wave = B spots of the workload beam, sample seeds differing per spot
    beams = [Beam(BEAM["x0"], BEAM["z0"], BEAM["theta0"], BEAM["E0"], BEAM["W"], BEAM["sigma_x"],
                  BEAM["sigma_theta"], BEAM["sigma_E"], BEAM["n_samples"], seed) for seed in spot_seeds(rank, B)]
    beam_arr = (Beam * B)(*beams)
    lib = t._lib

    def one_wave():
        t.batch_inject(beams)
        t.run_async(MAX_IT)

    for _ in range(max(args.warmup, 3)):
        one_wave()
    torch.cuda.synchronize()
    res = t.batch_results(B)
    iters = [r["iterations"] for r in res]

    # ---- timed region: K waves of B spots, device time per wave (every wave
    # streams GBs of phase space, far more than L2; L2 is flushed between waves too)
    times = []
    launches = 0
    cell_steps = 0.0
    barrier()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            one_wave()
            e1.record(ext)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            rs = t.batch_results(B)
            passes = max(r["iterations"] for r in rs) + 1
            cell_steps += sum(r["cell_steps"] for r in rs)
            # reset 3 + injection 6 + loop limit 1, then per pass of the device
            # loop classify, claim pass, bucket and psi_out selection, deposit
            # pass, finalize (+ bucket move)
            launches += 10 + (7 if cfg.use_buckets else 6) * passes
    barrier()
    total_ms = max_over_ranks(np.sum(times), dist, "cuda")
    spots = args.steps * B * world
    value = spots / (total_ms / 1e3)

    # ---- end to end through the public batch entry with pinned host buffers:
    # beam descriptions in, one dose map per spot out
    dose_host = torch.zeros(B * cfg.Nx * cfg.Nz, dtype=torch.float64).pin_memory()
    beam_pin = torch.zeros(C.sizeof(Beam) * B, dtype=torch.uint8).pin_memory()
    C.memmove(beam_pin.data_ptr(), C.addressof(beam_arr), C.sizeof(Beam) * B)
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        rc = lib.sm2d_batch_run(t.h, C.c_void_p(beam_pin.data_ptr()), B, MAX_IT, C.c_void_p(dose_host.data_ptr()),
                                None)
        e1.record(ext)
        e1.synchronize()
        if rc != 0:
            raise RuntimeError(lib.sm2d_last_error().decode())
        e2e_times.append(e0.elapsed_time(e1))
    e2e_ms = max_over_ranks(np.sum(e2e_times), dist, "cuda")
    e2e_value = spots / (e2e_ms / 1e3)

    # ---- per-kernel device time: eager replay of one wave with CUDA events
    # around every launch on the library stream
    t.batch_inject(beams)
    n_it, ms, n_launch = t.run_profiled(MAX_IT)
    prs = t.batch_results(B)
    L = t.L
    slot_bytes = 4 + 4 * L
    alg_bytes = sum((r["slots_in"] + r["slots_out"]) * slot_bytes + 44.0 * r["cell_steps"] for r in prs)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peaks = json.load(open(peaks_path))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = alg_bytes / (ms["transport"] / 1e3) / 1e9 if ms["transport"] > 0 else 0.0
    traffic = None
    tp = os.path.join(ROOT, "profiles", "k_transport_traffic.json")
    if os.path.exists(tp) and not SMALL and args.grid == "reference":
        # DRAM bytes per deposit launch from the ncu capture of this workload
        # (recorded per lane; the lanes' work adds up)
        tr = json.load(open(tp))
        traffic = tr["dram_bytes_per_launch_per_lane"] * B
    step_total = sum(ms.values())
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_src, "kernel": "k_transport (deposit pass)",
                "algorithmic_bytes_per_launch": alg_bytes / max(n_it, 1),
                "avg_launch_ms": ms["transport"] / max(n_it, 1),
                "stage_share": {k: v / step_total for k, v in ms.items()} if step_total else {},
                "note": "per-launch times from an eager replay of one wave with CUDA events around each "
                        "kernel on the library stream"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        n_threads = os.cpu_count() or 1
        v, dt = cpu_spots_per_s(args.grid, n_threads, n_threads)
        cpu = {"value": v, "unit": "spots/s", "cores": n_threads, "kind": "port",
               "sample": f"{n_threads} spots, one per host thread, full transport ({dt:.1f} s wall)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "spots/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload_desc(args.grid, cfg.layout), "grid": args.grid,
                           "method": "plain K1-K6 (direct neighbour scatter), deterministic slot claims",
                           "step": f"one wave of {B} spots transported together (lanes)", "lanes": B,
                           "iterations_per_spot": float(np.mean(iters)),
                           "l2": "inputs larger than L2 (GBs of phase space per wave); 256 MB flush between waves",
                           "parallelism": f"{B} spots per GPU, replicas by spot x{world}"},
                "cell_steps_per_s": cell_steps * world / (total_ms / 1e3) if total_ms else None,
                "e2e": {"value": e2e_value, "unit": "spots/s", "h2d_bytes_per_step": int(C.sizeof(Beam) * B),
                        "d2h_bytes_per_step": int(cfg.Nx * cfg.Nz * 8 * B)},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": launches}
        print(json.dumps(line))
    t.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", default="reference", choices=["reference", "log"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--lanes", type=int, default=0, help="spots per wave (0: from free device memory)")
    ap.add_argument("--small", action="store_true",
                    help="100x200 cells, 80 MeV beam: a small case for profiler captures (not a bench line)")
    args = ap.parse_args()
    if args.small:
        global SMALL
        SMALL = True
        BEAM["E0"] = 80.0
        BEAM["sigma_E"] = 0.8
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
