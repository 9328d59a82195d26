#!/usr/bin/env python
"""Benchmark: spots/s of the SM_2D K1..K6 transport step on one GB300.

Workload (default, `--workload plan512`, the batching form): a plan of 512
independent pencil-beam spots, energies uniform on the 2 MeV layers of
70-230 MeV, lateral offsets on a 5 mm grid over +-50 mm, sigma_x uniform in
3-6 mm, weights lognormal(0, 0.5), sigma_theta 2 mrad, sigma_E 1 % of E0,
1000 LCG samples per spot; each spot on its own 200 x 400 water domain of
0.5 mm cells; parameters drawn from a seeded generator.  `--workload c2`
runs the production single beam instead: spots of a 150 MeV Gaussian beam
(sigma_x 3.8 mm, sigma_theta 2 mrad, sigma_E 1 % of E0, 1000 samples), sample
seeds differing per spot.  Full coarse/fine pipeline with the conservation
audit every iteration, FP32 phase space, each spot until its in-flight
weight falls below 1e-6 of its injected weight.  Phase-space grids are the
ones the reference code builds and runs: 36 angular bins on +-0.35 rad, the
default piecewise 1029-bin energy grid, 256 local bins (4 theta x 2 E x 8
x_sub x 4 z_sub).  `--grid log` runs the 256 log-E / 512 theta /
128-local-bin variant with the energy-split method instead.

A step is the whole plan: `lanes` spots in flight, a lane refilled with the
plan's next spot inside the device loop as its spot finishes, the lateral
post-convolution of every spot's dose on the device.

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
PLAN_SEED = 2024
PHANTOM_SEED = 7
C3_BEAM = dict(x0=0.0, z0=0.0, theta0=0.0, E0=230.0, W=1.0, sigma_x=5.0, sigma_theta=0.002, sigma_E=1.84,
               n_samples=1000)
MAX_IT = 4000


SMALL = False   # --small: 100 x 200 cells and an 80 MeV beam, for profiler captures


def slab_phantom(Nz, dz, seed=PHANTOM_SEED):
    """The precision form's phantom: 6-10 slabs of 5-30 mm stacked from the
    surface, densities drawn from {0.25 (lung-like), 1.0, 1.85 (bone-like)},
    water below them; one density per depth row."""
    rng = np.random.default_rng(seed)
    rho = np.ones(Nz, np.float32)
    z = 0.0
    for _ in range(int(rng.integers(6, 11))):
        t = float(rng.uniform(5.0, 30.0))
        r = float(rng.choice([0.25, 1.0, 1.85]))
        a, b = int(round(z / dz)), int(round((z + t) / dz))
        rho[a:min(b, Nz)] = r
        z += t
    return rho


def make_config(grid: str, workload: str = "plan512", method: str = "sampled"):
    """The engine configuration of a workload.  method "expect": the
    expectation form (redistribution weights instead of hashed MCS and
    straggling draws; energy split)."""
    cfg = _make_config(grid, workload)
    if method == "expect":
        cfg.energy_split = 1
        cfg.expectation = 1
        cfg.production()
    if method == "precision":
        cfg.precision_form = 1
    return cfg


def _make_config(grid: str, workload: str = "plan512"):
    import sm_2d_gb300 as sm
    if workload == "c3" and not SMALL:
        cfg = sm.Config.reference_runner(300, 600, 0.5, 0.5, N_theta=36, sigma_x_initial=5.0, E0=230.0)
        cfg.density_z = slab_phantom(600, 0.5)
        cfg.max_iterations = MAX_IT
        return cfg.production()
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


def oracle_problem(grid: str, workload: str = "plan512", method: str = "sampled"):
    """The problem of make_config as the CPU oracle takes it, built from the
    oracle's own grid tables (the reference arm loads no part of the GPU
    library): (oracle config dict, theta edges, E edges, density per row or
    None).  The production options are those of Config.production()."""
    from oracle import oracle as orc
    groups = [(0.1, 2.0, 0.1), (2.0, 20.0, 0.2), (20.0, 100.0, 0.25), (100.0, 250.0, 0.25)]
    rho = None
    if workload == "c3" and not SMALL:
        Nx, Nz, sx, E0 = 300, 600, 5.0, 230.0
        rho = slab_phantom(600, 0.5)
    elif SMALL:
        Nx, Nz, sx, E0 = 100, 200, BEAM["sigma_x"], BEAM["E0"]
    else:
        Nx, Nz, sx, E0 = 200, 400, BEAM["sigma_x"], BEAM["E0"]
    if grid == "log" and workload != "c3" and not SMALL:
        th, _ = orc.angular_grid(np.float32(-np.pi / 2), np.float32(np.pi / 2), 512)
        ee, _ = orc.energy_grid_log(0.1, 250.0, 256)
        layout = dict(nt_local=8, ne_local=4, nx_sub=4, nz_sub=1)
        split = 1
    else:
        th, _ = orc.angular_grid(-0.35, 0.35, 36)
        ee, _ = orc.energy_grid_piecewise(groups)
        layout = dict(nt_local=4, ne_local=2, nx_sub=8, nz_sub=4)
        split = 0
    expect = 1 if method == "expect" else 0
    split = 1 if expect else split
    cfg = dict(Nx=Nx, Nz=Nz, dx=0.5, dz=0.5, x_min=-(Nx * 0.5) / 2.0, z_min=0.0, E_fine_on=10.0, E_fine_off=11.0,
               weight_active_min=1e-12, step_coarse=5.0, sigma_x_initial=sx, E0=E0, enable_straggling=1,
               enable_nuclear=1, seed_slot_mode=1, energy_split=split, grid_E_min=0.1, grid_E_max=250.0,
               prune_coarse=0.0, prune_fine=0.0, split_min_weight=1e-7 if split else 0.0,
               stop_weight_fraction=1e-6, floor_cutoff=1, seed_iteration_salt=1, expectation=expect,
               precision_form=1 if method == "precision" else 0, **layout)
    return cfg, th, ee, rho


def spot_seeds(rank, n):
    """Sample seeds of a plan of n spots on `rank`: disjoint across ranks
    (replicas by spot), consecutive within a plan."""
    return [BEAM["seed"] + 100003 * rank + i for i in range(n)]


def plan_spots(workload, rank, n):
    """The plan of `rank`: n spot descriptions (dicts of sm2d_beam fields).
    plan512 draws energy layer, offset, width and weight per spot from a
    generator seeded by rank; c2 repeats the production beam."""
    seeds = spot_seeds(rank, n)
    if workload == "c2" or SMALL:
        return [dict(BEAM, seed=s) for s in seeds]
    if workload == "c3":
        return [dict(C3_BEAM, seed=s) for s in seeds]
    rng = np.random.default_rng(PLAN_SEED + rank)
    out = []
    for s in seeds:
        E0 = 70.0 + 2.0 * int(rng.integers(0, 81))
        x0 = -50.0 + 5.0 * int(rng.integers(0, 21))
        sx = float(rng.uniform(3.0, 6.0))
        w = float(rng.lognormal(0.0, 0.5))
        out.append(dict(x0=x0, z0=0.0, theta0=0.0, E0=E0, W=w, sigma_x=sx, sigma_theta=0.002, sigma_E=0.01 * E0,
                        n_samples=1000, seed=s))
    return out


def plan_sample(workload, n, k=8):
    """Indices of k spots of the plan spread over its energies (lowest and
    highest included): the accuracy sample."""
    spots = plan_spots(workload, 0, n)
    order = sorted(range(len(spots)), key=lambda i: (spots[i]["E0"], i))
    return sorted({order[int(round(j * (len(order) - 1) / (k - 1)))] for j in range(min(k, len(order)))})


def accuracy_leg(grid, workload, spots, idx, dose, results, n_threads, method="sampled"):
    """Errors of the GPU's post-convolved dose maps on the sample spots `idx`
    against the FP32 oracle (the same method and arithmetic) and the FP64
    oracle (the same method in double precision), and the plan's audit
    failure rates.  Dose error: max over cells |d - d_oracle| / max d_oracle,
    the largest over the sample; depth-dose error the same over the PDD."""
    from oracle import oracle as orc
    ocfg, th, ee, rho = oracle_problem(grid, workload, method)
    Nx, Nz, dx = ocfg["Nx"], ocfg["Nz"], ocfg["dx"]
    out = {"spots": [int(i) for i in idx], "energies_mev": [float(spots[i]["E0"]) for i in idx]}
    for fp64 in (False, True):
        os_ = []
        for i in idx:
            b = spots[i]
            o = orc.Oracle(dict(ocfg, E0=b["E0"], sigma_x_initial=b["sigma_x"]), th, ee, fp64=fp64)
            if rho is not None:
                o.set_density(rho)
            o.inject(**b)
            os_.append(o)
        t0 = time.perf_counter()
        orc.run_many(os_, MAX_IT, n_threads)
        wall = time.perf_counter() - t0
        derr, perr, same_peak, same_iters = [], [], 0, 0
        for o, i in zip(os_, idx):
            ref = orc.postprocess(o.tallies()["edep"], o.fe()[2], o.cfg["sigma_x_initial"], Nx, Nz, dx)
            d = dose[i]
            derr.append(float(np.abs(d - ref).max() / ref.max()))
            pg, pr = d.sum(axis=1), ref.sum(axis=1)
            perr.append(float(np.abs(pg - pr).max() / pr.max()))
            same_peak += int(np.argmax(pg) == np.argmax(pr))
            same_iters += int(o.scalars()["iterations"] == results[i]["iterations"])
            o.close()
        out["fp64" if fp64 else "fp32"] = {
            "max_dose_error": max(derr), "max_pdd_error": max(perr), "dose_error_per_spot": derr,
            "bragg_row_equal": f"{same_peak}/{len(idx)}", "iterations_equal": f"{same_iters}/{len(idx)}",
            "oracle_wall_s": wall}
    its = sum(r["iterations"] for r in results)
    out["weight_audit_failure_rate"] = sum(r["weight_audit_failures"] for r in results) / max(its, 1)
    out["energy_audit_failure_rate"] = sum(r["energy_audit_failures"] for r in results) / max(its, 1)
    out["note"] = ("dose errors relative to the oracle's maximum cell dose; audit rates are failed K5 checks "
                   "(W < 1e-6, E < 1e-5 relative) per spot-iteration over the whole plan")
    return out


def plan_rate(grid, workload, n_spots, lanes, steps, warmup, method="sampled", accuracy=False, surrogate=None,
              tol=0.005):
    """spots/s of a plan of n_spots on an engine of `lanes` lanes (0: from free
    memory), device-resident, CUDA events on the library stream; with
    accuracy, also the dose errors of the accuracy sample (accuracy_leg);
    with a calibrated surrogate (expectation form), K3's redistribution
    weights come from the network with the per-row fallback at tol."""
    import torch
    import sm_2d_gb300 as sm
    from sm_2d_gb300.runtime import Beam
    cfg = make_config(grid, workload, method)
    cfg.lanes = lanes if lanes > 0 else min(auto_lanes(cfg, torch.cuda.mem_get_info()[0]), n_spots)
    spots = plan_spots(workload, 0, n_spots)
    beams = [Beam(b["x0"], b["z0"], b["theta0"], b["E0"], b["W"], b["sigma_x"], b["sigma_theta"], b["sigma_E"],
                  b["n_samples"], b["seed"]) for b in spots]
    with sm.Transport(cfg) as t:
        if surrogate is not None:
            t.set_surrogate(surrogate, tol=tol)
        ext = torch.cuda.ExternalStream(t.stream())
        t.plan_load(beams, MAX_IT, dose=accuracy)
        if cfg.lanes > 1:   # the lanes in flight that run this plan fastest (speed only)
            t.tune_lanes_in_flight()
        for _ in range(warmup):
            t.plan_run_async()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            t.plan_run_async()
            e1.record(ext)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        dose, rs = t.plan_results(dose=accuracy)
        passes, _, bins = t.plan_stats()
        sc = t.scalars()
        lanes_used = t.lanes
        in_flight = t.lanes_in_flight()
        sst = t.surrogate_stats() if surrogate is not None else None
    out = {"value": n_spots * steps / (sum(ms) / 1e3), "unit": "spots/s", "lanes": lanes_used,
           "lanes_in_flight": in_flight, "spots": n_spots,
           "ms_per_step": float(np.mean(ms)), "passes_per_step": passes, "bins_per_step": bins,
           "iterations_per_spot": float(np.mean([r["iterations"] for r in rs])),
           "unfinished_spots": sum(1 for r in rs if not r["finished"]),
           "claim_table_overflows": sc["claim_table_overflows"]}
    if sst is not None:
        # rows of the last plan (the stats count since the plan's start)
        out["surrogate_rows_per_step"] = sst["rows"]
        out["fallback_share"] = sst["fallback_rows"] / max(sst["rows"], 1)
        out["rows_beyond_capacity"] = sst["overflow_bins"]
        out["fallback_tol"] = tol
    if accuracy:
        out["accuracy"] = accuracy_leg(grid, workload, spots, plan_sample(workload, n_spots), dose, rs,
                                       os.cpu_count() or 1, method)
    return out


def max_over_ranks(x, dist, device):
    """The largest of a per-rank value (timings take the slowest rank)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def lane_bytes(cfg):
    """Device bytes one lane of a batch engine holds (sm2d_create's allocation):
    ids and page bases per cell, the lane's value pages (32 MB of values
    unless the config says otherwise), tallies, claim rows, bin list and step
    records."""
    nc = cfg.Nx * cfg.Nz
    L = cfg.layout["nt_local"] * cfg.layout["ne_local"] * cfg.layout["nx_sub"] * cfg.layout["nz_sub"]
    pages = min(nc * 32, getattr(cfg, "slot_pages_per_lane", 0) or (8 << 20) // L)
    psi = nc * 32 * 4 + nc * 3 * 4 + pages * (8 + 4 * L)
    per_cell = nc * (2 * 8 + 44 + 44 + 8 + 1 + 4 + 8)
    listed = min(nc, 2048)
    rows = nc * 4096 + listed * 4 * (4096 + 128 + 256 + 4)   # psi_out rows; bucket rows, kept ids, slot map
    bins = min(nc * L // 4, pages * 32) * (56 if getattr(cfg, "expectation", 0) else 48)   # bin list + step records
    return psi + per_cell + rows + bins


def auto_lanes(cfg, free_bytes, cap=512):
    """Lanes filling at most 85 % of the free device memory (at most `cap`,
    the engine's limit).  A pass has a fixed cost that the lanes share: on the
    512-spot plan 16 lanes ran 571, 37 lanes 987, 74 lanes 1280 spots/s with
    dense storage, and 256 lanes 1733, 512 lanes 2135 with value pages."""
    return int(max(1, min(cap, 0.85 * free_bytes // lane_bytes(cfg))))


def workload_desc(workload, grid, n_spots):
    if SMALL:
        return ("profiling case: 80 MeV Gaussian beam (sigma_x 3.8 mm, sigma_theta 2 mrad, sigma_E 0.8 MeV, "
                "1000 samples) in water 100x200 cells @0.5 mm; reference grids; full K1-K6 + audit per iteration")
    if grid == "log":
        ph = "256 log E bins 0.1-250 MeV, 512 theta bins +-pi/2, 128 local bins (8x4x4x1), energy-split method"
    else:
        ph = "reference grids: 1029 piecewise E bins, 36 theta bins +-0.35 rad, 256 local bins (4x2x8x4)"
    if workload == "c3":
        return (f"{n_spots} spots of a 230 MeV Gaussian beam (sigma_x 5 mm, sigma_theta 2 mrad, sigma_E 0.8% E0, 1000 "
                f"samples, sample seeds per spot) into a slab phantom 300x600 cells @0.5 mm (6-10 slabs of 5-30 mm, "
                f"densities 0.25/1.0/1.85, seed {PHANTOM_SEED}); {ph}; full K1-K6 + audit per iteration + lateral dose "
                "post-convolution; each spot until in-flight weight < 1e-6 W0")
    if workload == "c2":
        spots = (f"{n_spots} spots of a 150 MeV Gaussian beam (sigma_x 3.8 mm, sigma_theta 2 mrad, sigma_E 1.5 MeV, "
                 "1000 samples, sample seeds per spot)")
    else:
        spots = (f"{n_spots} pencil-beam spots: E uniform on 70-230 MeV 2 MeV layers, x0 on a 5 mm grid over "
                 "+-50 mm, sigma_x U[3,6] mm, weights lognormal(0,0.5), sigma_theta 2 mrad, sigma_E 1% E0, "
                 f"1000 samples each (generator seed {PLAN_SEED})")
    return (f"{spots}; each spot in its own water domain 200x400 cells @0.5 mm; {ph}; full K1-K6 + audit per "
            "iteration + lateral dose post-convolution; each spot until in-flight weight < 1e-6 W0")


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
def cpu_spots_per_s(grid: str, workload: str, n_threads: int, n_spots: int):
    """Transport the first n_spots spots of the plan on the CPU oracle (each
    with the Fermi-Eyges tables of its own energy and width), n_threads at a
    time; returns (spots/s, wall seconds)."""
    from oracle import oracle as orc
    ocfg, th, ee, rho = oracle_problem(grid, workload)
    oracles = []
    for b in plan_spots(workload, 0, n_spots):
        o = orc.Oracle(dict(ocfg, E0=b["E0"], sigma_x_initial=b["sigma_x"]), th, ee)
        if rho is not None:
            o.set_density(rho)
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
        cpu_spots_per_s(args.grid, args.workload, n_threads, n_threads)
    vals, walls = [], []
    for _ in range(args.steps):
        v, dt = cpu_spots_per_s(args.grid, args.workload, n_threads, n_threads)
        vals.append(v)
        walls.append(dt)
    value = float(len(vals) * n_threads / sum(walls))
    sample = (f"the first {n_threads} spots of the plan per step (one per host thread), full transport of each "
              "(the plan's spots are independent: spots/s of a sample is the plan's rate)")
    line = {"metric": METRIC, "value": value, "unit": "spots/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(walls)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_desc(args.workload, args.grid, args.spots), "grid": args.grid},
            "cpu_baseline": {"value": value, "unit": "spots/s", "cores": n_threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "spots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU arm
def surrogate_leg(n_train=10_000_000, steps=10000, n_eval=1 << 22, tol=0.005):
    """The learned redistribution surrogate next to the method it replaces.

    Trains the network on the method's own tables (K3 physics on the device),
    calibrates the per-region fallback, and times on the library stream with
    CUDA events, on n_eval fresh rows: the method's table kernel, the
    network's tcgen05 inference kernel, and the network with fallback.  The
    tensor roofline of the inference kernel counts the network's algorithmic
    FLOPs, 2 (4*128 + 128*128 + 128*32) = 41,984 per row.
    """
    import torch
    import sm_2d_gb300 as sm

    s = sm.Surrogate()
    L, m = s.L, s.m
    stream = torch.cuda.ExternalStream(s.t.stream())
    f = s.features(n_train, 101)
    y = s.plain(f)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    hist = s.train(f, y, steps=steps)
    ev[1].record(stream)
    torch.cuda.synchronize()
    train_ms = ev[0].elapsed_time(ev[1])
    s.calibrate(s.features(1 << 20, 102))
    fe = s.features(n_eval, 103)
    out = torch.empty((n_eval, 32), dtype=torch.float32, device="cuda")
    ref = torch.empty_like(out)
    fb = torch.zeros(n_eval, dtype=torch.int32, device="cuda")
    P = C.c_void_p

    def timed(fn, reps=10):
        fn()
        s.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        s.sync()
        return e0.elapsed_time(e1) / reps

    ck = sm.runtime.check   # a refused or failed launch raises instead of timing nothing
    t_plain = timed(lambda: ck(L.sm2d_redistribution_table(s.t.h, P(fe.data_ptr()), n_eval, P(ref.data_ptr()))))
    t_net = timed(lambda: ck(L.sm2d_mlp_forward(m, P(fe.data_ptr()), n_eval, P(out.data_ptr()))))
    err = (out - ref).abs()
    mean_err = float(err.mean())
    t_fb = timed(lambda: ck(L.sm2d_mlp_redistribute(m, s.t.h, P(fe.data_ptr()), n_eval, tol, P(out.data_ptr()),
                                                    P(fb.data_ptr()))))
    row_err = (out - ref).abs().max(dim=1).values
    fb_share = float(fb.float().mean())
    flops = 41984.0 * n_eval
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, src = float(json.load(open(peaks_path))["bf16_tflops"]), "measured (cuBLAS bf16 burst)"
    else:
        peak, src = 1900.0, "fallback"
    achieved = flops / (t_net * 1e-3) / 1e12
    train_flops = 3.0 * 41984.0 * s.batch * steps
    res = {
        "network": "4-128-128-32 ReLU MLP, softmax, bf16 operands, fp32 accumulate (tcgen05)",
        "training": {"samples": n_train, "steps": steps, "batch": s.batch, "ms": train_ms,
                     "samples_per_s": s.batch * steps / (train_ms * 1e-3),
                     "tflops": train_flops / (train_ms * 1e-3) / 1e12,
                     "loss_first": float(hist[0]), "loss_last": float(np.mean(hist[-50:]))},
        "rows": n_eval,
        "plain_rows_per_s": n_eval / (t_plain * 1e-3),
        "surrogate_rows_per_s": n_eval / (t_net * 1e-3),
        "surrogate_with_fallback_rows_per_s": n_eval / (t_fb * 1e-3),
        "surrogate_over_plain": t_plain / t_net,
        "mean_abs_weight_error": mean_err,
        "fallback_tol": tol, "fallback_share": fb_share,
        "row_max_error_q99": float(torch.quantile(row_err[:1 << 20], 0.99)),
        "row_max_error_max": float(row_err.max()),
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_source": src, "kernel": "k_infer",
                     "avg_launch_ms": t_net, "algorithmic_flops_per_launch": flops},
    }
    return res, s


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

    cfg = make_config(args.grid, args.workload)
    cfg.lanes = args.lanes if args.lanes > 0 else min(auto_lanes(cfg, torch.cuda.mem_get_info()[0]), args.spots)
    t = sm.Transport(cfg)
    B = t.lanes
    ext = torch.cuda.ExternalStream(t.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2
    lib = t._lib

    # this rank's plan: the spots are independent (replicas by spot)
    n = args.spots
    spots = plan_spots(args.workload, rank, n)
    beams = [Beam(b["x0"], b["z0"], b["theta0"], b["E0"], b["W"], b["sigma_x"], b["sigma_theta"], b["sigma_E"],
                  b["n_samples"], b["seed"]) for b in spots]
    beam_arr = (Beam * n)(*beams)

    # ---- device-resident plan: beams and Fermi-Eyges tables staged in HBM
    # before the timed region; each step transports the whole plan and
    # leaves the post-convolved dose of every spot in HBM
    t.plan_load(beams, MAX_IT, dose=True)
    # the launch shape (blocks per SM of each pass kernel) from the autotuner,
    # on this plan, before the timed region
    shape, tune_ms = t.autotune() if not args.no_tune else (t.launch_shape(), None)
    if args.lanes_in_flight > 0:   # a fixed number of lanes in flight instead of the tuner's choice
        t.set_lanes_in_flight(min(args.lanes_in_flight, B))
    lif = t.lanes_in_flight()   # the tuner's choice of lanes in flight (every lane with --no-tune)
    for _ in range(max(args.warmup, 3)):
        t.plan_run_async()
    torch.cuda.synchronize()
    times, launches, cell_steps, bins_done, iters = [], 0, 0.0, 0.0, []
    per_pass = 7 if cfg.use_buckets else 6
    barrier()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            t.plan_run_async()
            e1.record(ext)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            _, rs = t.plan_results(dose=False)
            passes, refills, bins = t.plan_stats()
            cell_steps += sum(r["cell_steps"] for r in rs)
            bins_done += bins
            iters = [r["iterations"] for r in rs]
            # reset 3, plan begin 1, first fill 9 (dose/tally clear, lane
            # assignment and fill, injection 6), plan end 1; per pass of the
            # device loop (the halting one included) classify, claim pass,
            # bucket and psi_out selection, deposit pass, finalize (+ bucket
            # move); 9 per refill
            launches += 14 + (passes + 1) * per_pass + 9 * (refills - 1)
    barrier()
    total_ms = max_over_ranks(np.sum(times), dist, "cuda")
    value = args.steps * n * world / (total_ms / 1e3)
    unfinished = sum(1 for r in rs if not r["finished"])

    # ---- end to end through the public batch entry with pinned host buffers:
    # beam descriptions in (the Fermi-Eyges tables computed on the host per
    # spot), one post-convolved dose map per spot out
    dose_host = torch.zeros(n * cfg.Nx * cfg.Nz, dtype=torch.float64).pin_memory()
    beam_pin = torch.zeros(C.sizeof(Beam) * n, dtype=torch.uint8).pin_memory()
    C.memmove(beam_pin.data_ptr(), C.addressof(beam_arr), C.sizeof(Beam) * n)
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        rc = lib.sm2d_batch_run(t.h, C.c_void_p(beam_pin.data_ptr()), n, MAX_IT, C.c_void_p(dose_host.data_ptr()),
                                None)
        e1.record(ext)
        e1.synchronize()
        if rc != 0:
            raise RuntimeError(lib.sm2d_last_error().decode())
        e2e_times.append(e0.elapsed_time(e1))
    e2e_ms = max_over_ranks(np.sum(e2e_times), dist, "cuda")
    e2e_value = args.steps * n * world / (e2e_ms / 1e3)

    # ---- per-kernel device time: eager replay of one wave of the plan's first
    # `lanes` spots with CUDA events around every launch on the library stream
    t.batch_inject(beams[:lif])   # the wave holds as many spots as a plan keeps in flight
    n_it, ms, n_launch, wave_passes = t.run_profiled(MAX_IT)
    prs = t.batch_results(min(B, n))
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
    plan_passes = passes
    traffic = None
    tp = os.path.join(ROOT, "profiles", f"k_transport_traffic_{args.workload}.json")
    if os.path.exists(tp) and not SMALL and args.grid == "reference":
        # DRAM bytes per deposit launch from an ncu capture of the same kind of
        # wave, per lane, scaled by the wave's lanes (the lanes' work adds up)
        tr = json.load(open(tp))
        traffic = tr["dram_bytes_per_launch_per_lane"] * lif
    step_total = sum(ms.values())
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_src, "kernel": "k_transport (deposit pass)",
                "algorithmic_bytes_per_launch": alg_bytes / max(wave_passes, 1),
                "avg_launch_ms": ms["transport"] / max(wave_passes, 1),
                "launches_timed": wave_passes, "launches_per_step": plan_passes,
                "stage_share": {k: v / step_total for k, v in ms.items()} if step_total else {},
                "note": "per-launch times from an eager replay of one wave (the plan's first lanes' spots, "
                        "launches_timed passes) with CUDA events around each kernel on the library stream; one "
                        "deposit launch per pass, launches_per_step passes per plan"}

    plan_scalars = t.scalars()
    accuracy = None
    if rank == 0 and not args.no_accuracy and not SMALL:
        dose_all, rs_all = t.plan_results(dose=True)
        accuracy = accuracy_leg(args.grid, args.workload, spots, plan_sample(args.workload, n), dose_all, rs_all,
                                os.cpu_count() or 1)
        del dose_all
    t.close()
    del flush
    torch.cuda.empty_cache()

    # context figures on the same box: the plan on the 256 log-E / 512 theta /
    # 128-local-bin grid (energy-split method), and the plain engine with one
    # lane (one spot at a time, as the reference runner transports them)
    extra = {}
    if rank == 0 and not args.no_context and not SMALL and args.workload == "plan512":
        if args.grid == "reference":
            extra["grid_log"] = plan_rate("log", args.workload, n, 0, 2, 1)
        extra["single_lane"] = plan_rate(args.grid, args.workload, 24, 1, 2, 1)
        extra["single_lane"]["note"] = ("the first 24 spots of the plan on an engine of one lane (one spot in "
                                        "flight, refilled on the device)")
        extra["expectation"] = plan_rate(args.grid, args.workload, n, 0, 2, 1, "expect", accuracy=True)
        extra["expectation"]["method"] = ("expectation form: K2/K3 emit the expected re-binning of their MCS angle "
                                          "and straggling loss (up to 15 theta x 4 E children per component) "
                                          "instead of one hashed draw; energy split")
        # the precision form on its own workload (C3: 230 MeV through the slab
        # phantom, 64 spots): weight increments in the audit, the R-LUT
        # inverted in double below 10 MeV; and on the 512-spot plan
        extra["precision"] = plan_rate(args.grid, "c3", 64, 0, 2, 1, "precision", accuracy=True)
        extra["precision"]["workload"] = workload_desc("c3", args.grid, 64)
        extra["precision_plan512"] = plan_rate(args.grid, args.workload, n, 0, 2, 1, "precision", accuracy=True)

    cpu = None
    if rank == 0 and not args.no_cpu:
        n_threads = os.cpu_count() or 1
        v, dt = cpu_spots_per_s(args.grid, args.workload, n_threads, n_threads)
        cpu = {"value": v, "unit": "spots/s", "cores": n_threads, "kind": "port",
               "sample": f"the plan's first {n_threads} spots, one per host thread, full transport ({dt:.1f} s wall)"}

    surrogate = None
    if rank == 0 and not args.no_surrogate and not SMALL:
        surrogate, net = surrogate_leg()
        if args.workload == "plan512" and not args.no_context:
            # surrogate + batched: the plan in the expectation form with K3's
            # redistribution weights from the network, the per-row fallback at
            # the workload's 0.5 % and at a stricter 0.2 %
            for key, tol in (("transport", 0.005), ("transport_tol_0.002", 0.002)):
                st = plan_rate(args.grid, args.workload, n, 0, 2, 1, "expect", accuracy=True, surrogate=net, tol=tol)
                st["method"] = ("expectation form with the learned surrogate: K3 bins whose energy window has "
                                "uniformly spaced centres take their 8 theta x 4 E weights from the network; rows "
                                "whose calibrated region error exceeds the tolerance keep the closed forms")
                st["over_plain"] = st["value"] / value
                if "expectation" in extra:
                    st["over_expectation_form"] = st["value"] / extra["expectation"]["value"]
                surrogate[key] = st
        net.close()

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "spots/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload_desc(args.workload, args.grid, n), "grid": args.grid,
                           "method": "plain K1-K6 (direct neighbour scatter), deterministic slot claims",
                           "step": f"one plan of {n} spots, {lif} in flight on {B} lanes, lanes refilled on the device",
                           "lanes": B, "lanes_in_flight": lif, "spots_per_step": n,
                           "iterations_per_spot": float(np.mean(iters)),
                           "launch_shape": {"blocks_per_sm": dict(zip(["cell_kernels", "finalize", "claim_pass",
                                                                       "deposit_pass"], shape)),
                                            "source": "sm2d_autotune on this plan" if tune_ms else "default",
                                            "tuned_plan_ms": tune_ms},
                           "unfinished_spots": unfinished,
                           "l2": "inputs larger than L2 (GBs of phase space per step); 256 MB flush between steps",
                           "parallelism": f"{n} spots per GPU per step, replicas by spot x{world}"},
                "cell_steps_per_s": cell_steps * world / (total_ms / 1e3) if total_ms else None,
                "bins_per_s": bins_done * world / (total_ms / 1e3) if total_ms else None,
                "e2e": {"value": e2e_value, "unit": "spots/s", "h2d_bytes_per_step": int(C.sizeof(Beam) * n),
                        "d2h_bytes_per_step": int(cfg.Nx * cfg.Nz * 8 * n)},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": launches, "accuracy": accuracy,
                "claim_table_overflows": plan_scalars["claim_table_overflows"], **extra, "surrogate": surrogate}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def stage_profile(lanes=128):
    """Per-pass device time of each stage (µs, CUDA events around every kernel
    of an eager replay) for one wave of the plan's first `lanes` spots, in the
    sampled form, the expectation form and the expectation form with the
    learned surrogate serving K3's redistribution (fallback at 0.5 %)."""
    import sm_2d_gb300 as sm
    from sm_2d_gb300.runtime import Beam
    spots = plan_spots("plan512", 0, lanes)
    beams = [Beam(b["x0"], b["z0"], b["theta0"], b["E0"], b["W"], b["sigma_x"], b["sigma_theta"], b["sigma_E"],
                  b["n_samples"], b["seed"]) for b in spots]
    _, net = surrogate_leg()
    out = {}
    for key, method, use_net in (("sampled", "sampled", False), ("expectation", "expect", False),
                                 ("surrogate", "expect", True)):
        cfg = make_config("reference", "plan512", method)
        cfg.lanes = lanes
        with sm.Transport(cfg) as t:
            if use_net:
                t.set_surrogate(net, tol=0.005)
            t.batch_inject(beams)
            _, ms, _, passes = t.run_profiled(MAX_IT)
        out[key] = {"passes": passes, "us_per_pass": {k: round(v / passes * 1000.0, 1) for k, v in ms.items()},
                    "wave_ms": round(sum(ms.values()), 1)}
    net.close()
    return {"workload": f"the 512-spot plan's first {lanes} spots as one wave on {lanes} lanes", "forms": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", default="reference", choices=["reference", "log"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the learned-surrogate leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the dose-error leg against the oracles")
    ap.add_argument("--no-context", action="store_true", help="skip the log-grid and single-lane context figures")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape (no autotuner run)")
    ap.add_argument("--lanes", type=int, default=0, help="spots in flight (0: from free device memory)")
    ap.add_argument("--lanes-in-flight", type=int, default=0,
                    help="lanes a plan keeps in flight (0: the autotuner's choice, every lane with --no-tune)")
    ap.add_argument("--workload", default="plan512", choices=["plan512", "c2", "c3"])
    ap.add_argument("--spots", type=int, default=0, help="spots per step, the plan (0: 512; 64 for c3)")
    ap.add_argument("--small", action="store_true",
                    help="100x200 cells, 80 MeV beam: a small case for profiler captures (not a bench line)")
    ap.add_argument("--stage-profile", action="store_true",
                    help="print the per-pass stage times of the sampled, expectation and surrogate forms (not a bench line)")
    args = ap.parse_args()
    if args.stage_profile:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(stage_profile()))
        return 0
    if args.spots <= 0:
        args.spots = 64 if args.workload == "c3" else 512
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
