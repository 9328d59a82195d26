"""Golden fixtures from the reference's own GPU build, run on a GB300.

``oracle/ref_gpu_build.sh stage`` (where the SM_2D tree is mounted) and
``oracle/ref_gpu_build.sh build`` (on the box) give
``oracle/_ref/gpu/run_simulation_dumps``: the reference tree's run_simulation
compiled for sm_103a with SM2D_ENABLE_DEBUG_DUMPS.  This script runs it on the
four one-step validation cases (docs/val_test/cases/case_{a..d}.ini, stored
here as one_step_case_X/case.ini) for ten iterations each and keeps the dumps
the reference writes (results/debug_ps_raw_iter_NN_*.csv: the phase space
after source injection and after K4 of iterations 1..10, with slots, block ids,
local bins and weights): ``ref_gpu/case_X/``.

With --timing it also runs the reference's plain build (no dumps) on spots of
the benchmark's workloads and writes their wall times (the reference_gpu
figure of the design notes) to the output directory.

Usage on a GB300, from the repository root:
    python tests/golden/make_golden_gpu.py --out <output folder> [--timing]
"""
import argparse
import configparser
import json
import os
import shutil
import subprocess
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE_DIR = os.path.join(ROOT, "oracle", "_ref", "gpu")
ITERATIONS = 10


def read_ini(path):
    """The case's INI sections with the key spelling the reference's loader expects."""
    cp = configparser.ConfigParser()
    cp.optionxform = str
    cp.read(path)
    return {sec: dict(cp[sec]) for sec in cp.sections()}


def write_ini(path, cfg):
    with open(path, "w") as fh:
        for sec, kv in cfg.items():
            fh.write(f"[{sec}]\n")
            for k, v in kv.items():
                fh.write(f"{k} = {v}\n")
            fh.write("\n")


def run(exe, cfg, work):
    """run_simulation on cfg in directory work (its dumps go to work/results);
    returns the wall time and the exit code."""
    os.makedirs(os.path.join(work, "results"), exist_ok=True)
    cfg["output"]["output_dir"] = os.path.join(work, "out")
    os.makedirs(cfg["output"]["output_dir"], exist_ok=True)
    ini = os.path.join(work, "case.ini")
    write_ini(ini, cfg)
    # the reference reads its PSTAR table from src/data/nist (a path relative to the working directory)
    os.makedirs(os.path.join(work, "src", "data", "nist"), exist_ok=True)
    shutil.copyfile(os.path.join(ROOT, "oracle", "_ref", "tree", "src", "data", "nist", "pstar_water.txt"),
                    os.path.join(work, "src", "data", "nist", "pstar_water.txt"))
    t0 = time.perf_counter()
    r = subprocess.run([exe, ini], cwd=work, capture_output=True, text=True, timeout=1800)
    dt = time.perf_counter() - t0
    with open(os.path.join(work, "stdout.txt"), "w") as fh:
        fh.write(r.stdout[-20000:] + "\n--- stderr ---\n" + r.stderr[-20000:])
    return dt, r.returncode


def golden(out):
    exe = os.path.join(EXE_DIR, "run_simulation_dumps")
    for case in "ABCD":
        cfg = read_ini(os.path.join(HERE, f"one_step_case_{case}", "case.ini"))
        cfg["transport"]["max_iterations"] = str(ITERATIONS)
        cfg["grid"]["max_steps"] = str(ITERATIONS)
        cfg["transport"]["log_level"] = "0"
        work = tempfile.mkdtemp(prefix=f"ref_case_{case}_")
        dt, rc = run(exe, cfg, work)
        dst = os.path.join(out, f"case_{case}")
        os.makedirs(dst, exist_ok=True)
        kept = []
        for f in sorted(os.listdir(os.path.join(work, "results"))):
            if f.startswith("debug_ps_raw_iter_") or f.startswith("debug_channels_totals"):
                shutil.copyfile(os.path.join(work, "results", f), os.path.join(dst, f))
                kept.append(f)
        shutil.copyfile(os.path.join(work, "stdout.txt"), os.path.join(dst, "stdout.txt"))
        print(f"case {case}: rc {rc}, {dt:.1f} s, {len(kept)} dumps")


def timing(out):
    """Wall time of the reference's run_simulation (plain build, log level 0)
    per spot: the production beam (C2) and four spots of the 512-spot plan,
    each on its own 200 x 400 water domain at 0.5 mm, on the reference's own
    grids, until no cell holds weight (at most 1000 iterations)."""
    exe = os.path.join(EXE_DIR, "run_simulation")
    base = read_ini(os.path.join(HERE, "one_step_case_C", "case.ini"))
    spots = [("C2 150 MeV", 150.0, 3.8, 1.5), ("plan 70 MeV", 70.0, 4.1, 0.7), ("plan 118 MeV", 118.0, 5.2, 1.18),
             ("plan 160 MeV", 160.0, 3.3, 1.6), ("plan 230 MeV", 230.0, 4.6, 2.3)]
    res = []
    for name, E0, sx, sE in spots:
        cfg = json.loads(json.dumps(base))
        cfg["energy"].update(mean_MeV=str(E0), sigma_MeV=str(sE))
        cfg["spatial"].update(sigma_x_mm=str(sx))
        cfg["angular"].update(sigma_theta_rad="0.002")
        cfg["sampling"].update(n_samples="1000", random_seed="42")
        cfg["grid"].update(Nx="200", Nz="400", max_steps="1000")
        cfg["transport"] = {"E_fine_on_MeV": "10.0", "E_fine_off_MeV": "11.0", "max_iterations": "1000",
                            "log_level": "1"}
        work = tempfile.mkdtemp(prefix="ref_time_")
        dt, rc = run(exe, cfg, work)
        with open(os.path.join(work, "stdout.txt")) as fh:
            log = fh.read()
        res.append({"spot": name, "E0": E0, "sigma_x": sx, "wall_s": dt, "rc": rc, "log_tail": log[-1500:]})
        print(f"{name}: rc {rc}, {dt:.2f} s")
    with open(os.path.join(out, "timing.json"), "w") as fh:
        json.dump(res, fh, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--timing", action="store_true")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    golden(args.out)
    if args.timing:
        timing(args.out)


if __name__ == "__main__":
    main()
