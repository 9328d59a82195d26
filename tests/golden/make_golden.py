"""Regenerate the golden fixtures in this directory from the SM_2D reference.

Two sources, both produced by the reference itself:

1. ``one_step_case_{A,B,C,D}/`` -- the reference GPU build's own debug dumps
   (SM2D_ENABLE_DEBUG_DUMPS=ON, commit aeef09b2) for one K1..K6 iteration of
   a 150 MeV beam on an 80x40 grid at 0.5 mm: the phase space after source
   injection (``debug_ps_raw_iter_00_initial.csv``), after K2/K3 + K4
   (``debug_ps_raw_iter_01_after_K4.csv``), and the channel totals.  The
   case INI files are stored beside them, as written (``case.ini``) and as
   JSON.
2. ``ref_host_tables.json`` -- grids, R-LUTs and host lookups printed by
   ``oracle/ref_probe`` linked against the reference's own host sources
   (``oracle/ref_build.sh``).
3. ``writers/<case>/`` -- the reference's own output writers and depth-dose
   metrics (``oracle/ref_writer_probe``, linked against run_simulation.cpp,
   deterministic_beam.cpp and bragg_peak.cpp) applied to seeded synthetic
   dose grids (``dose.bin``): dose_2d.txt and pdd.txt with and without
   normalisation, and the metrics.

Run from the repository root where the reference tree is mounted:
SM2D_REFERENCE=<reference root> python tests/golden/make_golden.py
"""
import configparser
import json
import os
import shutil
import subprocess
import sys

REF = os.environ.get("SM2D_REFERENCE", "")   # root of the reference tree (required)
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

FILES = ["debug_ps_raw_iter_00_initial.csv", "debug_ps_raw_iter_01_after_K4.csv",
         "debug_channels_totals_iter01.csv", "debug_cells_iter_01_after_K4.csv"]


def one_step_cases():
    for case in "ABCD":
        src = os.path.join(REF, "results", f"one_step_case_{case}")
        dst = os.path.join(HERE, f"one_step_case_{case}")
        os.makedirs(dst, exist_ok=True)
        for f in FILES:
            shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        ini = [f for f in os.listdir(src) if f.endswith(".ini")][0]
        shutil.copyfile(os.path.join(src, ini), os.path.join(dst, "case.ini"))   # the INI front end's input
        cp = configparser.ConfigParser()
        cp.read(os.path.join(src, ini))
        cfg = {s: dict(cp[s]) for s in cp.sections()}
        cfg["output"].pop("output_dir", None)
        with open(os.path.join(dst, "case.json"), "w") as fh:
            json.dump(cfg, fh, indent=1, sort_keys=True)


def host_tables():
    exe = subprocess.run(["sh", os.path.join(ROOT, "oracle", "ref_build.sh")], check=True,
                         capture_output=True, text=True).stdout.strip().splitlines()[-1]
    out = subprocess.run([exe], check=True, capture_output=True, text=True, cwd="/tmp").stdout
    data = json.loads(out)
    with open(os.path.join(HERE, "ref_host_tables.json"), "w") as fh:
        json.dump(data, fh)


def writer_cases():
    """Synthetic dose grids: a Bragg-like depth profile times a lateral
    Gaussian with seeded noise; the second case holds a NaN cell (the
    writers print such cells as 0)."""
    import numpy as np
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "ref_build.sh")], check=True, capture_output=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_writer_probe")
    rng = np.random.default_rng(7)
    for case, (Nx, Nz, dx, dz, nan) in {"smooth": (24, 50, 0.5, 0.5, False), "nan_cell": (30, 41, 1.0, 0.25, True)}.items():
        z = np.arange(Nz)[:, None]
        x = (np.arange(Nx)[None, :] + 0.5) * dx - Nx * dx / 2
        depth = 0.4 + 1.1 * np.exp(-((z - 0.7 * Nz) / (0.06 * Nz)) ** 2)
        depth[z[:, 0] > 0.78 * Nz] *= 0.02
        dose = depth * np.exp(-x ** 2 / (2 * (0.15 * Nx * dx) ** 2)) * (1 + 0.01 * rng.standard_normal((Nz, Nx)))
        if nan:
            dose[Nz // 3, Nx // 2] = np.nan
        dst = os.path.join(HERE, "writers", case)
        os.makedirs(dst, exist_ok=True)
        with open(os.path.join(dst, "dose.bin"), "wb") as fh:
            fh.write(np.array([Nx, Nz], np.int32).tobytes() + np.array([dx, dz], np.float32).tobytes())
            fh.write(np.ascontiguousarray(dose, np.float64).tobytes())
        out = subprocess.run([exe, os.path.join(dst, "dose.bin"), dst], check=True, capture_output=True, text=True)
        with open(os.path.join(dst, "metrics.json"), "w") as fh:
            json.dump(json.loads(out.stdout), fh, indent=1)


if __name__ == "__main__":
    if not REF:
        sys.exit("set SM2D_REFERENCE to the root of the reference tree")
    if not os.path.isdir(REF):
        sys.exit(f"reference tree not found at {REF}")
    one_step_cases()
    host_tables()
    writer_cases()
    print("golden fixtures written to", HERE)
