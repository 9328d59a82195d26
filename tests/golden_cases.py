"""Loaders for the reference golden fixtures in tests/golden/.

``load_case(X)`` returns the problem of results/one_step_case_X as the
reference runner builds it (gpu_transport_runner.cpp:55-172): angular grid
+-0.35 rad with N_theta bins, the default piecewise energy grid, grid origin
x_min = -Nx*dx/2, plus the dumped phase space before and after one iteration.
"""
from __future__ import annotations

import csv
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KB = 32
EMPTY = 0xFFFFFFFF
DEFAULT_GROUPS = [(0.1, 2.0, 0.1), (2.0, 20.0, 0.2), (20.0, 100.0, 0.25), (100.0, 250.0, 0.25)]
REF_LAYOUT = dict(nt_local=4, ne_local=2, nx_sub=8, nz_sub=4)   # local_bins.hpp:49-52


def host_tables():
    with open(os.path.join(GOLDEN, "ref_host_tables.json")) as fh:
        return json.load(fh)


def read_rows(path):
    with open(path) as fh:
        return list(csv.DictReader(fh))


def read_channels(path):
    out = {}
    for r in read_rows(path):
        out[(int(r["iter"]), r["channel"])] = float(r["value"])
    return out


def rows_to_dense(rows, Nc, L):
    bid = np.full(Nc * KB, EMPTY, np.uint32)
    val = np.zeros(Nc * KB * L, np.float32)
    for r in rows:
        cell, slot, lidx = int(r["cell"]), int(r["slot"]), int(r["lidx"])
        bid[cell * KB + slot] = int(r["bid"])
        val[(cell * KB + slot) * L + lidx] = float(r["weight"])
    return bid, val


def load_case(name: str):
    d = os.path.join(GOLDEN, f"one_step_case_{name}")
    with open(os.path.join(d, "case.json")) as fh:
        ini = json.load(fh)
    tables = host_tables()
    Nx, Nz = int(ini["grid"]["nx"]), int(ini["grid"]["nz"])
    dx, dz = float(ini["grid"]["dx_mm"]), float(ini["grid"]["dz_mm"])
    tr = ini.get("transport", {})
    N_theta = int(tr.get("n_theta", 36))
    theta_key = {36: "theta_0.35_36", 360: "theta_0.35_360"}[N_theta]
    theta_edges = np.asarray(tables[theta_key]["edges"], np.float32)
    E_edges = np.asarray(tables["piecewise_default"]["edges"], np.float32)
    L = 4 * 2 * 8 * 4
    cfg = dict(Nx=Nx, Nz=Nz, dx=dx, dz=dz, x_min=-(Nx * dx) / 2.0, z_min=0.0,
               E_fine_on=float(tr.get("e_fine_on_mev", 10.0)),
               E_fine_off=float(tr.get("e_fine_off_mev", 11.0)),
               weight_active_min=1e-12, step_coarse=5.0,
               sigma_x_initial=float(ini["spatial"]["sigma_x_mm"]),
               E0=float(ini["energy"]["mean_mev"]),
               enable_straggling=1, enable_nuclear=1, seed_slot_mode=0, energy_split=0,
               grid_E_min=0.1, grid_E_max=250.0, **REF_LAYOUT)
    beam = dict(x0=float(ini["spatial"]["x0_mm"]), z0=float(ini["spatial"]["z0_mm"]),
                theta0=float(ini["angular"]["theta0_rad"]), E0=float(ini["energy"]["mean_mev"]),
                W=float(ini["beam"]["weight"]), sigma_x=float(ini["spatial"]["sigma_x_mm"]),
                sigma_theta=float(ini["angular"]["sigma_theta_rad"]),
                sigma_E=float(ini["energy"]["sigma_mev"]),
                n_samples=int(ini["sampling"]["n_samples"]),
                seed=int(ini["sampling"]["random_seed"]))
    rows_in = read_rows(os.path.join(d, "debug_ps_raw_iter_00_initial.csv"))
    rows_out = read_rows(os.path.join(d, "debug_ps_raw_iter_01_after_K4.csv"))
    channels = read_channels(os.path.join(d, "debug_channels_totals_iter01.csv"))
    bid_in, val_in = rows_to_dense(rows_in, Nx * Nz, L)
    return dict(name=name, cfg=cfg, beam=beam, theta_edges=theta_edges, E_edges=E_edges, L=L,
                rows_in=rows_in, rows_out=rows_out, channels=channels,
                bid_in=bid_in, val_in=val_in)


def row_key_sets(rows):
    """{(cell, bid, lidx): weight} from dump rows or psi_rows output."""
    if isinstance(rows, dict):
        return {(int(c), int(b), int(l)): float(w) for c, b, l, w in
                zip(rows["cell"], rows["bid"], rows["lidx"], rows["weight"])}
    return {(int(r["cell"]), int(r["bid"]), int(r["lidx"])): float(r["weight"]) for r in rows}
