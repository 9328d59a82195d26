"""ctypes front end of the CPU oracle (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module.  It builds ``oracle/_build/liborc{32,64}.so`` with the
Makefile next to it on first use and exposes the oracle as a small Python
class.  ``Oracle(..., fp64=True)`` is the FP64 oracle of the same method.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
_LIBS = {}
_LOCK = threading.Lock()
KB = 32
EMPTY = 0xFFFFFFFF


class OrcConfig(C.Structure):
    _fields_ = [
        ("Nx", C.c_int), ("Nz", C.c_int),
        ("dx", C.c_float), ("dz", C.c_float), ("x_min", C.c_float), ("z_min", C.c_float),
        ("nt_local", C.c_int), ("ne_local", C.c_int), ("nx_sub", C.c_int), ("nz_sub", C.c_int),
        ("E_fine_on", C.c_float), ("E_fine_off", C.c_float), ("weight_active_min", C.c_float),
        ("step_coarse", C.c_float), ("sigma_x_initial", C.c_float), ("E0", C.c_float),
        ("enable_straggling", C.c_int), ("enable_nuclear", C.c_int),
        ("seed_slot_mode", C.c_int), ("energy_split", C.c_int),
        ("grid_E_min", C.c_float), ("grid_E_max", C.c_float),
        ("prune_coarse", C.c_float), ("prune_fine", C.c_float),
        ("split_min_weight", C.c_float), ("stop_weight_fraction", C.c_float),
        ("claim_reserve_weight", C.c_float), ("slots_per_cell", C.c_int),
        ("floor_cutoff", C.c_int), ("seed_iteration_salt", C.c_int), ("expectation", C.c_int),
        ("surrogate_tables", C.c_int), ("precision_form", C.c_int),
    ]


class OrcAudit(C.Structure):
    _fields_ = [
        ("W_error", C.c_float), ("W_pass", C.c_int), ("E_error", C.c_float), ("E_pass", C.c_int),
        ("W_in_total", C.c_float), ("W_out_total", C.c_float), ("W_cutoff_total", C.c_float),
        ("W_nuclear_total", C.c_float), ("W_boundary_total", C.c_float),
        ("W_source_out_of_grid_total", C.c_float), ("W_source_slot_drop_total", C.c_float),
        ("W_transport_drop_total", C.c_float),
        ("E_in_total", C.c_double), ("E_out_total", C.c_double), ("E_dep_total", C.c_double),
        ("E_cutoff_total", C.c_double), ("E_nuclear_total", C.c_double),
        ("E_boundary_total", C.c_double), ("E_source_out_of_grid_total", C.c_double),
        ("E_source_slot_drop_total", C.c_double), ("E_transport_drop_total", C.c_double),
        ("processed_cells", C.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def build():
    """Compile the oracle libraries (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _lib(fp64: bool):
    key = 64 if fp64 else 32
    with _LOCK:
        if key in _LIBS:
            return _LIBS[key]
        path = os.path.join(BUILD, f"liborc{key}.so")
        srcs = [os.path.join(HERE, "sm2d_oracle.c"), os.path.join(HERE, "sm2d_oracle.h"),
                os.path.join(HERE, "..", "sm_2d_gb300", "csrc", "sm2d_math.h"),
                os.path.join(HERE, "..", "sm_2d_gb300", "csrc", "sm2d_redist.h")]
        if not os.path.exists(path) or os.path.getmtime(path) < max(os.path.getmtime(f) for f in srcs):
            build()
        lib = C.CDLL(path)
        P = C.c_void_p
        lib.orc_create.restype = P
        lib.orc_create.argtypes = [C.POINTER(OrcConfig), C.c_int, P, C.c_int, P]
        lib.orc_destroy.argtypes = [P]
        lib.orc_local_bins.argtypes = [P]
        lib.orc_slots_per_cell.argtypes = [P]
        lib.orc_inject.argtypes = [P] + [C.c_float] * 8 + [C.c_int, C.c_uint]
        lib.orc_inject_quadrature.argtypes = [P] + [C.c_float] * 7
        lib.orc_get_drop_channels.argtypes = [P, P, P]
        lib.orc_set_psi_in.argtypes = [P, P, P]
        lib.orc_get_psi_in.argtypes = [P, P, P]
        lib.orc_step.argtypes = [P]
        lib.orc_run.argtypes = [P, C.c_int]
        lib.orc_get_mask.argtypes = [P, P]
        lib.orc_get_lists.argtypes = [P, P, C.POINTER(C.c_int), P, C.POINTER(C.c_int)]
        lib.orc_get_tallies.argtypes = [P] * 8
        lib.orc_get_audit.argtypes = [P, C.POINTER(OrcAudit)]
        lib.orc_get_scalars.argtypes = [P, P]
        lib.orc_get_fe.argtypes = [P, P, P, P]
        lib.orc_run_many.argtypes = [P, C.c_int, C.c_int, C.c_int]
        lib.orc_energy_grid_log.argtypes = [C.c_float, C.c_float, C.c_int, P, P]
        lib.orc_energy_grid_piecewise.argtypes = [C.c_int, P, P, P]
        lib.orc_angular_grid.argtypes = [C.c_float, C.c_float, C.c_int, P, P]
        lib.orc_generate_rlut.argtypes = [C.c_int] + [P] * 6
        lib.orc_fe_precompute.argtypes = [C.c_float, C.c_int, C.c_float, C.c_float, P, P, P]
        lib.orc_fe_precompute_density.argtypes = [C.c_float, C.c_int, C.c_float, C.c_float, P, P, P, P]
        lib.orc_set_density.argtypes = [P, P]
        lib.orc_postprocess.argtypes = [P, P, C.c_float, C.c_int, C.c_int, C.c_float, P]
        lib.orc_math.argtypes = [C.c_int, P, P, C.c_int]
        lib.orc_redistribution_table.argtypes = [P, C.c_int, P, P]
        lib.orc_track_claims.argtypes = [P, C.c_int]
        lib.orc_redist_masses.argtypes = [C.c_double, C.c_double, C.c_double, P, C.c_int, P, P]
        lib.orc_claim_demand.argtypes = [P]
        lib.orc_k4_raw.argtypes = [P, C.c_int, P, P, P, P, P, P]
        lib.orc_set_surrogate.argtypes = [P, P, P, C.c_float]
        lib.orc_surrogate_counts.argtypes = [P, P]
        _LIBS[key] = lib
        return lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ---- grids and tables -------------------------------------------------------
def energy_grid_log(E_min, E_max, N):
    lib = _lib(False)
    e = np.zeros(N + 1, np.float32)
    r = np.zeros(N, np.float32)
    lib.orc_energy_grid_log(E_min, E_max, N, _p(e), _p(r))
    return e, r


def energy_grid_piecewise(groups):
    lib = _lib(False)
    g = np.asarray(groups, np.float32).reshape(-1)
    n = lib.orc_energy_grid_piecewise(len(groups), _p(g), None, None)
    e = np.zeros(n + 1, np.float32)
    r = np.zeros(n, np.float32)
    lib.orc_energy_grid_piecewise(len(groups), _p(g), _p(e), _p(r))
    return e, r


def angular_grid(th_min, th_max, N):
    lib = _lib(False)
    e = np.zeros(N + 1, np.float32)
    r = np.zeros(N, np.float32)
    lib.orc_angular_grid(th_min, th_max, N, _p(e), _p(r))
    return e, r


def generate_rlut(rep):
    lib = _lib(False)
    rep = np.ascontiguousarray(rep, np.float32)
    n = rep.size
    out = [np.zeros(n, np.float32) for _ in range(5)]
    lib.orc_generate_rlut(n, _p(rep), *[_p(a) for a in out])
    return dict(zip(["R", "S", "logE", "logR", "logS"], out))


def fe_precompute(E0, Nz, dz, sigma_x0, rho=None):
    """Fermi-Eyges A, B, sigma_total; through a density per depth row when rho is given."""
    lib = _lib(False)
    A, B, S = (np.zeros(Nz, np.float32) for _ in range(3))
    if rho is None:
        lib.orc_fe_precompute(E0, Nz, dz, sigma_x0, _p(A), _p(B), _p(S))
    else:
        r = np.ascontiguousarray(rho, np.float32)
        lib.orc_fe_precompute_density(E0, Nz, dz, sigma_x0, _p(r), _p(A), _p(B), _p(S))
    return A, B, S


def postprocess(edep, sigma_total, sigma_x0, Nx, Nz, dx):
    lib = _lib(False)
    edep = np.ascontiguousarray(edep, np.float64).reshape(-1)
    st = np.ascontiguousarray(sigma_total, np.float32)
    out = np.zeros_like(edep)
    lib.orc_postprocess(_p(edep), _p(st), sigma_x0, Nx, Nz, dx, _p(out))
    return out.reshape(Nz, Nx)


# ---- transport ---------------------------------------------------------------
class Oracle:
    """One transport problem on the CPU oracle."""

    def __init__(self, cfg: dict, theta_edges, E_edges, fp64: bool = False):
        self.lib = _lib(fp64)
        self.fp64 = fp64
        self.dtype = np.float64 if fp64 else np.float32
        c = OrcConfig()
        defaults = dict(x_min=0.0, z_min=0.0, E_fine_on=10.0, E_fine_off=11.0,
                        weight_active_min=1e-12, step_coarse=5.0, sigma_x_initial=0.0, E0=0.0,
                        enable_straggling=1, enable_nuclear=1, seed_slot_mode=0, energy_split=0,
                        grid_E_min=0.0, grid_E_max=0.0, prune_coarse=0.0, prune_fine=0.0, split_min_weight=0.0, stop_weight_fraction=0.0, claim_reserve_weight=0.0, slots_per_cell=32, floor_cutoff=0, seed_iteration_salt=0, expectation=0,
                        surrogate_tables=0, precision_form=0)
        defaults.update(cfg)
        for name, _ in OrcConfig._fields_:
            setattr(c, name, defaults[name])
        self.cfg = defaults
        self.theta_edges = np.ascontiguousarray(theta_edges, np.float32)
        self.E_edges = np.ascontiguousarray(E_edges, np.float32)
        self.N_theta = self.theta_edges.size - 1
        self.N_E = self.E_edges.size - 1
        self.ctx = self.lib.orc_create(C.byref(c), self.N_theta, _p(self.theta_edges),
                                       self.N_E, _p(self.E_edges))
        self.Nx, self.Nz = c.Nx, c.Nz
        self.Nc = c.Nx * c.Nz
        self.L = self.lib.orc_local_bins(self.ctx)
        self.Kb = self.lib.orc_slots_per_cell(self.ctx)

    def close(self):
        if self.ctx:
            self.lib.orc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def inject(self, x0, z0, theta0, E0, W, sigma_x=0.0, sigma_theta=0.0, sigma_E=0.0,
               n_samples=1, seed=42):
        self.lib.orc_inject(self.ctx, x0, z0, theta0, E0, W, sigma_x, sigma_theta, sigma_E,
                            int(n_samples), int(seed) & 0xFFFFFFFF)

    def inject_quadrature(self, x0, z0, theta0, sigma_theta, E0, W, sigma_x):
        """inject_source_kernel with its spreads (the quadrature source)."""
        self.lib.orc_inject_quadrature(self.ctx, x0, z0, theta0, sigma_theta, E0, W, sigma_x)

    def set_density(self, rho):
        """Slab phantom: density per depth row (None: water)."""
        if rho is None:
            self.lib.orc_set_density(self.ctx, None)
            return
        self._rho = np.ascontiguousarray(rho, np.float32)
        assert self._rho.size == self.Nz
        self.lib.orc_set_density(self.ctx, _p(self._rho))

    def set_psi_in(self, bid, val):
        bid = np.ascontiguousarray(bid, np.uint32)
        val = np.ascontiguousarray(val, self.dtype)
        assert bid.size == self.Nc * self.Kb and val.size == self.Nc * self.Kb * self.L
        self.lib.orc_set_psi_in(self.ctx, _p(bid), _p(val))

    def psi_in(self, values=True):
        bid = np.zeros(self.Nc * self.Kb, np.uint32)
        val = np.zeros(self.Nc * self.Kb * self.L, self.dtype) if values else None
        self.lib.orc_get_psi_in(self.ctx, _p(bid), _p(val) if values else None)
        return bid, val

    def step(self) -> int:
        return self.lib.orc_step(self.ctx)

    def run(self, max_iterations: int) -> int:
        return self.lib.orc_run(self.ctx, max_iterations)

    def mask(self):
        m = np.zeros(self.Nc, np.uint8)
        self.lib.orc_get_mask(self.ctx, _p(m))
        return m

    def lists(self):
        a = np.zeros(self.Nc, np.uint32)
        co = np.zeros(self.Nc, np.uint32)
        na, nc = C.c_int(), C.c_int()
        self.lib.orc_get_lists(self.ctx, _p(a), C.byref(na), _p(co), C.byref(nc))
        return a[: na.value].copy(), co[: nc.value].copy()

    def tallies(self):
        n = self.Nc
        out = dict(edep=np.zeros(n), w_cut=np.zeros(n, np.float32), e_cut=np.zeros(n),
                   w_nuc=np.zeros(n, np.float32), e_nuc=np.zeros(n),
                   w_bnd=np.zeros(n, np.float32), e_bnd=np.zeros(n))
        self.lib.orc_get_tallies(self.ctx, *[_p(out[k]) for k in
                                             ["edep", "w_cut", "e_cut", "w_nuc", "e_nuc", "w_bnd", "e_bnd"]])
        return out

    def audit(self):
        a = OrcAudit()
        self.lib.orc_get_audit(self.ctx, C.byref(a))
        return a.as_dict()

    def drop_channels(self):
        """{(stage, kind): (weight, energy)} of the drops since create, stage
        2/3/4 (K2, K3, K4), kind slot/bucket/pruned."""
        w, e = np.zeros(9), np.zeros(9)
        self.lib.orc_get_drop_channels(self.ctx, _p(w), _p(e))
        kinds = ("slot", "bucket", "pruned")
        return {(2 + i // 3, kinds[i % 3]): (float(w[i]), float(e[i])) for i in range(9)}

    def scalars(self):
        s = np.zeros(14)
        self.lib.orc_get_scalars(self.ctx, _p(s))
        keys = ["transport_dropped_weight", "transport_dropped_energy", "audit_residual_energy",
                "source_injected_weight", "source_injected_energy", "source_out_of_grid_weight",
                "source_out_of_grid_energy", "source_slot_dropped_weight", "source_slot_dropped_energy",
                "source_representation_loss_energy", "iterations", "cell_steps", "slots_in", "slots_out"]
        return dict(zip(keys, s.tolist()))

    def redistribution_table(self, feats):
        """The expectation form's 8 theta x 4 E redistribution of each feature
        row (s, u, r, cap) (redistribution_table below; the context is not used)."""
        f = np.ascontiguousarray(feats, np.float32).reshape(-1, 4)
        out = np.zeros((f.shape[0], 32), np.float32)
        self.lib.orc_redistribution_table(self.ctx, f.shape[0], _p(f), _p(out))
        return out

    def set_surrogate(self, params, region_err, tol):
        """The network of surrogate_tables = 2: fp32 parameters, per-region
        calibrated errors [4096], fallback tolerance."""
        self._net = (np.ascontiguousarray(params, np.float32), np.ascontiguousarray(region_err, np.float32))
        self.lib.orc_set_surrogate(self.ctx, _p(self._net[0]), _p(self._net[1]), float(tol))

    def surrogate_counts(self):
        """(rows the network was asked for, rows that fell back)"""
        o = np.zeros(2, np.int64)
        self.lib.orc_surrogate_counts(self.ctx, _p(o))
        return int(o[0]), int(o[1])

    def k4_raw(self, bkt_bid, bkt_val, c2b, out_bid, out_val):
        """K4 on caller arrays: buckets [nb][Kb] ids and [nb][Kb][L] values,
        c2b [Nc]; returns the updated psi_out ids and values and the dropped
        (weight, energy)."""
        bb = np.ascontiguousarray(bkt_bid, np.uint32)
        bv = np.ascontiguousarray(bkt_val, self.dtype)
        cb = np.ascontiguousarray(c2b, np.int32)
        ob = np.array(out_bid, np.uint32, copy=True)
        ov = np.array(out_val, self.dtype, copy=True)
        drop = np.zeros(2)
        self.lib.orc_k4_raw(self.ctx, bb.shape[0], _p(bb), _p(bv), _p(cb), _p(ob), _p(ov), _p(drop))
        return ob, ov, (float(drop[0]), float(drop[1]))

    def track_claims(self, on=True):
        """Record the distinct block ids aimed at each container per iteration."""
        self.lib.orc_track_claims(self.ctx, 1 if on else 0)

    def claim_demand(self):
        """Largest number of distinct block ids aimed at one container (psi_out
        cell or bucket) in one iteration while tracking was on."""
        return self.lib.orc_claim_demand(self.ctx)

    def fe(self):
        A, B, S = (np.zeros(self.Nz, np.float32) for _ in range(3))
        self.lib.orc_get_fe(self.ctx, _p(A), _p(B), _p(S))
        return A, B, S


def run_many(oracles, max_iterations, n_threads):
    """Transport several independent problems on n_threads host threads."""
    if not oracles:
        return 0
    lib = oracles[0].lib
    arr = (C.c_void_p * len(oracles))(*[o.ctx for o in oracles])
    return lib.orc_run_many(C.cast(arr, C.c_void_p), len(oracles), max_iterations, n_threads)


# ---- psi rows in the reference debug-dump format ----------------------------
def psi_rows(bid, val, L, thresh=1e-12, Kb=KB):
    """Non-zero rows (cell, slot, bid, lidx, weight) with weight > thresh, the
    filter of the reference raw phase-space dump (k1k6_pipeline.cu:252)."""
    v = val.reshape(-1, Kb, L)
    b = bid.reshape(-1, Kb)
    cells, slots, lidx = np.nonzero((v > thresh) & (b[:, :, None] != EMPTY))
    return dict(cell=cells, slot=slots, bid=b[cells, slots], lidx=lidx,
                weight=v[cells, slots, lidx])


def redistribution_table(feats, fp64=False):
    """The surrogate's targets: the expectation form's 8 theta x 4 E table of
    each feature row (s, u, r, cap), on centres of uniform spacing."""
    f = np.ascontiguousarray(feats, np.float32).reshape(-1, 4)
    out = np.zeros((f.shape[0], 32), np.float32)
    _lib(fp64).orc_redistribution_table(None, f.shape[0], _p(f), _p(out))
    return out


def redist_masses(s, Em, sE, cen, fp64=False):
    """The expectation form's masses (sm2d_redist.h): angular Mt[8] for
    s = sigma_theta / dtheta, energy Me[4] for E' ~ N(Em, sE^2) over the
    descending centres cen (1 to 4 of them)."""
    cen = np.ascontiguousarray(cen, np.float64)
    Mt, Me = np.zeros(8), np.zeros(4)
    _lib(fp64).orc_redist_masses(float(s), float(Em), float(sE), _p(cen), cen.size - 1, _p(Mt), _p(Me))
    return Mt, Me


MATH_FUNCS = ("exp", "log", "sin", "cos", "erf")


def math_eval(name: str, x) -> np.ndarray:
    """The transport's elementary function `name` (sm2d_math.h) as the float
    oracle evaluates it."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    _lib(False).orc_math(MATH_FUNCS.index(name), x.ctypes.data, y.ctypes.data, x.size)
    return y
