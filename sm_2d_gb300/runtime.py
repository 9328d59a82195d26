"""Host-side mirror of the reference transport interface over the C ABI.

``Transport`` corresponds to one call of the reference wrapper
``sm_2d::run_k1k6_pipeline_transport(x0, z0, theta0, E0, W, sigma_x,
sigma_theta, sigma_E, n_samples, seed, Nx, Nz, dx, dz, x_min, z_min, ...,
edep)`` (src/include/cuda/gpu_transport_wrapper.hpp:78-90) split into its
steps: allocate (sm2d_create), inject, iterate, read the dose.  Grids are
built by the library's own host tables (EnergyGrid / AngularGrid
semantics of src/core/grids.cpp).  Everything runs through libsm2d.so; there
is no Python or CPU fallback: a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

KB = 32
EMPTY = 0xFFFFFFFF
_LIB = None
_LOCK = threading.Lock()


class Sm2dError(RuntimeError):
    pass


class Problem(C.Structure):
    _fields_ = [
        ("Nx", C.c_int), ("Nz", C.c_int), ("dx", C.c_float), ("dz", C.c_float),
        ("x_min", C.c_float), ("z_min", C.c_float),
        ("N_theta", C.c_int), ("theta_edges", C.c_void_p),
        ("N_E", C.c_int), ("E_edges", C.c_void_p), ("E_min", C.c_float), ("E_max", C.c_float),
        ("nt_local", C.c_int), ("ne_local", C.c_int), ("nx_sub", C.c_int), ("nz_sub", C.c_int),
        ("E_fine_on", C.c_float), ("E_fine_off", C.c_float), ("weight_active_min", C.c_float),
        ("step_coarse", C.c_float), ("sigma_x_initial", C.c_float), ("E0", C.c_float),
        ("enable_straggling", C.c_int), ("enable_nuclear", C.c_int),
        ("seed_slot_mode", C.c_int), ("energy_split", C.c_int), ("use_buckets", C.c_int),
        ("max_iterations", C.c_int),
        ("prune_coarse", C.c_float), ("prune_fine", C.c_float), ("split_min_weight", C.c_float),
        ("stop_weight_fraction", C.c_float), ("floor_cutoff", C.c_int), ("seed_iteration_salt", C.c_int),
        ("lanes", C.c_int), ("density_z", C.c_void_p), ("expectation", C.c_int), ("precision_form", C.c_int),
        ("slot_pages_per_lane", C.c_int),
    ]


class Beam(C.Structure):
    _fields_ = [("x0", C.c_float), ("z0", C.c_float), ("theta0", C.c_float), ("E0", C.c_float),
                ("W_total", C.c_float), ("sigma_x", C.c_float), ("sigma_theta", C.c_float),
                ("sigma_E", C.c_float), ("n_samples", C.c_int), ("seed", C.c_uint)]


class RunConfig(C.Structure):
    """sm2d_run_config: one run as the reference's INI file describes it."""
    _fields_ = [("problem", Problem), ("beam", Beam), ("max_iterations", C.c_int), ("log_level", C.c_int),
                ("fail_fast_on_audit", C.c_int), ("normalize_dose", C.c_int), ("save_2d", C.c_int),
                ("save_pdd", C.c_int), ("output_dir", C.c_char * 1024), ("dose_2d_file", C.c_char * 256),
                ("pdd_file", C.c_char * 256), ("theta_edges_buf", C.c_void_p), ("E_edges_buf", C.c_void_p)]


class Audit(C.Structure):
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
        return {n: getattr(self, n) for n, _ in self._fields_}


class SpotResult(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("finished", C.c_int), ("weight_audit_failures", C.c_int),
        ("energy_audit_failures", C.c_int),
        ("injected_weight", C.c_double), ("injected_energy", C.c_double),
        ("source_out_of_grid_weight", C.c_double), ("source_slot_dropped_weight", C.c_double),
        ("transport_dropped_weight", C.c_double), ("transport_dropped_energy", C.c_double),
        ("audit_residual_energy", C.c_double), ("representation_loss_energy", C.c_double),
        ("cell_steps", C.c_double), ("slots_in", C.c_double), ("slots_out", C.c_double), ("last", Audit),
    ]

    def as_dict(self):
        out = {n: getattr(self, n) for n, _ in self._fields_ if n != "last"}
        out["last"] = self.last.as_dict()
        return out


SCALAR_KEYS = ["transport_dropped_weight", "transport_dropped_energy", "audit_residual_energy",
               "source_injected_weight", "source_injected_energy", "source_out_of_grid_weight",
               "source_out_of_grid_energy", "source_slot_dropped_weight", "source_slot_dropped_energy",
               "source_representation_loss_energy", "iterations", "cell_steps", "slots_in", "slots_out",
               "claim_table_overflows", "claim_misses", "bin_list_overflows"]
# device stages of one iteration, in launch order (sm2d_get_step_timing)
STAGES = ["classify", "lists", "claims", "select", "transport", "k4", "finalize"]


def lib(build_if_needed: bool = True):
    """Load libsm2d.so (building it in-tree when sources are newer)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if build_if_needed and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise Sm2dError(f"CUDA library {path} is missing; run sm_2d_gb300.build")
        L = C.CDLL(path)
        P, I, F, D = C.c_void_p, C.c_int, C.c_float, C.c_double
        L.sm2d_last_error.restype = C.c_char_p
        L.sm2d_bucket_bytes.restype = C.c_size_t
        L.sm2d_bucket_bytes.argtypes = [I]
        L.sm2d_create.argtypes = [C.POINTER(Problem), C.POINTER(P)]
        for n in ["sm2d_destroy", "sm2d_local_bins"]:
            getattr(L, n).argtypes = [P]
        L.sm2d_inject.argtypes = [P, C.POINTER(Beam)]
        L.sm2d_inject_quadrature.argtypes = [P, C.POINTER(Beam)]
        L.sm2d_get_debug_counters.argtypes = [P, C.c_int, P, P, P]
        L.sm2d_reset_debug_counters.argtypes = [P, C.c_int]
        L.sm2d_set_psi_in.argtypes = [P, P, P]
        L.sm2d_get_psi_in.argtypes = [P, P, P]
        L.sm2d_step.argtypes = [P, C.POINTER(I), C.POINTER(I)]
        L.sm2d_run.argtypes = [P, I, C.POINTER(I)]
        L.sm2d_run_timed.argtypes = [P, I, C.POINTER(I), C.POINTER(F)]
        L.sm2d_get_mask.argtypes = [P, P]
        L.sm2d_get_lists.argtypes = [P, P, C.POINTER(I), P, C.POINTER(I)]
        L.sm2d_get_tallies.argtypes = [P] * 8
        L.sm2d_get_audit.argtypes = [P, C.POINTER(Audit)]
        L.sm2d_get_audit_history.argtypes = [P, P, I, C.POINTER(I)]
        L.sm2d_get_scalars.argtypes = [P, P]
        L.sm2d_get_fe.argtypes = [P, P, P, P]
        L.sm2d_get_dose.argtypes = [P, P]
        L.sm2d_get_step_timing.argtypes = [P, P]
        L.sm2d_stream.restype = P
        L.sm2d_stream.argtypes = [P]
        L.sm2d_reset.argtypes = [P]
        L.sm2d_inject_async.argtypes = [P, C.POINTER(Beam)]
        L.sm2d_run_async.argtypes = [P, I]
        L.sm2d_dose_async.argtypes = [P, P]
        L.sm2d_run_profiled.argtypes = [P, I, C.POINTER(I), P, C.POINTER(I), C.POINTER(I)]
        L.sm2d_energy_grid_log.argtypes = [F, F, I, P, P]
        L.sm2d_energy_grid_piecewise.argtypes = [I, P, P, P]
        L.sm2d_angular_grid.argtypes = [F, F, I, P, P]
        L.sm2d_range_lut.argtypes = [I] + [P] * 6
        L.sm2d_fermi_eyges.argtypes = [F, I, F, F, P, P, P]
        L.sm2d_fermi_eyges_density.argtypes = [F, I, F, F, P, P, P, P]
        L.sm2d_k1_active_mask.argtypes = [P, P, P, P, I, I, I, I, I, F, P]
        L.sm2d_compact_lists.argtypes = [P, P, P, I, I, I, P, P, P, P, P]
        L.sm2d_k4_bucket_transfer.argtypes = [P, P, P, P, I, I, I, I, I, I, P, I, I, P, P]
        L.sm2d_k5_conservation_audit.argtypes = ([P] * 18 + [F, F, D, D, F, D, I, P, I, I, I, I, P, I, P])
        L.sm2d_k5_conservation_audit_static.argtypes = L.sm2d_k5_conservation_audit.argtypes
        L.sm2d_math_eval.argtypes = [I, P, P, I]
        L.sm2d_lanes.argtypes = [P]
        L.sm2d_batch_run.argtypes = [P, P, I, I, P, P]
        L.sm2d_batch_inject.argtypes = [P, P, I]
        L.sm2d_batch_results.argtypes = [P, P, I]
        L.sm2d_batch_dose.argtypes = [P, P, I]
        L.sm2d_batch_audit_history.argtypes = [P, I, P, I, C.POINTER(I)]
        L.sm2d_load_ini.argtypes = [C.c_char_p, C.POINTER(RunConfig)]
        L.sm2d_run_config_free.argtypes = [C.POINTER(RunConfig)]
        L.sm2d_run_config_free.restype = None
        L.sm2d_run_simulation.argtypes = [C.c_char_p]
        L.sm2d_write_ps_raw_csv.argtypes = [C.c_char_p, C.POINTER(Problem), P, P, I, I]
        L.sm2d_write_cells_csv.argtypes = [C.c_char_p, C.POINTER(Problem), P, P]
        L.sm2d_write_channel_totals_csv.argtypes = [C.c_char_p, P]
        L.sm2d_channel_totals.argtypes = [P, I, I, P]
        L.sm2d_depth_dose.argtypes = [P, I, I, P]
        L.sm2d_bragg_peak_row.argtypes = [P, I, I]
        L.sm2d_bragg_metrics.argtypes = [P, I, I, F, P]
        L.sm2d_write_dose_2d.argtypes = [C.c_char_p, P, I, I, F, F, I]
        L.sm2d_write_pdd.argtypes = [C.c_char_p, P, I, I, F, I]
        L.sm2d_plan_load.argtypes = [P, P, I, I, I]
        L.sm2d_plan_run_async.argtypes = [P]
        L.sm2d_plan_results.argtypes = [P, P, P]
        L.sm2d_plan_stats.argtypes = [P, C.POINTER(I), C.POINTER(I), C.POINTER(D)]
        L.sm2d_page_stats.argtypes = [P, C.POINTER(I), C.POINTER(I)]
        L.sm2d_set_lanes_in_flight.argtypes = [P, I]
        L.sm2d_get_lanes_in_flight.argtypes = [P, C.POINTER(I)]
        L.sm2d_tune_lanes_in_flight.argtypes = [P, C.POINTER(I), C.POINTER(F)]
        L.sm2d_set_surrogate.argtypes = [P, P, F, I, I]
        L.sm2d_get_launch_shape.argtypes = [P, P]
        L.sm2d_set_launch_shape.argtypes = [P, P]
        L.sm2d_autotune.argtypes = [P, P, P]
        L.sm2d_surrogate_stats.argtypes = [P, P]
        _LIB = L
        return L


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def check(rc: int):
    if rc != 0:
        raise Sm2dError(f"sm2d error {rc}: {lib().sm2d_last_error().decode()}")


# ---------------------------------------------------------------- grids
def energy_grid_log(E_min, E_max, N):
    e = np.zeros(N + 1, np.float32)
    r = np.zeros(N, np.float32)
    check(lib().sm2d_energy_grid_log(E_min, E_max, N, _p(e), _p(r)))
    return e, r


def energy_grid_piecewise(groups):
    g = np.asarray(groups, np.float32).reshape(-1)
    n = lib().sm2d_energy_grid_piecewise(len(groups), _p(g), None, None)
    if n < 0:
        check(n)
    e = np.zeros(n + 1, np.float32)
    r = np.zeros(n, np.float32)
    lib().sm2d_energy_grid_piecewise(len(groups), _p(g), _p(e), _p(r))
    return e, r


def angular_grid(lo, hi, N):
    e = np.zeros(N + 1, np.float32)
    r = np.zeros(N, np.float32)
    check(lib().sm2d_angular_grid(lo, hi, N, _p(e), _p(r)))
    return e, r


def range_lut(rep):
    rep = np.ascontiguousarray(rep, np.float32)
    out = [np.zeros(rep.size, np.float32) for _ in range(5)]
    check(lib().sm2d_range_lut(rep.size, _p(rep), *[_p(a) for a in out]))
    return dict(zip(["R", "S", "logE", "logR", "logS"], out))


def fermi_eyges(E0, Nz, dz, sigma_x0, density_z=None):
    """Fermi-Eyges A, B, sigma_total along depth; through a slab phantom when
    density_z (g/cm^3 per depth row) is given."""
    A, B, S = (np.zeros(Nz, np.float32) for _ in range(3))
    if density_z is None:
        check(lib().sm2d_fermi_eyges(E0, Nz, dz, sigma_x0, _p(A), _p(B), _p(S)))
    else:
        r = np.ascontiguousarray(density_z, np.float32)
        check(lib().sm2d_fermi_eyges_density(E0, Nz, dz, sigma_x0, _p(r), _p(A), _p(B), _p(S)))
    return A, B, S


DEFAULT_ENERGY_GROUPS = [(0.1, 2.0, 0.1), (2.0, 20.0, 0.2), (20.0, 100.0, 0.25), (100.0, 250.0, 0.25)]
LAYOUT_REF = dict(nt_local=4, ne_local=2, nx_sub=8, nz_sub=4)      # 256 local bins
LAYOUT_B128 = dict(nt_local=8, ne_local=4, nx_sub=4, nz_sub=1)     # 128 local bins


@dataclass
class Config:
    """Spatial grid, phase-space grids and transport controls of one problem."""
    Nx: int
    Nz: int
    dx: float
    dz: float
    theta_edges: np.ndarray
    E_edges: np.ndarray
    E_min: float
    E_max: float
    x_min: float = 0.0
    z_min: float = 0.0
    layout: dict = field(default_factory=lambda: dict(LAYOUT_REF))
    E_fine_on: float = 10.0
    E_fine_off: float = 11.0
    weight_active_min: float = 1e-12
    step_coarse: float = 5.0
    sigma_x_initial: float = 0.0
    E0: float = 0.0
    enable_straggling: int = 1
    enable_nuclear: int = 1
    seed_slot_mode: int = 0
    energy_split: int = 0
    use_buckets: int = 0
    max_iterations: int = 4096
    prune_coarse: float = 0.0
    prune_fine: float = 0.0
    split_min_weight: float = 0.0
    stop_weight_fraction: float = 0.0
    floor_cutoff: int = 0
    seed_iteration_salt: int = 0
    lanes: int = 1          # spots transported together by Transport.batch_run
    density_z: np.ndarray = None   # slab phantom: density per depth row (None: water)
    expectation: int = 0    # 1: expectation form (redistribution weights instead of MCS/straggling draws)
    precision_form: int = 0  # 1: audit books weight increments; R-LUT inverted in double below 10 MeV
    slot_pages_per_lane: int = 0  # value pages per lane of a batch engine (0: 2^23 / local bins)

    def production(self):
        """Options of a production run: deterministic rank-ordered seeds salted
        per iteration, floor cutoff, and the stop at 1e-6 of the injected weight
        (the reference instead relies on max_iterations)."""
        self.seed_slot_mode = 1
        self.seed_iteration_salt = 1
        self.floor_cutoff = 1
        self.stop_weight_fraction = 1e-6
        if self.energy_split:
            self.split_min_weight = 1e-7
        return self

    def _problem(self):
        """The sm2d_problem of this config and the edge arrays it points into
        (keep them alive while the struct is used)."""
        th = np.ascontiguousarray(self.theta_edges, np.float32)
        E = np.ascontiguousarray(self.E_edges, np.float32)
        rho = None if self.density_z is None else np.ascontiguousarray(self.density_z, np.float32)
        if rho is not None and rho.size != self.Nz:
            raise ValueError("density_z needs one value per depth row")
        p = Problem(Nx=self.Nx, Nz=self.Nz, dx=self.dx, dz=self.dz, x_min=self.x_min, z_min=self.z_min,
                    N_theta=th.size - 1, theta_edges=th.ctypes.data, N_E=E.size - 1, E_edges=E.ctypes.data,
                    E_min=self.E_min, E_max=self.E_max, E_fine_on=self.E_fine_on, E_fine_off=self.E_fine_off,
                    weight_active_min=self.weight_active_min, step_coarse=self.step_coarse,
                    sigma_x_initial=self.sigma_x_initial, E0=self.E0,
                    enable_straggling=self.enable_straggling, enable_nuclear=self.enable_nuclear,
                    seed_slot_mode=self.seed_slot_mode, energy_split=self.energy_split,
                    use_buckets=self.use_buckets, max_iterations=self.max_iterations,
                    prune_coarse=self.prune_coarse, prune_fine=self.prune_fine,
                    split_min_weight=self.split_min_weight, stop_weight_fraction=self.stop_weight_fraction,
                    floor_cutoff=self.floor_cutoff, seed_iteration_salt=self.seed_iteration_salt, lanes=self.lanes,
                    density_z=None if rho is None else rho.ctypes.data, expectation=self.expectation,
                    precision_form=self.precision_form, slot_pages_per_lane=self.slot_pages_per_lane,
                    **self.layout)
        return p, (th, E, rho)

    def oracle_config(self):
        """The same problem as a CPU-oracle configuration dict."""
        return dict(Nx=self.Nx, Nz=self.Nz, dx=self.dx, dz=self.dz, x_min=self.x_min, z_min=self.z_min,
                    E_fine_on=self.E_fine_on, E_fine_off=self.E_fine_off,
                    weight_active_min=self.weight_active_min, step_coarse=self.step_coarse,
                    sigma_x_initial=self.sigma_x_initial, E0=self.E0,
                    enable_straggling=self.enable_straggling, enable_nuclear=self.enable_nuclear,
                    seed_slot_mode=self.seed_slot_mode, energy_split=self.energy_split,
                    grid_E_min=self.E_min, grid_E_max=self.E_max, prune_coarse=self.prune_coarse,
                    prune_fine=self.prune_fine, split_min_weight=self.split_min_weight,
                    stop_weight_fraction=self.stop_weight_fraction, floor_cutoff=self.floor_cutoff,
                    seed_iteration_salt=self.seed_iteration_salt, expectation=self.expectation,
                    precision_form=self.precision_form, **self.layout)

    @staticmethod
    def reference_runner(Nx, Nz, dx, dz, N_theta=36, E_fine_on=10.0, E_fine_off=11.0, **kw):
        """The grids GPUTransportRunner::run builds (gpu_transport_runner.cpp:85-98, 172):
        theta on +-0.35 rad, the default piecewise energy grid, x_min = -Nx*dx/2."""
        th, _ = angular_grid(-0.35, 0.35, N_theta)
        e, _ = energy_grid_piecewise(DEFAULT_ENERGY_GROUPS)
        return Config(Nx=Nx, Nz=Nz, dx=dx, dz=dz, theta_edges=th, E_edges=e, E_min=0.1, E_max=250.0,
                      x_min=-(Nx * dx) / 2.0, z_min=0.0, E_fine_on=E_fine_on, E_fine_off=E_fine_off, **kw)

    @staticmethod
    def log_grid(Nx, Nz, dx, dz, N_E=256, E_min=0.1, E_max=250.0, N_theta=512, theta_max=np.pi / 2,
                 layout=None, **kw):
        """Log-spaced energy grid and a uniform +-theta_max angular grid (EnergyGrid(E_min,E_max,N))."""
        th, _ = angular_grid(-theta_max, theta_max, N_theta)
        e, _ = energy_grid_log(E_min, E_max, N_E)
        return Config(Nx=Nx, Nz=Nz, dx=dx, dz=dz, theta_edges=th, E_edges=e, E_min=E_min, E_max=E_max,
                      x_min=-(Nx * dx) / 2.0, layout=dict(layout or LAYOUT_B128), **kw)


class Transport:
    """One transport problem resident on the GPU (handle over the C ABI)."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        p, (self._th, self._E, self._rho) = cfg._problem()
        h = C.c_void_p()
        self._lib = lib()
        check(self._lib.sm2d_create(C.byref(p), C.byref(h)))
        self.h = h
        self.Nc = cfg.Nx * cfg.Nz
        self.L = self._lib.sm2d_local_bins(h)
        self.lanes = self._lib.sm2d_lanes(h)

    def close(self):
        if getattr(self, "h", None):
            self._lib.sm2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- launch shape
    def launch_shape(self):
        """blocks per SM: warp-per-cell kernels, finalize, claim pass, deposit pass (0: all resident)"""
        o = np.zeros(4, np.int32)
        check(self._lib.sm2d_get_launch_shape(self.h, _p(o)))
        return o.tolist()

    def set_launch_shape(self, shape):
        check(self._lib.sm2d_set_launch_shape(self.h, _p(np.ascontiguousarray(shape, np.int32))))

    def autotune(self):
        """Tune the lanes in flight, then the launch shape, on the loaded plan;
        returns (shape, plan ms)."""
        o = np.zeros(4, np.int32)
        ms = C.c_float()
        check(self._lib.sm2d_autotune(self.h, _p(o), C.byref(ms)))
        return o.tolist(), ms.value

    def lanes_in_flight(self):
        n = C.c_int()
        check(self._lib.sm2d_get_lanes_in_flight(self.h, C.byref(n)))
        return n.value

    def set_lanes_in_flight(self, n):
        """A plan fills lanes 0..n-1 only (0: every lane); speed, not results."""
        check(self._lib.sm2d_set_lanes_in_flight(self.h, int(n)))

    def tune_lanes_in_flight(self):
        """Time every lane, 3/4, 1/2, 1/4, 1/8 and 1/16 of them (at least 8) on
        the loaded plan and keep the fastest; returns (lanes, plan ms)."""
        n, ms = C.c_int(), C.c_float()
        check(self._lib.sm2d_tune_lanes_in_flight(self.h, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    # -- learned surrogate in the fine step (expectation form)
    def set_surrogate(self, surrogate, tol=0.005, max_rows=0, method_tables=False):
        """K3 bins inside the network's domain take their redistribution
        weights from `surrogate` (a calibrated surrogate.Surrogate), with the
        closed forms where the calibrated error exceeds tol; method_tables:
        the plain table of each row instead of the network's; None detaches."""
        m = surrogate.m if surrogate is not None else None
        check(self._lib.sm2d_set_surrogate(self.h, m, float(tol), int(max_rows), 1 if method_tables else 0))
        self._surrogate = surrogate   # the network must outlive its use here

    def surrogate_stats(self):
        """rows served, rows that fell back, K3 bins beyond the row capacity (since the last reset)"""
        o = np.zeros(3)
        check(self._lib.sm2d_surrogate_stats(self.h, _p(o)))
        return dict(rows=int(o[0]), fallback_rows=int(o[1]), overflow_bins=int(o[2]))

    # -- source and phase space
    def inject(self, x0=0.0, z0=0.0, theta0=0.0, E0=150.0, W=1.0, sigma_x=0.0, sigma_theta=0.0,
               sigma_E=0.0, n_samples=1, seed=42):
        b = Beam(x0, z0, theta0, E0, W, sigma_x, sigma_theta, sigma_E, int(n_samples), int(seed) & 0xFFFFFFFF)
        check(self._lib.sm2d_inject(self.h, C.byref(b)))

    def inject_quadrature(self, x0=0.0, z0=0.0, theta0=0.0, sigma_theta=0.0, E0=150.0, W=1.0, sigma_x=0.0):
        """inject_source_kernel called with its spreads (k1k6_pipeline.cu:300-427):
        Gaussian cell weights over +-4 sigma_x, 7 angle nodes when
        sigma_theta > 1e-4; the pencil without spreads."""
        b = Beam(x0, z0, theta0, E0, W, sigma_x, sigma_theta, 0.0, 0, 0)
        check(self._lib.sm2d_inject_quadrature(self.h, C.byref(b)))

    def set_psi_in(self, bid, val):
        bid = np.ascontiguousarray(bid, np.uint32)
        val = np.ascontiguousarray(val, np.float32)
        if bid.size != self.Nc * KB or val.size != self.Nc * KB * self.L:
            raise ValueError("phase-space arrays have the wrong size")
        check(self._lib.sm2d_set_psi_in(self.h, _p(bid), _p(val)))

    def psi_in(self, values=True):
        bid = np.zeros(self.Nc * KB, np.uint32)
        val = np.zeros(self.Nc * KB * self.L, np.float32) if values else None
        check(self._lib.sm2d_get_psi_in(self.h, _p(bid), _p(val) if values else None))
        return bid, val

    # -- iteration
    def step(self):
        na, nc = C.c_int(), C.c_int()
        check(self._lib.sm2d_step(self.h, C.byref(na), C.byref(nc)))
        return na.value, nc.value

    def run(self, max_iterations=100000):
        n = C.c_int()
        check(self._lib.sm2d_run(self.h, int(max_iterations), C.byref(n)))
        return n.value

    def run_timed(self, max_iterations=100000):
        n, ms = C.c_int(), C.c_float()
        check(self._lib.sm2d_run_timed(self.h, int(max_iterations), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    # -- results
    def mask(self):
        m = np.zeros(self.Nc, np.uint8)
        check(self._lib.sm2d_get_mask(self.h, _p(m)))
        return m

    def lists(self):
        a = np.zeros(self.Nc, np.uint32)
        c = np.zeros(self.Nc, np.uint32)
        na, nc = C.c_int(), C.c_int()
        check(self._lib.sm2d_get_lists(self.h, _p(a), C.byref(na), _p(c), C.byref(nc)))
        return a[: na.value].copy(), c[: nc.value].copy()

    def tallies(self):
        n = self.Nc
        out = dict(edep=np.zeros(n), w_cut=np.zeros(n, np.float32), e_cut=np.zeros(n),
                   w_nuc=np.zeros(n, np.float32), e_nuc=np.zeros(n),
                   w_bnd=np.zeros(n, np.float32), e_bnd=np.zeros(n))
        check(self._lib.sm2d_get_tallies(self.h, *[_p(out[k]) for k in
                                                   ["edep", "w_cut", "e_cut", "w_nuc", "e_nuc", "w_bnd", "e_bnd"]]))
        return out

    def audit(self):
        a = Audit()
        check(self._lib.sm2d_get_audit(self.h, C.byref(a)))
        return a.as_dict()

    def audit_history(self, n_max=100000):
        arr = (Audit * n_max)()
        n = C.c_int()
        check(self._lib.sm2d_get_audit_history(self.h, C.cast(arr, C.c_void_p), n_max, C.byref(n)))
        return [arr[i].as_dict() for i in range(n.value)]

    def channel_totals(self):
        """The 17 channel totals of debug_channels_totals_iter01.csv
        (sm2d_channel_totals; CHANNELS order)."""
        out = np.zeros(17)
        check(self._lib.sm2d_channel_totals(self.h, self.cfg.Nx, self.cfg.Nz, _p(out)))
        return out

    def scalars(self):
        s = np.zeros(len(SCALAR_KEYS))
        check(self._lib.sm2d_get_scalars(self.h, _p(s)))
        return dict(zip(SCALAR_KEYS, s.tolist()))

    def debug_counters(self, stage):
        """k{stage}_get_debug_counters for stage 2 (K2), 3 (K3) or 4 (K4):
        {kind: (count, weight, energy)} for the output-slot, bucket and
        prune drops since the last reset."""
        n = np.zeros(3, np.uint64)
        w, e = np.zeros(3), np.zeros(3)
        check(self._lib.sm2d_get_debug_counters(self.h, int(stage), _p(n), _p(w), _p(e)))
        return {k: (int(n[i]), float(w[i]), float(e[i])) for i, k in enumerate(("slot", "bucket", "pruned"))}

    def reset_debug_counters(self, stage):
        check(self._lib.sm2d_reset_debug_counters(self.h, int(stage)))

    def fe(self):
        A, B, S = (np.zeros(self.cfg.Nz, np.float32) for _ in range(3))
        check(self._lib.sm2d_get_fe(self.h, _p(A), _p(B), _p(S)))
        return A, B, S

    def dose(self):
        """EdepC after the lateral MCS post-convolution, shape [Nz, Nx]."""
        d = np.zeros(self.Nc)
        check(self._lib.sm2d_get_dose(self.h, _p(d)))
        return d.reshape(self.cfg.Nz, self.cfg.Nx)

    # -- asynchronous spot pipeline
    def reset(self):
        check(self._lib.sm2d_reset(self.h))

    def inject_async(self, beam: "Beam"):
        check(self._lib.sm2d_inject_async(self.h, C.byref(beam)))

    def run_async(self, max_iterations=100000):
        check(self._lib.sm2d_run_async(self.h, int(max_iterations)))

    def dose_async(self, host_out: np.ndarray):
        check(self._lib.sm2d_dose_async(self.h, _p(host_out)))

    def stream(self):
        return self._lib.sm2d_stream(self.h)

    def batch_run(self, beams, max_iterations=100000, dose=True, results=True):
        """Transport a plan (list of Beam structures), `lanes` spots in flight,
        finished lanes refilled on the device.  Returns (dose [n, Nz, Nx] or
        None, list of result dicts or None)."""
        n = len(beams)
        arr = (Beam * max(n, 1))(*beams)
        d = np.zeros((n, self.cfg.Nz, self.cfg.Nx)) if dose else None
        r = (SpotResult * max(n, 1))() if results else None
        check(self._lib.sm2d_batch_run(self.h, C.cast(arr, C.c_void_p), n, int(max_iterations),
                                       _p(d) if dose else None, C.cast(r, C.c_void_p) if results else None))
        return d, ([r[i].as_dict() for i in range(n)] if results else None)

    def plan_load(self, beams, max_iterations=100000, dose=True):
        """Stage a plan on the device (sm2d_plan_load)."""
        arr = (Beam * max(len(beams), 1))(*beams)
        check(self._lib.sm2d_plan_load(self.h, C.cast(arr, C.c_void_p), len(beams), int(max_iterations),
                                       1 if dose else 0))
        self._plan_n = len(beams)

    def plan_run_async(self):
        check(self._lib.sm2d_plan_run_async(self.h))

    def plan_results(self, dose=True, results=True):
        n = getattr(self, "_plan_n", 0)
        d = np.zeros((n, self.cfg.Nz, self.cfg.Nx)) if dose else None
        r = (SpotResult * max(n, 1))() if results else None
        check(self._lib.sm2d_plan_results(self.h, _p(d) if dose else None, C.cast(r, C.c_void_p) if results else None))
        return d, ([r[i].as_dict() for i in range(n)] if results else None)

    def plan_stats(self):
        """(device passes, refill rounds, transported bins) of the last plan."""
        p, r, b = C.c_int(), C.c_int(), C.c_double()
        check(self._lib.sm2d_plan_stats(self.h, C.byref(p), C.byref(r), C.byref(b)))
        return p.value, r.value, b.value

    def page_stats(self):
        """(value pages per lane, the most pages one lane held) since the last
        plan's start or reset."""
        n, pk = C.c_int(), C.c_int()
        check(self._lib.sm2d_page_stats(self.h, C.byref(n), C.byref(pk)))
        return n.value, pk.value

    def batch_inject(self, beams):
        """Reset every lane and inject beams[i] into lane i (asynchronous)."""
        arr = (Beam * max(len(beams), 1))(*beams)
        check(self._lib.sm2d_batch_inject(self.h, C.cast(arr, C.c_void_p), len(beams)))

    def batch_results(self, n):
        r = (SpotResult * max(n, 1))()
        check(self._lib.sm2d_batch_results(self.h, C.cast(r, C.c_void_p), n))
        return [r[i].as_dict() for i in range(n)]

    def batch_audit_history(self, lane, n_max=100000):
        arr = (Audit * n_max)()
        n = C.c_int()
        check(self._lib.sm2d_batch_audit_history(self.h, int(lane), C.cast(arr, C.c_void_p), n_max, C.byref(n)))
        return [arr[i].as_dict() for i in range(n.value)]

    def batch_dose(self, n):
        d = np.zeros((n, self.cfg.Nz, self.cfg.Nx))
        check(self._lib.sm2d_batch_dose(self.h, _p(d), n))
        return d

    def run_profiled(self, n_iterations):
        """Eager replay with CUDA events around every kernel: (lane 0's
        iterations, {stage: summed ms}, kernel launches, passes timed)."""
        n, launches, passes = C.c_int(), C.c_int(), C.c_int()
        ms = np.zeros(len(STAGES), np.float32)
        check(self._lib.sm2d_run_profiled(self.h, int(n_iterations), C.byref(n), _p(ms), C.byref(launches),
                                          C.byref(passes)))
        return n.value, dict(zip(STAGES, ms.tolist())), launches.value, passes.value

    def step_timing(self):
        t = np.zeros(len(STAGES), np.float32)
        check(self._lib.sm2d_get_step_timing(self.h, _p(t)))
        return dict(zip(STAGES, t.tolist()))


MATH_FUNCS = ("exp", "log", "sin", "cos", "erf")


def math_eval(name: str, x) -> np.ndarray:
    """The transport's elementary function `name` evaluated on the device."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    check(lib().sm2d_math_eval(MATH_FUNCS.index(name), _p(x), _p(y), x.size))
    return y


def load_ini(path: str) -> tuple:
    """The reference's INI file as (Config, Beam, dict of run settings)
    (sm2d_load_ini: config_loader.hpp:324-411 and the runner's mapping)."""
    rc = RunConfig()
    check(lib().sm2d_load_ini(os.fsencode(path), C.byref(rc)))
    try:
        p = rc.problem
        th = np.ctypeslib.as_array(C.cast(p.theta_edges, C.POINTER(C.c_float)), (p.N_theta + 1,)).copy()
        ee = np.ctypeslib.as_array(C.cast(p.E_edges, C.POINTER(C.c_float)), (p.N_E + 1,)).copy()
        layout = dict(nt_local=p.nt_local, ne_local=p.ne_local, nx_sub=p.nx_sub, nz_sub=p.nz_sub)
        cfg = Config(Nx=p.Nx, Nz=p.Nz, dx=p.dx, dz=p.dz, theta_edges=th, E_edges=ee, E_min=p.E_min, E_max=p.E_max,
                     x_min=p.x_min, z_min=p.z_min, layout=layout, E_fine_on=p.E_fine_on, E_fine_off=p.E_fine_off,
                     weight_active_min=p.weight_active_min, step_coarse=p.step_coarse,
                     sigma_x_initial=p.sigma_x_initial, E0=p.E0, max_iterations=p.max_iterations)
        b = rc.beam
        beam = Beam(b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples, b.seed)
        run = dict(max_iterations=rc.max_iterations, log_level=rc.log_level,
                   fail_fast_on_audit=bool(rc.fail_fast_on_audit), normalize_dose=bool(rc.normalize_dose),
                   save_2d=bool(rc.save_2d), save_pdd=bool(rc.save_pdd), output_dir=rc.output_dir.decode(),
                   dose_2d_file=rc.dose_2d_file.decode(), pdd_file=rc.pdd_file.decode())
    finally:
        lib().sm2d_run_config_free(C.byref(rc))
    return cfg, beam, run


def run_simulation(path: str):
    """run_simulation's main over the GPU engine (sm2d_run_simulation)."""
    check(lib().sm2d_run_simulation(os.fsencode(path)))


CHANNELS = ["EdepC", "AbsorbedWeight_cutoff", "AbsorbedEnergy_cutoff", "AbsorbedWeight_nuclear",
            "AbsorbedEnergy_nuclear", "BoundaryLoss_weight", "BoundaryLoss_energy", "transport_dropped_weight",
            "transport_dropped_energy", "transport_audit_residual_energy", "source_injected_weight",
            "source_out_of_grid_weight", "source_slot_dropped_weight", "source_injected_energy",
            "source_out_of_grid_energy", "source_slot_dropped_energy", "source_representation_loss_energy"]


def write_ps_raw_csv(path: str, cfg: "Config", bid: np.ndarray, val: np.ndarray, iteration: int,
                     precision: int = 8):
    """debug_ps_raw_iter_NN_<stage>.csv of psi (bid [cells*32], val
    [cells*32*L]) on cfg's grids (sm2d_write_ps_raw_csv)."""
    p, keep = cfg._problem()
    b = np.ascontiguousarray(bid, np.uint32)
    v = np.ascontiguousarray(val, np.float32)
    check(lib().sm2d_write_ps_raw_csv(os.fsencode(path), C.byref(p), _p(b), _p(v), int(iteration), int(precision)))


def write_cells_csv(path: str, cfg: "Config", bid: np.ndarray, val: np.ndarray):
    """debug_cells_iter_NN_<stage>.csv (sm2d_write_cells_csv)."""
    p, keep = cfg._problem()
    b = np.ascontiguousarray(bid, np.uint32)
    v = np.ascontiguousarray(val, np.float32)
    check(lib().sm2d_write_cells_csv(os.fsencode(path), C.byref(p), _p(b), _p(v)))


def write_channel_totals_csv(path: str, totals):
    """debug_channels_totals_iter01.csv from the 17 totals (CHANNELS order)."""
    t = np.ascontiguousarray(totals, np.float64)
    if t.shape != (17,):
        raise ValueError("17 channel totals expected")
    check(lib().sm2d_write_channel_totals_csv(os.fsencode(path), _p(t)))


def _grid(dose_2d):
    d = np.ascontiguousarray(dose_2d, np.float64)
    if d.ndim != 2:
        raise ValueError("dose grid must be [Nz, Nx]")
    return d, d.shape[1], d.shape[0]


def depth_dose(dose_2d: np.ndarray) -> np.ndarray:
    """get_depth_dose (src/validation/deterministic_beam.cpp:224-236): the
    sum over x of each row, in column order (sm2d_depth_dose)."""
    d, nx, nz = _grid(dose_2d)
    out = np.zeros(nz)
    check(lib().sm2d_depth_dose(_p(d), nx, nz, _p(out)))
    return out


def bragg_peak_row(dose_2d: np.ndarray) -> int:
    """find_bragg_peak_z (deterministic_beam.cpp:207-222): the first row of
    the largest depth dose (sm2d_bragg_peak_row)."""
    d, nx, nz = _grid(dose_2d)
    r = lib().sm2d_bragg_peak_row(_p(d), nx, nz)
    check(min(r, 0))
    return r


BRAGG_KEYS = ("peak_mm", "fwhm_mm", "r80_mm", "r20_mm", "distal_falloff_mm")


def bragg_metrics(dose_2d: np.ndarray, dz: float) -> dict:
    """Bragg-peak depth, FWHM, R80, R20 and distal falloff in mm
    (src/validation/bragg_peak.cpp; sm2d_bragg_metrics)."""
    d, nx, nz = _grid(dose_2d)
    out = np.zeros(5, np.float32)
    check(lib().sm2d_bragg_metrics(_p(d), nx, nz, float(dz), _p(out)))
    return dict(zip(BRAGG_KEYS, (float(v) for v in out)))


def write_dose_2d(path: str, dose_2d: np.ndarray, dx: float, dz: float, normalize: bool = True):
    """The reference's dose_2d.txt (run_simulation.cpp:31-75; sm2d_write_dose_2d)."""
    d, nx, nz = _grid(dose_2d)
    check(lib().sm2d_write_dose_2d(os.fsencode(path), _p(d), nx, nz, float(dx), float(dz), 1 if normalize else 0))


def write_pdd(path: str, dose_2d: np.ndarray, dz: float, normalize: bool = True):
    """The reference's pdd.txt (run_simulation.cpp:80-114; sm2d_write_pdd)."""
    d, nx, nz = _grid(dose_2d)
    check(lib().sm2d_write_pdd(os.fsencode(path), _p(d), nx, nz, float(dz), 1 if normalize else 0))
