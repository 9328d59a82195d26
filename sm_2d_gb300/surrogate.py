"""Learned redistribution surrogate of the fine transport step (host side).

``Surrogate`` owns one network (sm2d_mlp_* in libsm2d.so) and one small
transport handle whose stream runs its work.  The network predicts the
expectation form's redistribution weights of one fine-step component -- the
8 theta x 4 E table of the expected Highland-MCS / Vavilov-straggling /
energy-split re-binning that K3_FineTransport (src/cuda/kernels/
k3_finetransport.cu:263-366) samples once per bin -- from four numbers:
s = sigma_theta / dtheta, u (the mean energy's position between the energy
centres around it), r = sigma_E / their spacing, and cap (the energy window's
top is the incoming bin).  sm2d_redistribution_table evaluates the method's
own closed forms.  Training, inference and the tables run on the GPU; torch
provides the device arrays.  There is no CPU path: without the library or a
GPU every call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .runtime import Config, Transport, check, lib

N_PARAMS = 22816
N_OUT = 32
REGIONS = 64 * 8 * 8
_READY = False


def _lib():
    global _READY
    L = lib()
    if not _READY:
        P, I, F = C.c_void_p, C.c_int, C.c_float
        L.sm2d_mlp_create.argtypes = [I, P, C.POINTER(P)]
        L.sm2d_mlp_destroy.argtypes = [P]
        L.sm2d_mlp_set_params.argtypes = [P, P]
        L.sm2d_mlp_get_params.argtypes = [P, P]
        L.sm2d_mlp_gradients.argtypes = [P, P, P, I, P, P]
        L.sm2d_mlp_train.argtypes = [P, P, P, I, I, I, F, F, P]
        L.sm2d_mlp_forward.argtypes = [P, P, I, P]
        L.sm2d_redistribution_features.argtypes = [I, C.c_uint32, P, P]
        L.sm2d_redistribution_table.argtypes = [P, P, I, P]
        L.sm2d_mlp_calibrate.argtypes = [P, P, P, P, I, P]
        L.sm2d_mlp_redistribute.argtypes = [P, P, P, I, F, P, P]
        L.sm2d_mlp_geometry.argtypes = [P]
        L.sm2d_mlp_sync.argtypes = [P]
        _READY = True
    return L


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class Surrogate:
    """The network, its training set and the method's tables on cuda:0."""

    def __init__(self, max_batch: int | None = None):
        import torch

        self.torch = torch
        if not torch.cuda.is_available():
            raise RuntimeError("the redistribution surrogate needs a CUDA device")
        self.L = _lib()
        # a small transport handle: its stream runs the surrogate's work
        self.t = Transport(Config.reference_runner(4, 4, 0.5, 0.5))
        self.sms = torch.cuda.get_device_properties(0).multi_processor_count
        self.batch = 128 * self.sms   # one 128-sample tile per SM
        h = C.c_void_p()
        check(self.L.sm2d_mlp_create(max(self.batch, max_batch or 0), self.t.stream(), C.byref(h)))
        self.m = h

    def close(self):
        if getattr(self, "m", None):
            self.L.sm2d_mlp_destroy(self.m)
            self.m = None
        if getattr(self, "t", None):
            self.t.close()
            self.t = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _sync(self):
        self.torch.cuda.synchronize()

    def sync(self):
        """Wait for the handle's stream; raises if a kernel's bounded wait gave up."""
        check(self.L.sm2d_mlp_sync(self.m))

    def features(self, n: int, seed: int):
        """n inputs (s, u, r, cap) of the training distribution, [n][4] on the device."""
        f = self.torch.empty((n, 4), dtype=self.torch.float32, device="cuda")
        self._sync()
        check(self.L.sm2d_redistribution_features(n, seed, _ptr(f), self.t.stream()))
        self._sync()
        return f

    def plain(self, feats):
        """The method's own tables of the rows of feats, [n][32] on the device."""
        out = self.torch.empty((feats.shape[0], N_OUT), dtype=self.torch.float32, device="cuda")
        self._sync()
        check(self.L.sm2d_redistribution_table(self.t.h, _ptr(feats), feats.shape[0], _ptr(out)))
        self._sync()
        return out

    def forward(self, feats):
        out = self.torch.empty((feats.shape[0], N_OUT), dtype=self.torch.float32, device="cuda")
        self._sync()
        check(self.L.sm2d_mlp_forward(self.m, _ptr(feats), feats.shape[0], _ptr(out)))
        self.sync()
        self._sync()
        return out

    def params(self) -> np.ndarray:
        p = np.zeros(N_PARAMS, np.float32)
        check(self.L.sm2d_mlp_get_params(self.m, p.ctypes.data_as(C.c_void_p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(self.L.sm2d_mlp_set_params(self.m, p.ctypes.data_as(C.c_void_p)))

    def gradients(self, feats, target):
        """(loss, gradient) of the mean cross-entropy of the rows; no update."""
        g = self.torch.empty(N_PARAMS, dtype=self.torch.float32, device="cuda")
        loss = self.torch.empty(1, dtype=self.torch.float32, device="cuda")
        self._sync()
        check(self.L.sm2d_mlp_gradients(self.m, _ptr(feats), _ptr(target), feats.shape[0], _ptr(g), _ptr(loss)))
        self.sync()
        self._sync()
        return float(loss.item()), g.cpu().numpy()

    def train(self, feats, target, steps: int, lr0: float = 2e-3, lr_min: float = 2e-5, batch: int | None = None):
        """Adam steps over the set; returns the per-step loss."""
        batch = batch or self.batch
        hist = self.torch.zeros(max(steps, 1), dtype=self.torch.float32, device="cuda")
        self._sync()
        check(self.L.sm2d_mlp_train(self.m, _ptr(feats), _ptr(target), feats.shape[0], batch, steps, lr0, lr_min,
                                    _ptr(hist)))
        self.sync()
        return hist[:steps].cpu().numpy()

    def calibrate(self, feats, plain=None):
        """Per-region largest weight error of the network against the method, as float [4096]."""
        plain = self.plain(feats) if plain is None else plain
        surr = self.forward(feats)
        err = np.zeros(REGIONS, np.float32)
        check(self.L.sm2d_mlp_calibrate(self.m, _ptr(feats), _ptr(plain), _ptr(surr), feats.shape[0],
                                        err.ctypes.data_as(C.c_void_p)))
        return err

    def redistribute(self, feats, tol: float = 0.005):
        """Network tables with the method's rows where the calibrated error exceeds tol."""
        n = feats.shape[0]
        out = self.torch.empty((n, N_OUT), dtype=self.torch.float32, device="cuda")
        fb = self.torch.zeros(n, dtype=self.torch.int32, device="cuda")
        self._sync()
        check(self.L.sm2d_mlp_redistribute(self.m, self.t.h, _ptr(feats), n, tol, _ptr(out), _ptr(fb)))
        self.sync()
        self._sync()
        return out, fb

    @staticmethod
    def geometry():
        g = np.zeros(8, np.float32)
        check(_lib().sm2d_mlp_geometry(g.ctypes.data_as(C.c_void_p)))
        return dict(zip(["s_max", "u_max", "r_max", "cap_max", "regions_s", "regions_u", "regions_r",
                         "regions_cap"], g.tolist()))


def main(argv=None):
    """Train the surrogate on the method's tables and report its accuracy and speed.

    python -m sm_2d_gb300.surrogate [--train N] [--steps S] [--rows R]
    """
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=1 << 20, help="training rows")
    ap.add_argument("--steps", type=int, default=1000, help="Adam steps")
    ap.add_argument("--rows", type=int, default=1 << 20, help="rows of the inference pass")
    a = ap.parse_args(argv)
    with Surrogate() as s:
        f = s.features(a.train, 1)
        hist = s.train(f, s.plain(f), steps=a.steps)
        fe = s.features(a.rows, 2)
        ref = s.plain(fe)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream = torch.cuda.ExternalStream(s.t.stream())
        e0.record(stream)
        out = s.forward(fe)
        e1.record(stream)
        torch.cuda.synchronize()
        print(json.dumps({"loss_first": float(hist[0]), "loss_last": float(hist[-1]),
                          "mean_abs_weight_error": float((out - ref).abs().mean()),
                          "forward_ms": e0.elapsed_time(e1), "rows": a.rows}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
