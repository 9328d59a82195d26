"""Allocation-free K5 audit entry (sm2d_k5_conservation_audit_static):
the same report as the allocating entry (sm2d_k5_conservation_audit) on the
same device arrays, on two calls in a row, and a clear refusal of grids
larger than its static scratch.  Collected last: it must also pass after
every other test has used the library in this process."""
import ctypes as C

import numpy as np
import pytest

from sm_2d_gb300 import runtime as rt

KEMPTY = 0xFFFFFFFF
MAX_CELLS = 2048 * 256


def _args(ptrs, n_cells, E, report, stream=None):
    P = C.c_void_p
    return ([P(p) for p in ptrs] + [C.c_float(2e-4), C.c_float(1e-4), C.c_double(3e-3), C.c_double(1e-3),
                                    C.c_float(5e-5), C.c_double(2e-3), C.c_int(1), P(E), C.c_int(256),
                                    C.c_int(4), C.c_int(2), C.c_int(256), P(report), C.c_int(n_cells), P(stream)])


def _case(torch, n_cells, seed=5):
    """Caller-owned device arrays of one K5 call: psi_in/psi_out with random
    claimed slots and weights, cumulative and previous tallies."""
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda:0")
    edges, _ = rt.energy_grid_log(0.1, 250.0, 256)
    arrays = []
    for _ in range(2):   # psi_in, psi_out
        bid = np.full((n_cells, 32), KEMPTY, np.uint32)
        val = np.zeros((n_cells, 32, 256), np.float32)
        for c in range(n_cells):
            k = int(rng.integers(0, 33))
            bid[c, :k] = rng.choice(128 * 4096, size=k, replace=False).astype(np.uint32) % (128 << 12)
            v = rng.random((k, 256)).astype(np.float32) * np.float32(1e-4)
            v[rng.random((k, 256)) < 0.7] = 0.0
            val[c, :k] = v
        arrays += [torch.from_numpy(bid.view(np.int32)).to(dev), torch.from_numpy(val).to(dev)]
    bid_in, val_in, bid_out, val_out = arrays
    dbl = [torch.from_numpy(rng.random(n_cells) * 1e-3).to(dev) for _ in range(8)]
    flt = [torch.from_numpy((rng.random(n_cells) * 1e-4).astype(np.float32)).to(dev) for _ in range(6)]
    E = torch.from_numpy(edges.astype(np.float32)).to(dev)
    ptrs = [bid_in.data_ptr(), val_in.data_ptr(), bid_out.data_ptr(), val_out.data_ptr()]
    ptrs += [t.data_ptr() for t in dbl] + [t.data_ptr() for t in flt]
    keep = [bid_in, val_in, bid_out, val_out, E] + dbl + flt
    return ptrs, E.data_ptr(), keep


def _report(lib_fn, ptrs, n_cells, E, torch):
    rep = torch.zeros(C.sizeof(rt.Audit), dtype=torch.uint8, device="cuda:0")
    rc = lib_fn(*_args(ptrs, n_cells, E, rep.data_ptr()))
    assert rc == 0, rt.lib().sm2d_last_error()
    raw = bytes(rep.cpu().numpy().tobytes())
    return raw, rt.Audit.from_buffer_copy(raw).as_dict()


@pytest.mark.gpu
def test_static_k5_matches_allocating_k5_on_two_calls():
    torch = pytest.importorskip("torch")
    L = rt.lib()
    n_cells = 3000
    ptrs, E, keep = _case(torch, n_cells)
    _, want = _report(L.sm2d_k5_conservation_audit, ptrs, n_cells, E, torch)
    raw1, got1 = _report(L.sm2d_k5_conservation_audit_static, ptrs, n_cells, E, torch)
    raw2, got2 = _report(L.sm2d_k5_conservation_audit_static, ptrs, n_cells, E, torch)
    assert raw1 == raw2    # fixed-order reduction: the second call repeats the first bit for bit
    for got in (got1, got2):
        for k, v in want.items():
            if k.endswith("_total"):
                assert abs(got[k] - v) <= 1e-9 + 1e-5 * abs(v), (k, got[k], v)
        assert abs(got["W_error"] - want["W_error"]) <= 1e-6
        assert abs(got["E_error"] - want["E_error"]) <= 1e-6
        assert (got["W_pass"], got["E_pass"]) == (want["W_pass"], want["E_pass"])
        assert got["processed_cells"] == want["processed_cells"] == n_cells
    assert want["W_in_total"] > 0 and want["E_dep_total"] > 0
    del keep


def test_static_k5_refuses_grids_past_its_scratch():
    L = rt.lib()
    ptrs = [16] * 18   # never dereferenced: the size check comes first
    rc = L.sm2d_k5_conservation_audit_static(*_args(ptrs, MAX_CELLS + 1, 16, 16))
    assert rc == -1
    msg = L.sm2d_last_error()
    msg = msg.decode() if isinstance(msg, bytes) else msg
    assert "524288" in msg and "static scratch" in msg
