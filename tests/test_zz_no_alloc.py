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


def _args(ptrs, n_cells, E, report, stream=None, layout=(4, 2, 256)):
    P = C.c_void_p
    nt, ne, L = layout
    return ([P(p) for p in ptrs] + [C.c_float(2e-4), C.c_float(1e-4), C.c_double(3e-3), C.c_double(1e-3),
                                    C.c_float(5e-5), C.c_double(2e-3), C.c_int(1), P(E), C.c_int(256),
                                    C.c_int(nt), C.c_int(ne), C.c_int(L), P(report), C.c_int(n_cells), P(stream)])


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


def _case_device(torch, n_cells, seed=7):
    """The same kind of K5 inputs generated on the device, for grids too large
    to build on the host: 128 local bins (8 theta x 4 E x 4 x_sub), up to 4
    claimed slots per cell, 30 % of their bins holding weight."""
    g = torch.Generator(device="cuda:0")
    g.manual_seed(seed)
    dev = torch.device("cuda:0")
    L = 128
    edges, _ = rt.energy_grid_log(0.1, 250.0, 256)
    arrays = []
    for _ in range(2):   # psi_in, psi_out
        k = torch.randint(0, 5, (n_cells, 1), device=dev, generator=g)
        slot = torch.arange(32, device=dev).unsqueeze(0)
        ids = (torch.randint(0, 64, (n_cells, 32), device=dev, generator=g) << 12) | torch.randint(
            0, 64, (n_cells, 32), device=dev, generator=g)
        bid = torch.where(slot < k, ids, torch.full_like(ids, -1)).to(torch.int32)
        val = torch.empty((n_cells, 32, L), dtype=torch.float32, device=dev)
        for c0 in range(0, n_cells, 65536):   # in chunks: no full-size temporaries
            v = val[c0:c0 + 65536]
            v.uniform_(0.0, 1.0, generator=g)
            v.masked_fill_(v < 0.7, 0.0)
            v.mul_(1e-4)
        arrays += [bid, val]
    bid_in, val_in, bid_out, val_out = arrays
    dbl = [torch.rand(n_cells, dtype=torch.float64, device=dev, generator=g) * 1e-3 for _ in range(8)]
    flt = [torch.rand(n_cells, dtype=torch.float32, device=dev, generator=g) * 1e-4 for _ in range(6)]
    E = torch.from_numpy(edges.astype(np.float32)).to(dev)
    ptrs = [bid_in.data_ptr(), val_in.data_ptr(), bid_out.data_ptr(), val_out.data_ptr()]
    ptrs += [t.data_ptr() for t in dbl] + [t.data_ptr() for t in flt]
    keep = [bid_in, val_in, bid_out, val_out, E] + dbl + flt
    return ptrs, E.data_ptr(), keep


def _report(lib_fn, ptrs, n_cells, E, torch, layout=(4, 2, 256)):
    rep = torch.zeros(C.sizeof(rt.Audit), dtype=torch.uint8, device="cuda:0")
    rc = lib_fn(*_args(ptrs, n_cells, E, rep.data_ptr(), layout=layout))
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


@pytest.mark.gpu
@pytest.mark.parametrize("n_cells", [70000, MAX_CELLS])
def test_static_k5_on_large_grids(n_cells):
    """Grids of more than 256 blocks, where the last block's final sum strides
    over the block rows, and a grid of exactly the scratch's 524288 cells:
    the static entry equals the allocating one, and repeats itself bit for
    bit on a second call."""
    torch = pytest.importorskip("torch")
    L = rt.lib()
    layout = (8, 4, 128)
    ptrs, E, keep = _case_device(torch, n_cells)
    _, want = _report(L.sm2d_k5_conservation_audit, ptrs, n_cells, E, torch, layout)
    raw1, got = _report(L.sm2d_k5_conservation_audit_static, ptrs, n_cells, E, torch, layout)
    raw2, _ = _report(L.sm2d_k5_conservation_audit_static, ptrs, n_cells, E, torch, layout)
    assert raw1 == raw2
    for k, v in want.items():
        if k.endswith("_total"):
            assert abs(got[k] - v) <= 1e-9 + 1e-5 * abs(v), (k, got[k], v)
    assert abs(got["E_error"] - want["E_error"]) <= 1e-6
    assert got["processed_cells"] == want["processed_cells"] == n_cells
    assert want["W_in_total"] > 0 and want["W_out_total"] > 0
    del keep
    torch.cuda.empty_cache()


def test_static_k5_refuses_grids_past_its_scratch():
    L = rt.lib()
    ptrs = [16] * 18   # never dereferenced: the size check comes first
    rc = L.sm2d_k5_conservation_audit_static(*_args(ptrs, MAX_CELLS + 1, 16, 16))
    assert rc == -1
    msg = L.sm2d_last_error()
    msg = msg.decode() if isinstance(msg, bytes) else msg
    assert "524288" in msg and "static scratch" in msg
