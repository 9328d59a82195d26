"""The raw stage entries on caller-owned device arrays against the oracle:
sm2d_k1_active_mask and sm2d_compact_lists on the reference's golden phase
spaces (results/one_step_case_{A..D}; mask and both lists bit-exact against
the oracle's first iteration, k1_activemask.cu:6-48, k1k6_pipeline.cu:589-665),
sm2d_k5_conservation_audit on the same iteration's psi_in, psi_out and
tallies (the oracle's audit record, k5_audit.cu:22-167, totals within 1e-5),
and sm2d_k4_bucket_transfer on synthetic buckets that saturate their
destination cells (k4_transfer.cu:174-333: the block id of every slot
bit-exact, values within float-summation noise, the dropped weight)."""
import ctypes as C

import numpy as np
import pytest

import sm_2d_gb300 as sm
from sm_2d_gb300 import runtime as rt
from golden_cases import load_case

pytestmark = pytest.mark.gpu
KB, EMPTY = 32, 0xFFFFFFFF
P = C.c_void_p


def _dev(torch, a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a).to("cuda:0")


def _find_bin(edges, E):
    """EnergyGrid::FindBin (grids.cpp): the bin holding E, clamped."""
    n = edges.size - 1
    if E <= edges[0]:
        return 0
    if E >= edges[n]:
        return n - 1
    return int(np.searchsorted(edges, np.float32(E), side="right")) - 1


@pytest.mark.parametrize("name", ["A", "B", "C", "D"])
def test_k1_compaction_k5_equal_the_oracle_on_golden_cases(name, oracle_mod):
    import torch
    case = load_case(name)
    cfg = case["cfg"]
    Nx, Nz = cfg["Nx"], cfg["Nz"]
    Nc, L = Nx * Nz, 256
    o = oracle_mod.Oracle(cfg, case["theta_edges"], case["E_edges"])
    o.set_psi_in(case["bid_in"], case["val_in"])
    o.step()
    E = np.asarray(case["E_edges"], np.float32)
    b_on = _find_bin(E, cfg.get("E_fine_on", 10.0)) // 2
    b_off = _find_bin(E, cfg.get("E_fine_off", 11.0)) // 2
    lib = rt.lib()
    bid, val = _dev(torch, case["bid_in"]), _dev(torch, case["val_in"])
    mask = torch.zeros(Nc, dtype=torch.uint8, device="cuda:0")
    prev = torch.zeros_like(mask)
    rt.check(lib.sm2d_k1_active_mask(P(bid.data_ptr()), P(val.data_ptr()), P(mask.data_ptr()), P(prev.data_ptr()),
                                     Nx, Nz, L, b_on, b_off, C.c_float(cfg.get("weight_active_min", 1e-12)), None))
    act = torch.zeros(Nc, dtype=torch.int32, device="cuda:0")
    coa = torch.zeros_like(act)
    cnt = torch.zeros(2, dtype=torch.int32, device="cuda:0")
    rt.check(lib.sm2d_compact_lists(P(mask.data_ptr()), P(bid.data_ptr()), P(val.data_ptr()), Nx, Nz, L,
                                    P(act.data_ptr()), P(cnt.data_ptr()), P(coa.data_ptr()), P(cnt.data_ptr() + 4),
                                    None))
    torch.cuda.synchronize()
    assert np.array_equal(mask.cpu().numpy(), o.mask())
    na, nc = cnt.cpu().numpy().tolist()
    oa, oc = o.lists()
    assert np.array_equal(act.cpu().numpy()[:na].view(np.uint32), oa)
    assert np.array_equal(coa.cpu().numpy()[:nc].view(np.uint32), oc)
    # K5 over the iteration: psi_in before, psi_out after, the tallies it
    # booked (the previous tallies are zero before the first iteration)
    ob, ov = o.psi_in()
    tal = o.tallies()
    sc = o.scalars()
    bout, vout = _dev(torch, ob), _dev(torch, ov)
    d = {k: _dev(torch, np.asarray(tal[k])) for k in ("edep", "e_nuc", "e_bnd", "e_cut", "w_cut", "w_nuc", "w_bnd")}
    zd = torch.zeros(Nc, dtype=torch.float64, device="cuda:0")
    zf = torch.zeros(Nc, dtype=torch.float32, device="cuda:0")
    Ed = _dev(torch, E)
    rep = torch.zeros(256, dtype=torch.uint8, device="cuda:0")
    ptrs = [bid, val, bout, vout, d["edep"], d["e_nuc"], d["e_bnd"], d["e_cut"], zd, zd, zd, zd, d["w_cut"], d["w_nuc"],
            d["w_bnd"], zf, zf, zf]
    rt.check(lib.sm2d_k5_conservation_audit(
        *[P(t.data_ptr()) for t in ptrs], C.c_float(sc["source_out_of_grid_weight"]),
        C.c_float(sc["source_slot_dropped_weight"]), C.c_double(sc["source_out_of_grid_energy"]),
        C.c_double(sc["source_slot_dropped_energy"]), C.c_float(sc["transport_dropped_weight"]),
        C.c_double(sc["transport_dropped_energy"]), 1, P(Ed.data_ptr()), E.size - 1, 4, 2, L, P(rep.data_ptr()), Nc,
        None))
    torch.cuda.synchronize()
    got = rt.Audit.from_buffer_copy(rep.cpu().numpy().tobytes()[:C.sizeof(rt.Audit)]).as_dict()
    want = o.audit()
    for k, v in want.items():
        if k.endswith("_total"):
            assert abs(got[k] - v) <= 1e-9 + 1e-5 * abs(v), (name, k, got[k], v)
    assert got["processed_cells"] == want["processed_cells"]
    assert (got["W_pass"], got["E_pass"]) == (want["W_pass"], want["E_pass"])


def test_k4_equals_the_oracle_on_saturating_buckets(oracle_mod):
    """Buckets of 12 x 10 cells with 40 candidate ids per destination (more
    than its 32 slots), some destinations already holding slots: claims,
    nearest-block fallback with the local-bin remap, and drops."""
    import torch
    Nx, Nz, L = 12, 10, 256
    Nc = Nx * Nz
    cfg = sm.Config.reference_runner(Nx, Nz, 0.5, 0.5)
    E = np.asarray(cfg.E_edges, np.float32)
    rng = np.random.default_rng(3)
    listed = np.sort(rng.choice(Nc, size=70, replace=False))
    c2b = np.full(Nc, -1, np.int32)
    c2b[listed] = 4 * np.arange(listed.size)
    nb = 4 * listed.size
    pool = np.array([((be & 0xFFF) << 12) | (bt & 0xFFF) for be in range(60, 100, 4) for bt in range(4)], np.uint32)
    bb = np.full((nb, KB), EMPTY, np.uint32)
    bv = np.zeros((nb, KB, L), np.float32)
    for i in range(nb):
        k = int(rng.integers(0, KB + 1))
        bb[i, :k] = rng.choice(pool, size=k, replace=False)
        v = (rng.random((k, L)) * 1e-3).astype(np.float32)
        v[rng.random((k, L)) < 0.8] = 0.0
        bv[i, :k] = v
    ob = np.full((Nc, KB), EMPTY, np.uint32)
    ov = np.zeros((Nc, KB, L), np.float32)
    for cell in rng.choice(Nc, size=30, replace=False):
        k = int(rng.integers(1, 20))
        ob[cell, :k] = rng.choice(pool, size=k, replace=False)
        ov[cell, :k, :] = (rng.random((k, L)) * 1e-3).astype(np.float32)
    o = oracle_mod.Oracle(cfg.oracle_config(), cfg.theta_edges, cfg.E_edges)
    wb, wv, wdrop = o.k4_raw(bb, bv, c2b, ob.ravel(), ov.ravel())
    # the DeviceOutflowBucket bytes: ids, counts, values, three moments
    bucket_bytes = rt.lib().sm2d_bucket_bytes(L)
    raw = np.zeros((nb, bucket_bytes), np.uint8)
    raw[:, :128] = bb.view(np.uint8).reshape(nb, 128)
    raw[:, 192:192 + KB * L * 4] = bv.reshape(nb, -1).view(np.uint8)
    dbkt, dc2b = _dev(torch, raw), _dev(torch, c2b)
    gb, gv = _dev(torch, ob.ravel()), _dev(torch, ov.ravel())
    Ed = _dev(torch, E)
    drop = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    lib = rt.lib()
    rt.check(lib.sm2d_k4_bucket_transfer(P(dbkt.data_ptr()), P(dc2b.data_ptr()), P(gv.data_ptr()), P(gb.data_ptr()),
                                         Nx, Nz, L, 4, 2, 8, P(Ed.data_ptr()), E.size - 1, 2, P(drop.data_ptr()),
                                         None))
    torch.cuda.synchronize()
    got_b = gb.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_b, wb)
    np.testing.assert_allclose(gv.cpu().numpy(), wv, rtol=1e-5, atol=1e-9)
    gd = drop.cpu().numpy()
    assert (wb.reshape(Nc, KB) != EMPTY).all(axis=1).sum() >= 5   # destinations filled all 32 slots (fallback ran)
    np.testing.assert_allclose(gd, wdrop, rtol=1e-9, atol=1e-12)
