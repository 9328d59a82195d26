// sm2d_transport.cuh -- per-bin coarse (K2) and fine (K3) transport and the
// emission of the moved weight, for one warp per listed cell.
//
// Method (reference files cited inline): every nonzero local bin of a
// listed cell is one component at its bin-centre angle/energy and sub-cell
// centre.  K2 (cells without low-energy blocks) takes a step of
// min(step_coarse, dx, dz), split at the fine-transport threshold; K3 takes
// an R-limited step capped by the distance to the cell boundary, with
// hashed Vavilov straggling.  Both apply nuclear attenuation and one hashed
// MCS angle sample, then either cross a face or stay in the cell.
//
// Every bin is transported twice with the same arithmetic.  PASS_KEYS
// gathers, per psi_out cell and per outflow bucket, the block ids aimed at
// it with their sequential claim keys (see the claim tables in
// sm2d_device.cuh); the selection kernels then fix each container's slots.
// The deposit pass resolves every emission to its slot and adds the weight:
//   * PASS_DIRECT scatters straight into psi_out of the destination cell
//     (the neighbour-scatter form of K4 fused into the transport kernel,
//     through the bucket's kept id as K4 would);
//   * PASS_BUCKET writes the reference's DeviceOutflowBucket of the source
//     cell and face; the bucket move kernel then runs K4_BucketTransfer.
#pragma once
#include "sm2d_device.cuh"
#include "sm2d_redist.h"

namespace sm2d {

enum { FACE_ZP = 0, FACE_ZM = 1, FACE_XP = 2, FACE_XM = 3 };
enum { PASS_KEYS = 0, PASS_DIRECT = 1, PASS_BUCKET = 2 };

struct Tally {                // per-lane accumulators of one work item
    double edep, e_cut, e_nuc, e_bnd;
    float w_cut, w_nuc, w_bnd;
    double drop_w, drop_e;    // slot / bucket / prune drops
};

// The component being transported: its cell, psi_in slot and local bin give
// the sequential claim order; k3 selects the batch; E is its energy after
// the step (the energy its drops are booked with).
struct Src {
    int cell, slot, lidx, k3;
    uint32_t tag;   // classification number of this pass
    float E;
};

__device__ __forceinline__ float e_center(const Dev& d, int b) { return d.Ee[b] + 0.5f * (d.Ee[b + 1] - d.Ee[b]); }

struct EParts {
    int n;
    int bin[2];
    float frac[2];
    float Erep;
};
// Energy re-binning of an emitted component: the bin containing E
// (device_find_bin_edges), or with the energy split a mean-preserving pair of
// neighbouring bin centres.
__device__ __forceinline__ EParts bin_energy(const Dev& d, float E, float w) {
    EParts p;
    int k = find_ebin(d, E);
    p.n = 1;
    p.bin[0] = p.bin[1] = k;
    p.frac[0] = 1.0f;
    p.frac[1] = 0.0f;
    p.Erep = e_center(d, k);
    if (!d.esplit) return p;
    float ck = p.Erep;
    int lo = E >= ck ? k : k - 1, hi = lo + 1;
    if (lo < 0 || hi > d.N_E - 1) return p;
    float cl = e_center(d, lo), ch = e_center(d, hi);
    float fh = (E - cl) / (ch - cl);
    if (fh <= 0.0f) { p.bin[0] = lo; p.Erep = cl; return p; }
    if (fh >= 1.0f) { p.bin[0] = hi; p.Erep = ch; return p; }
    if (w * fminf(fh, 1.0f - fh) < d.split_min_w) {   // light minor part stays with the major bin
        if (fh >= 0.5f) { p.bin[0] = hi; p.Erep = ch; } else { p.bin[0] = lo; p.Erep = cl; }
        return p;
    }
    p.n = 2;
    p.bin[0] = lo; p.frac[0] = 1.0f - fh;
    p.bin[1] = hi; p.frac[1] = fh;
    p.Erep = p.frac[0] * cl + p.frac[1] * ch;
    return p;
}

__device__ __forceinline__ unsigned long long* psi_row(const Dev& d, int cell) {
    return d.ctab + (size_t)cell * (2 * kCand);
}
__device__ __forceinline__ unsigned long long* bucket_row(const Dev& d, int bf) {
    return d.ctab + ((size_t)d.B * d.Nc + bf) * (2 * kCand);
}
// claim keys: psi_out rows [batch:1][part:3][slot:5][lidx:8][part index:6]
// (part 0 in-cell deposit, 1 + f the K4 transfer of face f by bucket slot);
// bucket rows [emitting column 0..10:4][slot:5][lidx:8][emission index:6].
// The emission index is the energy part (sampled form) or the child
// 16 e + k of the expectation form, in the order the oracle emits them.
__device__ __forceinline__ uint32_t stay_key(int k3, int slot, int lidx, int ei) {
    return ((uint32_t)k3 << 22) | ((uint32_t)slot << 14) | ((uint32_t)lidx << 6) | (uint32_t)ei;
}
__device__ __forceinline__ uint32_t k4_key(int k3, int face, int kslot) {
    return ((uint32_t)k3 << 22) | ((uint32_t)(1 + face) << 19) | (uint32_t)kslot;
}
__device__ __forceinline__ uint32_t bucket_key(int col, int slot, int lidx, int seq) {
    return ((uint32_t)col << 19) | ((uint32_t)slot << 14) | ((uint32_t)lidx << 6) | (uint32_t)seq;
}
template <class Lay>
__device__ __forceinline__ int ebin_of(const Dev& d, uint32_t bid, int l) {
    return max(0, min((int)((bid >> 12) & 0xFFFu) * Lay::NE + (l / Lay::NT) % Lay::NE, d.N_E - 1));
}

// Slot of block `want` in a selected container and the kept id there (want
// itself or the nearest kept id it folds into).  An id that was not
// gathered (claim-table overflow) takes the nearest kept id and is counted.
// An id the row did not gather: the slot of the nearest kept id, -1 if none.
static __device__ __noinline__ int resolve_miss(const Dev& d, const uint32_t* kept, uint32_t want) {
    atomicAdd(&d.gs->cand_miss, 1);
    int s = -1, bd = 0x7fffffff;
    for (int k = 0; k < kKb; ++k) {
        const uint32_t x = kept[k];
        if (x == kEmpty) continue;
        const int dd = bid_distance(x, want);
        if (dd < bd) { bd = dd; s = k; }
    }
    return s;
}
template <bool RO = false>
__device__ __forceinline__ int resolve(const Dev& d, const unsigned long long* row, const uint32_t* kept, uint32_t tag,
                                       uint32_t want, uint32_t& sel) {
    int s = cand_find<RO>(row, tag, want, sel);
    if (s >= 0) return s;
    s = resolve_miss(d, kept, want);
    sel = s >= 0 ? kept[s] : want;
    return s;
}

// Weight w of local bin lidx of block `want` leaving through bucket
// (bcell, face) towards dcell; col is the emitting column seen from bcell
// (0..10, 5 = bcell itself) and seq the emission index within the bin.
// Returns the weight that found no container.
// Angle and energy re-binning of an emitted component at (theta, E), the
// weight-independent part of emit_component: the nearest theta-bin centre
// and its neighbour with the frac^2 share, and the energy bin (with the
// energy split: the neighbouring centres and the upper share).  The lateral
// spread emits the same (theta, E) into up to 11 cells, so it is computed
// once per component.
struct EmitPlan {
    int bc, tb1;      // theta: nearest centre bin, neighbour (== bc: none)
    float tw1;        // frac^2 share of the neighbour
    int k;            // energy bin containing E (device_find_bin_edges)
    int lo, hi;       // split method: centres around E (lo < 0: no split)
    float fh;         // split method: share of hi
};
__device__ __forceinline__ EmitPlan plan_emission(const Dev& d, float theta, float E) {
    EmitPlan p;
    const float tmin = d.th[0], tmax = d.th[d.N_theta];
    const float dth = (tmax - tmin) / (float)d.N_theta;
    const float tc = fmaxf(tmin, fminf(theta, tmax));
    const float c0 = tmin + 0.5f * dth;
    int bc = (int)floorf((tc - c0) / dth + 0.5f);
    bc = max(0, min(bc, d.N_theta - 1));
    const float delta = tc - (c0 + (float)bc * dth);
    int tb1 = bc;
    if (delta > 0.0f && bc < d.N_theta - 1) tb1 = bc + 1;
    else if (delta < 0.0f && bc > 0) tb1 = bc - 1;
    p.bc = bc;
    p.tb1 = tb1;
    p.tw1 = 0.0f;
    if (tb1 != bc) {
        const float f = fminf(1.0f, fabsf(delta) / dth);
        p.tw1 = f * f;
    }
    const float Ec = fmaxf(d.Ee[0], fminf(E, d.Ee[d.N_E]));
    const int k = find_ebin(d, Ec);
    p.k = k;
    p.lo = -1;
    p.hi = -1;
    p.fh = 0.0f;
    if (d.esplit) {
        const float ck = e_center(d, k);
        const int lo = Ec >= ck ? k : k - 1, hi = lo + 1;
        if (lo >= 0 && hi <= d.N_E - 1) {
            const float cl = e_center(d, lo), ch = e_center(d, hi);
            p.lo = lo;
            p.hi = hi;
            p.fh = (Ec - cl) / (ch - cl);
        }
    }
    return p;
}
// bin_energy of a planned component of weight w
__device__ __forceinline__ EParts plan_energy(const Dev& d, const EmitPlan& p, float w) {
    EParts e;
    e.n = 1;
    e.bin[0] = e.bin[1] = p.k;
    e.frac[0] = 1.0f;
    e.frac[1] = 0.0f;
    e.Erep = e_center(d, p.k);
    if (!d.esplit || p.lo < 0) return e;
    const float cl = e_center(d, p.lo), ch = e_center(d, p.hi), fh = p.fh;
    if (fh <= 0.0f) { e.bin[0] = p.lo; e.Erep = cl; return e; }
    if (fh >= 1.0f) { e.bin[0] = p.hi; e.Erep = ch; return e; }
    if (w * fminf(fh, 1.0f - fh) < d.split_min_w) {   // light minor part stays with the major bin
        if (fh >= 0.5f) { e.bin[0] = p.hi; e.Erep = ch; } else { e.bin[0] = p.lo; e.Erep = cl; }
        return e;
    }
    e.n = 2;
    e.bin[0] = p.lo; e.frac[0] = 1.0f - fh;
    e.bin[1] = p.hi; e.frac[1] = fh;
    e.Erep = e.frac[0] * cl + e.frac[1] * ch;
    return e;
}

template <class Lay, int PASS>
__device__ __forceinline__ float put(const Dev& d, const Src& src, int par, int bcell, int face, int dcell, int col,
                                     int seq, uint32_t want, int lidx, float w, Tally& t) {
    // a drop leaves through the single exit at the end: a bucket drop of the
    // transport's stage, or an output-slot drop of the fused K4
    int stage = src.k3;
    const int base = d.c2b[bcell];
    if (base >= 0) {
        const int bf = base + face;
        if (PASS == PASS_KEYS) {
            cand_insert(bucket_row(d, bf), d.ccount + (size_t)d.B * d.Nc + bf, src.tag, want,
                        bucket_key(col, src.slot, src.lidx, seq),
                        &d.gs->cand_ovf);
            return 0.0f;
        }
        // the bucket's kept id from the probe; for the fused pass its psi_out
        // slot and that slot's id in one entry (bkt_slot_pack)
        uint32_t selb;
        const int kb = resolve<true>(d, bucket_row(d, bf), d.bkt_ids + (size_t)bf * kKb, src.tag, want, selb);
        if (kb >= 0) {
            const uint2 m = PASS == PASS_BUCKET ? make_uint2(0u, 0u) : __ldg(d.bkt_os + (size_t)bf * kKb + kb);
            const int le = (selb == want) ? lidx : remap_lidx<Lay>(lidx, want, selb);
            if (selb != want && d.esplit)   // split method: a re-binned part keeps its energy
                t.edep += (double)((e_center(d, ebin_of<Lay>(d, want, lidx)) - e_center(d, ebin_of<Lay>(d, selb, le))) * w);
            if (PASS == PASS_BUCKET) {
                float* vals = bucket_vals(d.buckets + (size_t)bf * d.bucket_bytes);
                atomicAdd(vals + (size_t)kb * Lay::L + le, w);
                return 0.0f;
            }
            // K4 of the fused pass: the bucket's kept id lands in dcell's psi_out
            // slot (its value page) that the selection resolved for it
            const int pg = bkt_slot_page(m);
            if (pg >= 0) {
                const uint32_t seld = m.y;
                const int le2 = (seld == selb) ? le : remap_lidx<Lay>(le, selb, seld);
                if (seld != selb && d.esplit)
                    atomicAdd(d.dl_edep + bcell,
                              (double)((e_center(d, ebin_of<Lay>(d, selb, le)) - e_center(d, ebin_of<Lay>(d, seld, le2))) * w));
                vadd(d, (size_t)pg, Lay::L, le2, w);
                return 0.0f;
            }
            stage = 2;
        }
    }
    if (PASS != PASS_KEYS) count_drop(d.gs, stage, stage == 2 ? DROP_SLOT : DROP_BUCKET, (double)w, (double)(src.E * w));
    return w;
}

// Two-bin theta split around the nearest bin centre with frac^2 weight to
// the neighbour, energy re-binning, bucket claim (device_bucket.cuh:431-533),
// for a component planned by plan_emission.
template <class Lay, int PASS>
__device__ float emit_component(const Dev& d, const Src& src, int par, int bcell, int face, int dcell, int col,
                                const EmitPlan& pl, float weight, int xs, int zs, Tally& t) {
    if (weight <= 0.0f) return 0.0f;
    float tw0 = 1.0f, tw1 = 0.0f;
    if (pl.tb1 != pl.bc) {
        tw1 = pl.tw1;
        tw0 = 1.0f - tw1;
        if (d.esplit && weight * tw1 < d.split_min_w) { tw1 = 0.0f; tw0 = 1.0f; }
    }
    const EParts ep = plan_energy(d, pl, weight);
    float dropped = 0.0f;
    for (int ei = 0; ei < ep.n; ++ei) {
        const int Eb = ep.bin[ei];
        const int El = Eb % Lay::NE;
        const uint32_t bE = (uint32_t)(Eb / Lay::NE);
#pragma unroll
        for (int ti = 0; ti < 2; ++ti) {
            const float wt = ti ? tw1 : tw0;
            if (wt <= 0.0f) continue;
            float we = weight * wt;
            if (d.esplit) we = we * ep.frac[ei];
            const int tb = ti ? pl.tb1 : pl.bc;
            const uint32_t want = make_bid((uint32_t)(tb / Lay::NT), bE);
            const int l = Lay::enc(tb % Lay::NT, El, xs, zs);
            dropped += put<Lay, PASS>(d, src, par, bcell, face, dcell, col, 2 * ei + ti, want, l, we, t);
        }
    }
    return dropped;
}

// Expectation form: the children of one component (sm2d_redist.h).  c is
// its incoming angle bin; j the top of its energy window: the second centre
// above the step's mean energy Em, at most the incoming bin jin (a step
// gains no energy).  Child k of energy offset e goes to angle bin c - t or
// c + t (t = (k + 1) / 2) and energy bin j - e.
struct Kids {
    int c, j, emax;
    float Mt[SM2D_RD_NT], Me[SM2D_RD_NE];
    float Erep;   // represented energy of the children
    uint32_t live;   // bit t + 8 e: the child of angular distance t, energy offset e has weight
};
__device__ __forceinline__ int kid_window_top(const Dev& d, int jin, float Em) {
    const float Ec = fmaxf(d.Ee[0], fminf(Em, d.Ee[d.N_E]));
    const int b = find_ebin(d, Ec);
    const int up = Ec >= e_center(d, b) ? b + 1 : b;   // the lowest centre at or above Em
    return min(jin, up + 1);
}
// The learned surrogate's features of a component (sm2d_surrogate.cu):
// s = sigma_theta / dtheta; u, where the mean energy Em lies between the
// centres around it; r = sigma_E / their spacing; cap = 1 when the window's
// top is the incoming bin.  cap = -1 marks a component outside the network's
// domain (a window of fewer than four centres or of uneven spacing), which
// keeps the closed forms.
__device__ __forceinline__ float4 surr_features(const Dev& d, int jin, float s, float Em, float sE) {
    const float Ec = fmaxf(d.Ee[0], fminf(Em, d.Ee[d.N_E]));
    const int b = find_ebin(d, Ec);
    const int up = Ec >= e_center(d, b) ? b + 1 : b;   // the lowest centre at or above Em
    const int jt = min(jin, up + 1);
    if (up < 1 || up > d.N_E - 1 || jt < SM2D_RD_NE - 1) return make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    const float ch = e_center(d, up), cl = e_center(d, up - 1), D = ch - cl;
    for (int e = 0; e < SM2D_RD_NE - 1; ++e) {
        const float de = e_center(d, jt - e) - e_center(d, jt - e - 1);
        if (fabsf(de - D) > 1e-3f * D) return make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    }
    return make_float4(s, fminf(fmaxf((Em - cl) / D, 0.0f), 0.99999994f), sE / D, jt == up ? 1.0f : 0.0f);
}
__device__ __forceinline__ void make_kids(const Dev& d, int c, int jin, float s, float Em, float sE, float w, Kids& k) {
    const int j = kid_window_top(d, jin, Em);
    k.c = c;
    k.j = j;
    k.emax = min(SM2D_RD_NE - 1, j);
    float cen[SM2D_RD_NE];
    for (int e = 0; e <= k.emax; ++e) cen[e] = e_center(d, j - e);
    sm2d_rd_theta(s, k.Mt);
    sm2d_rd_energy(Em, sE, cen, k.emax, k.Me);
    k.Erep = sm2d_rd_fold(w, d.split_min_w, k.Mt, k.Me, cen, k.emax);
    uint32_t live = 0u;
#pragma unroll
    for (int e = 0; e < SM2D_RD_NE; ++e)
#pragma unroll
        for (int t = 0; t < SM2D_RD_NT; ++t)
            if (e <= k.emax && k.Me[e] > 0.0f && k.Mt[t] > 0.0f) live |= 1u << (t + 8 * e);
    k.live = live;
}
// The children from the learned surrogate's table of the component (its
// row of the network's output, T[t + 8 e]; the window is complete, emax 3).
// As in the closed forms (sm2d_rd_fold), an angular distance whose total
// mass (over the energy offsets) is light folds into the centre angle, and
// the represented energy counts each offset's whole mass.
struct KidsT {
    int c, j;
    float T[SM2D_RD_NT * SM2D_RD_NE];
    float Erep;
    uint32_t live;   // bit t + 8 e: T[t + 8 e] > 0
};
__device__ __forceinline__ void make_kids_t(const Dev& d, int c, int jin, float Em, float w, const float* row,
                                            KidsT& k) {
    const int j = kid_window_top(d, jin, Em);
    k.c = c;
    k.j = j;
    const float4* r4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float4 v = __ldcg(r4 + q);
        k.T[4 * q] = fmaxf(v.x, 0.0f); k.T[4 * q + 1] = fmaxf(v.y, 0.0f);
        k.T[4 * q + 2] = fmaxf(v.z, 0.0f); k.T[4 * q + 3] = fmaxf(v.w, 0.0f);
    }
    float Er = 0.0f;
#pragma unroll
    for (int e = 0; e < SM2D_RD_NE; ++e) {
        float me = 0.0f;
#pragma unroll
        for (int t = 0; t < SM2D_RD_NT; ++t) me += k.T[t + 8 * e];
        Er += me * e_center(d, j - e);
    }
    k.Erep = Er;
#pragma unroll
    for (int t = 1; t < SM2D_RD_NT; ++t) {
        float mt = 0.0f;
#pragma unroll
        for (int e = 0; e < SM2D_RD_NE; ++e) mt += k.T[t + 8 * e];
        if (mt > 0.0f && w * mt < d.split_min_w) {
#pragma unroll
            for (int e = 0; e < SM2D_RD_NE; ++e) {
                k.T[8 * e] += k.T[t + 8 * e];
                k.T[t + 8 * e] = 0.0f;
            }
        }
    }
    uint32_t live = 0u;
#pragma unroll
    for (int q = 0; q < SM2D_RD_NT * SM2D_RD_NE; ++q)
        if (k.T[q] > 0.0f) live |= 1u << q;
    k.live = live;
}
// accessors shared by both kinds of children
__device__ __forceinline__ int kid_emax(const Kids& k) { return k.emax; }
__device__ __forceinline__ int kid_emax(const KidsT&) { return SM2D_RD_NE - 1; }
__device__ __forceinline__ bool kid_live(const Kids& k, int t, int e) { return (k.live >> (t + 8 * e)) & 1u; }
__device__ __forceinline__ bool kid_live(const KidsT& k, int t, int e) { return (k.live >> (t + 8 * e)) & 1u; }
__device__ __forceinline__ float kid_weight(const Kids& k, float w, int kk, int e) {
    return sm2d_rd_kid_w(w, k.Mt, k.Me, kk, e);
}
__device__ __forceinline__ float kid_weight(const KidsT& k, float w, int kk, int e) {
    const int t = sm2d_rd_kid_t(kk);
    const float m = k.T[t + 8 * e];
    return w * (t == 0 ? m : m * 0.5f);
}
template <class K>
__device__ __forceinline__ int kid_tbin(const Dev& d, const K& k, int kk) {
    return max(0, min(k.c + sm2d_rd_kid_side(kk) * sm2d_rd_kid_t(kk), d.N_theta - 1));
}
// the children of a component of weight `weight` into one container, in
// child order (the claim key's emission index is the child number)
template <class Lay, int PASS, class K>
__device__ float emit_component(const Dev& d, const Src& src, int par, int bcell, int face, int dcell, int col,
                                const K& kd, float weight, int xs, int zs, Tally& t) {
    if (weight <= 0.0f) return 0.0f;
    float dropped = 0.0f;
    for (int e = 0; e <= kid_emax(kd); ++e) {
        const int Eb = kd.j - e;
        const int El = Eb % Lay::NE;
        const uint32_t bE = (uint32_t)(Eb / Lay::NE);
        for (int k = 0; k < SM2D_RD_KIDS; ++k) {
            if (!kid_live(kd, sm2d_rd_kid_t(k), e)) continue;
            const float wk = kid_weight(kd, weight, k, e);
            if (PASS != PASS_KEYS && wk <= 0.0f) continue;
            const int tb = kid_tbin(d, kd, k);
            const uint32_t want = make_bid((uint32_t)(tb / Lay::NT), bE);
            const int l = Lay::enc(tb % Lay::NT, El, xs, zs);
            dropped += put<Lay, PASS>(d, src, par, bcell, face, dcell, col, 16 * e + k, want, l, wk, t);
        }
    }
    return dropped;
}
// The sampled form plans a component where it is emitted (plan_emission of
// its new angle and energy); the expectation form's children are planned
// once per component.
struct AngleEnergy {
    float theta, E;
};
__device__ __forceinline__ EmitPlan plan_of(const Dev& d, const AngleEnergy& a) { return plan_emission(d, a.theta, a.E); }
__device__ __forceinline__ const Kids& plan_of(const Dev&, const Kids& k) { return k; }
__device__ __forceinline__ const KidsT& plan_of(const Dev&, const KidsT& k) { return k; }
// energy of the re-binned parts of a planned component
__device__ __forceinline__ float plan_erep(const Dev& d, const AngleEnergy&, float E, float w) {
    return bin_energy(d, E, w).Erep;
}
__device__ __forceinline__ float plan_erep(const Dev&, const Kids& k, float, float) { return k.Erep; }
__device__ __forceinline__ float plan_erep(const Dev&, const KidsT& k, float, float) { return k.Erep; }

// +z crossing with the N-cell lateral Gaussian split: the share of column
// ix+k goes through the +z bucket of cell (ix+k, iz) to cell (ix+k, iz+1)
// (device_bucket.cuh:857-987).
template <class Lay, int PASS, class Plan>
__device__ float emit_forward(const Dev& d, const Src& sc, int par, int src, int my_cls, const Plan& pl, float E,
                              float weight, float xoff, float sigma, float& boundary_w, Tally& t) {
    if (weight <= 0.0f) return 0.0f;
    constexpr int N = 11;
    sigma = fmaxf(sigma, 1e-6f);
    {
        // the centre column's edges xmin + 5 dx and xmin + 6 dx, as the loop
        // below computes them: beyond 8 sigma on both sides every CDF value is
        // exactly 0 left of the column and 1 right of it (gauss_cdf), so the
        // weights are exactly (0, .., 1, .., 0) after both normalisations
        const float xmin = xoff - 0.5f * (float)N * d.dx;
        const float dl = (xmin + (float)(N / 2) * d.dx) - xoff, dr = (xmin + (float)(N / 2 + 1) * d.dx) - xoff;
        if (dl < -8.0f * sigma && dr > 8.0f * sigma) {
            if ((src / d.Nx) % d.Nz + 1 >= d.Nz) {
                boundary_w += weight;
                return 0.0f;
            }
            const auto& pk = plan_of(d, pl);
            return emit_component<Lay, PASS>(d, sc, par, src, FACE_ZP, src + d.Nx, N / 2, pk, weight, Lay::NX / 2, 0, t);
        }
    }
    float w[N];
    {
        const float dx = d.dx;
        const float xmin = xoff - 0.5f * (float)N * dx;
        float prev = gauss_cdf(xmin, xoff, sigma);
        for (int i = 0; i < N; ++i) {
            float cur = gauss_cdf(xmin + (float)(i + 1) * dx, xoff, sigma);
            w[i] = cur - prev;
            prev = cur;
        }
        float s = 0.0f;
        for (int i = 0; i < N; ++i) s += w[i];
        if (s > 1e-10f) {
            for (int i = 0; i < N; ++i)
                if (w[i] != 0.0f) w[i] /= s;   // 0 / s is 0: skip the division
        } else {
            for (int i = 0; i < N; ++i) w[i] = (i == N / 2) ? 1.0f : 0.0f;
        }
    }
    float s = 0.0f;
    for (int i = 0; i < N; ++i) { w[i] = fmaxf(0.0f, w[i]); s += w[i]; }
    if (s < 1e-12f) {
        for (int i = 0; i < N; ++i) w[i] = 0.0f;
        w[N / 2] = 1.0f;
    } else {
        for (int i = 0; i < N; ++i)
            if (w[i] != 0.0f) w[i] /= s;
    }
    const int ixs = src % d.Nx, izs = (src / d.Nx) % d.Nz, tz = izs + 1;
    const auto& pk = plan_of(d, pl);
    float dropped = 0.0f;
    for (int i = 0; i < N; ++i) {
        const float wf = w[i];
        if (wf <= 0.0f) continue;
        const int off = i - N / 2;
        const int ixt = ixs + off;
        if (ixt < 0 || ixt >= d.Nx || tz >= d.Nz) { boundary_w += weight * wf; continue; }
        const int ecell = src + off;   // same row of the same lane
        // the bucket of another column exists only if that cell is listed
        // in the same pass (k1k6_pipeline.cu:800-847 maps one list at a time)
        if (ecell != src && d.cls[ecell] != my_cls) {
            if (PASS != PASS_KEYS) count_drop(d.gs, sc.k3, DROP_BUCKET, (double)(weight * wf), (double)(E * (weight * wf)));
            dropped += weight * wf;
            continue;
        }
        const int xt = off < 0 ? Lay::NX - 1 : (off > 0 ? 0 : Lay::NX / 2);
        dropped += emit_component<Lay, PASS>(d, sc, par, ecell, FACE_ZP, ecell + d.Nx, N - 1 - i, pk, weight * wf,
                                             xt, 0, t);
    }
    return dropped;
}

// Component stays in its cell: re-bin angle/energy, spread over the x
// sub-bins, send Gaussian tails past the cell edges to the lateral
// neighbours, fold the re-binning energy error into the deposit
// (k2_coarsetransport.cu:460-690, k3_finetransport.cu:504-747).
template <class Lay, int PASS>
__device__ void emit_stay(const Dev& d, const Src& sc, int par, bool k3, int cell, float theta_new, float E_new,
                          float w_new, float x_new, float z_new, float sig_sub, float sig_cell, Tally& t) {
    const float dx = d.dx, dz = d.dz;
    const float tmin = d.th[0], tmax = d.th[d.N_theta];
    const float dth = (tmax - tmin) / (float)d.N_theta;
    int tbn = (int)((theta_new - tmin) / dth);
    tbn = (int)fmaxf(0.0f, fminf((float)tbn, (float)(d.N_theta - 1)));
    const EParts ep = bin_energy(d, E_new, w_new);
    const int ix = cell % d.Nx;
    const int zst = sub_bin(z_new, dz, Lay::NZ);
    const float lb = -dx * 0.5f, rb = dx * 0.5f;
    const float win = gauss_cdf(rb, x_new, sig_cell) - gauss_cdf(lb, x_new, sig_cell);
    const float wcf = fminf(1.0f, fmaxf(0.0f, win));
    const int outp = par ^ 1;
    float E_emit = ep.Erep;
    if (PASS == PASS_KEYS) {
        for (int ei = 0; ei < ep.n; ++ei) {
            const int Eb = ep.bin[ei];
            const uint32_t want = ((uint32_t)(Eb / Lay::NE) << 12) | ((uint32_t)(tbn / Lay::NT) & 0xFFFu);
            cand_insert(psi_row(d, cell), d.ccount + cell, sc.tag, want, stay_key(sc.k3, sc.slot, sc.lidx, ei),
                        &d.gs->cand_ovf);
        }
        mark_occupied(d, outp, cell);
    } else {
        float w[Lay::NX];
        const float sg = fmaxf(sig_sub, 1e-6f);
        const float dxs = dx / (float)Lay::NX;
        const float xmin = -dx * 0.5f;
        // the sub-bin k holding x_new, with its edges as the loop below
        // computes them: beyond 8 sigma on both sides every CDF value is
        // exactly 0 left of it and 1 right of it, so the weights are exactly
        // the unit vector e_k and their sum 1 (any other k fails the test)
        const int kc = max(0, min((int)floorf((x_new - xmin) / dxs), Lay::NX - 1));
        const bool unit = ((xmin + (float)kc * dxs) - x_new < -8.0f * sg) &&
                          ((xmin + (float)(kc + 1) * dxs) - x_new > 8.0f * sg);
        if (unit) {
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) w[i] = (i == kc) ? 1.0f : 0.0f;
        } else {
            float prev = gauss_cdf(xmin, x_new, sg);
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) {
                float cur = gauss_cdf(xmin + (float)(i + 1) * dxs, x_new, sg);
                w[i] = cur - prev;
                prev = cur;
            }
            float s = 0.0f;
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) s += w[i];
            if (s > 1e-10f) {
#pragma unroll
                for (int i = 0; i < Lay::NX; ++i)
                    if (w[i] != 0.0f) w[i] /= s;
            } else {
#pragma unroll
                for (int i = 0; i < Lay::NX; ++i) w[i] = (i == Lay::NX / 2) ? 1.0f : 0.0f;
            }
        }
        float wsum = 0.0f;
#pragma unroll
        for (int i = 0; i < Lay::NX; ++i) { w[i] = fmaxf(0.0f, w[i]); wsum += w[i]; }
        if (wsum < 1e-12f) {
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) w[i] = 0.0f;
            w[Lay::NX / 2] = 1.0f;
            wsum = 1.0f;
        }
        const uint32_t* kept = d.bid + (size_t)cell * kKb;
        const size_t pg0 = page_of<true>(d, cell, 0);   // the cell's psi_out pages
        float* vals = d.val + pg0 * Lay::L;
        for (int ei = 0; ei < ep.n; ++ei) {
            const int Eb = ep.bin[ei];
            const uint32_t want = ((uint32_t)(Eb / Lay::NE) << 12) | ((uint32_t)(tbn / Lay::NT) & 0xFFFu);
            uint32_t sel;
            const int os = resolve<true>(d, psi_row(d, cell), kept, sc.tag, want, sel);
            const float wpart = d.esplit ? w_new * ep.frac[ei] : w_new;
            if (os < 0) {
                t.drop_w += (double)wpart;
                t.drop_e += (double)(E_new * wpart);
                count_drop(d.gs, sc.k3, DROP_SLOT, (double)wpart, (double)(E_new * wpart));
                if (!d.esplit) return;
                continue;
            }
            int tbe = tbn, Ebe = Eb;
            if (sel != want) {
                const int t0 = (int)(sel & 0xFFFu) * Lay::NT, e0 = (int)((sel >> 12) & 0xFFFu) * Lay::NE;
                tbe = max(t0, min(tbe, t0 + Lay::NT - 1));
                Ebe = max(e0, min(Ebe, e0 + Lay::NE - 1));
            }
            if (!d.esplit) E_emit = e_center(d, Ebe);
            else if (Ebe != Eb) t.edep += (double)((e_center(d, Eb) - e_center(d, Ebe)) * wpart * wcf);
            const int tl = tbe % Lay::NT, El = Ebe % Lay::NE;
            float* vs = vals + (size_t)os * Lay::L;
            VBits vb;
#pragma unroll
            for (int xs = 0; xs < Lay::NX; ++xs) {
                if (w[xs] <= 0.0f) continue;   // its share would be 0
                const float wf = (w[xs] / wsum) * wcf;
                if (wf <= 0.0f) continue;
                const float ws = wpart * wf;
                const int l = Lay::enc(tl, El, xs, zst);
                atomicAdd(vs + l, ws);
                vb.add(l);
            }
            vb.flush(d, pg0 + os);
        }
    }
    float wl = 0.0f, wr = 0.0f;
    if (wcf < 1.0f - 1e-6f) {
        const EmitPlan pl = plan_emission(d, theta_new, E_new);
        const float wlr = fmaxf(0.0f, gauss_cdf(lb, x_new, sig_cell));
        const float wrr = fmaxf(0.0f, 1.0f - gauss_cdf(rb, x_new, sig_cell));
        const float tt = fmaxf(0.0f, 1.0f - wcf);
        const float ts = wlr + wrr;
        if (tt > 0.0f && ts > 1e-12f) {
            const float sc_ = tt / ts;
            wl = wlr * sc_;
            wr = wrr * sc_;
        }
        if (wl > 0.0f) {
            const float ws = w_new * wl;
            if (ix > 0) {
                const float dr = emit_component<Lay, PASS>(d, sc, par, cell, FACE_XM, cell - 1, 5, pl, ws, Lay::NX - 1,
                                                           zst, t);
                if (dr > 0.0f) { t.drop_w += (double)dr; t.drop_e += (double)(E_new * dr); }
            } else {
                t.w_bnd += ws;
                t.e_bnd += (double)(E_new * ws);
            }
        }
        if (wr > 0.0f) {
            const float ws = w_new * wr;
            if (ix < d.Nx - 1) {
                const float dr = emit_component<Lay, PASS>(d, sc, par, cell, FACE_XP, cell + 1, 5, pl, ws, 0, zst, t);
                if (dr > 0.0f) { t.drop_w += (double)dr; t.drop_e += (double)(E_new * dr); }
            } else {
                t.w_bnd += ws;
                t.e_bnd += (double)(E_new * ws);
            }
        }
    }
    if (PASS != PASS_KEYS && (k3 || d.esplit)) {
        float rf = wcf;
        if (ix > 0) rf += wl;
        if (ix < d.Nx - 1) rf += wr;
        rf = fminf(1.0f, fmaxf(0.0f, rf));
        const float rw = w_new * rf;
        if (rw > 0.0f) t.edep += (double)((E_new - E_emit) * rw);
    }
}

// Expectation form of emit_stay: the component's children stay in the cell,
// each spread over the x sub-bins as emit_stay spreads a component; the
// Gaussian tails past the cell edges go to the lateral neighbours as
// children; the difference between the step's mean energy and the
// children's represented energy is folded into the deposit.
template <class Lay, int PASS, class K>
__device__ void emit_stay_kids(const Dev& d, const Src& sc, int par, int cell, const K& kd, float E_new,
                               float w_new, float x_new, float z_new, float sig_sub, float sig_cell, Tally& t) {
    const float dx = d.dx, dz = d.dz;
    const int ix = cell % d.Nx;
    const int zst = sub_bin(z_new, dz, Lay::NZ);
    const float lb = -dx * 0.5f, rb = dx * 0.5f;
    const float win = gauss_cdf(rb, x_new, sig_cell) - gauss_cdf(lb, x_new, sig_cell);
    const float wcf = fminf(1.0f, fmaxf(0.0f, win));
    if (PASS == PASS_KEYS) {
        for (int e = 0; e <= kid_emax(kd); ++e) {
            const uint32_t bE = (uint32_t)((kd.j - e) / Lay::NE);
            for (int k = 0; k < SM2D_RD_KIDS; ++k) {
                if (!kid_live(kd, sm2d_rd_kid_t(k), e)) continue;
                const uint32_t want = make_bid((uint32_t)(kid_tbin(d, kd, k) / Lay::NT), bE);
                cand_insert(psi_row(d, cell), d.ccount + cell, sc.tag, want, stay_key(sc.k3, sc.slot, sc.lidx, 16 * e + k),
                            &d.gs->cand_ovf);
            }
        }
        mark_occupied(d, par ^ 1, cell);
    } else {
        float w[Lay::NX];
        const float sg = fmaxf(sig_sub, 1e-6f);
        const float dxs = dx / (float)Lay::NX;
        const float xmin = -dx * 0.5f;
        const int kc = max(0, min((int)floorf((x_new - xmin) / dxs), Lay::NX - 1));
        const bool unit = ((xmin + (float)kc * dxs) - x_new < -8.0f * sg) &&
                          ((xmin + (float)(kc + 1) * dxs) - x_new > 8.0f * sg);
        if (unit) {
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) w[i] = (i == kc) ? 1.0f : 0.0f;
        } else {
            float prev = gauss_cdf(xmin, x_new, sg);
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) {
                float cur = gauss_cdf(xmin + (float)(i + 1) * dxs, x_new, sg);
                w[i] = cur - prev;
                prev = cur;
            }
            float s = 0.0f;
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) s += w[i];
            if (s > 1e-10f) {
#pragma unroll
                for (int i = 0; i < Lay::NX; ++i)
                    if (w[i] != 0.0f) w[i] /= s;
            } else {
#pragma unroll
                for (int i = 0; i < Lay::NX; ++i) w[i] = (i == Lay::NX / 2) ? 1.0f : 0.0f;
            }
        }
        float wsum = 0.0f;
#pragma unroll
        for (int i = 0; i < Lay::NX; ++i) { w[i] = fmaxf(0.0f, w[i]); wsum += w[i]; }
        if (wsum < 1e-12f) {
#pragma unroll
            for (int i = 0; i < Lay::NX; ++i) w[i] = 0.0f;
            w[Lay::NX / 2] = 1.0f;
            wsum = 1.0f;
        }
        const uint32_t* kept = d.bid + (size_t)cell * kKb;
        const size_t pg0 = page_of<true>(d, cell, 0);   // the cell's psi_out pages
        float* vals = d.val + pg0 * Lay::L;
        for (int e = 0; e <= kid_emax(kd); ++e) {
            const int Eb = kd.j - e;
            const uint32_t bE = (uint32_t)(Eb / Lay::NE);
            for (int k = 0; k < SM2D_RD_KIDS; ++k) {
                if (!kid_live(kd, sm2d_rd_kid_t(k), e)) continue;
                const float wk = kid_weight(kd, w_new, k, e);
                if (wk <= 0.0f) continue;
                const int tbn = kid_tbin(d, kd, k);
                const uint32_t want = make_bid((uint32_t)(tbn / Lay::NT), bE);
                uint32_t sel;
                const int os = resolve<true>(d, psi_row(d, cell), kept, sc.tag, want, sel);
                if (os < 0) {
                    t.drop_w += (double)wk;
                    t.drop_e += (double)(E_new * wk);
                    count_drop(d.gs, sc.k3, DROP_SLOT, (double)wk, (double)(E_new * wk));
                    continue;
                }
                int tbe = tbn, Ebe = Eb;
                if (sel != want) {
                    const int t0 = (int)(sel & 0xFFFu) * Lay::NT, e0 = (int)((sel >> 12) & 0xFFFu) * Lay::NE;
                    tbe = max(t0, min(tbe, t0 + Lay::NT - 1));
                    Ebe = max(e0, min(Ebe, e0 + Lay::NE - 1));
                }
                if (Ebe != Eb) t.edep += (double)((e_center(d, Eb) - e_center(d, Ebe)) * wk * wcf);
                const int tl = tbe % Lay::NT, El = Ebe % Lay::NE;
                float* vs = vals + (size_t)os * Lay::L;
                VBits vb;
#pragma unroll
                for (int xs = 0; xs < Lay::NX; ++xs) {
                    if (w[xs] <= 0.0f) continue;
                    const float wf = (w[xs] / wsum) * wcf;
                    if (wf <= 0.0f) continue;
                    const int l = Lay::enc(tl, El, xs, zst);
                    atomicAdd(vs + l, wk * wf);
                    vb.add(l);
                }
                vb.flush(d, pg0 + os);
            }
        }
    }
    float wl = 0.0f, wr = 0.0f;
    if (wcf < 1.0f - 1e-6f) {
        const float wlr = fmaxf(0.0f, gauss_cdf(lb, x_new, sig_cell));
        const float wrr = fmaxf(0.0f, 1.0f - gauss_cdf(rb, x_new, sig_cell));
        const float tt = fmaxf(0.0f, 1.0f - wcf);
        const float ts = wlr + wrr;
        if (tt > 0.0f && ts > 1e-12f) {
            const float sc_ = tt / ts;
            wl = wlr * sc_;
            wr = wrr * sc_;
        }
        if (wl > 0.0f) {
            const float ws = w_new * wl;
            if (ix > 0) {
                const float dr = emit_component<Lay, PASS>(d, sc, par, cell, FACE_XM, cell - 1, 5, kd, ws, Lay::NX - 1,
                                                           zst, t);
                if (dr > 0.0f) { t.drop_w += (double)dr; t.drop_e += (double)(E_new * dr); }
            } else {
                t.w_bnd += ws;
                t.e_bnd += (double)(E_new * ws);
            }
        }
        if (wr > 0.0f) {
            const float ws = w_new * wr;
            if (ix < d.Nx - 1) {
                const float dr = emit_component<Lay, PASS>(d, sc, par, cell, FACE_XP, cell + 1, 5, kd, ws, 0, zst, t);
                if (dr > 0.0f) { t.drop_w += (double)dr; t.drop_e += (double)(E_new * dr); }
            } else {
                t.w_bnd += ws;
                t.e_bnd += (double)(E_new * ws);
            }
        }
    }
    if (PASS != PASS_KEYS) {
        float rf = wcf;
        if (ix > 0) rf += wl;
        if (ix < d.Nx - 1) rf += wr;
        rf = fminf(1.0f, fmaxf(0.0f, rf));
        const float rw = w_new * rf;
        if (rw > 0.0f) t.edep += (double)((E_new - kd.Erep) * rw);
    }
}

// Component crosses `face` (k2_coarsetransport.cu:363-459, k3_finetransport.cu:380-503);
// pl: plan_emission of its new angle and energy, or its children (expectation form).
template <class Lay, int PASS, class Plan>
__device__ void emit_cross(const Dev& d, const Src& sc, int par, bool k3, int cell, int my_cls, int face,
                           const Plan& pl, float E_new, float w_new, float x_new, float z_new, float sig_tr, Tally& t) {
    const int ix = cell % d.Nx, iz = (cell / d.Nx) % d.Nz;
    int nb = -1;
    if (face == FACE_ZP) nb = iz + 1 < d.Nz ? cell + d.Nx : -1;
    else if (face == FACE_ZM) nb = iz > 0 ? cell - d.Nx : -1;
    else if (face == FACE_XP) nb = ix + 1 < d.Nx ? cell + 1 : -1;
    else nb = ix > 0 ? cell - 1 : -1;
    if (nb < 0) {
        t.w_bnd += w_new;
        t.e_bnd += (double)(E_new * w_new);
        return;
    }
    const float E_emit = plan_erep(d, pl, E_new, w_new);
    const bool fold = PASS != PASS_KEYS && (k3 || d.esplit);
    if (face == FACE_ZP) {
        float lbw = 0.0f;
        const float dr = emit_forward<Lay, PASS>(d, sc, par, cell, my_cls, pl, E_new, w_new, x_new, sig_tr, lbw, t);
        if (lbw > 0.0f) { t.w_bnd += lbw; t.e_bnd += (double)(E_new * lbw); }
        if (dr > 0.0f) { t.drop_w += (double)dr; t.drop_e += (double)(E_new * dr); }
        if (fold) {
            const float tw = fmaxf(0.0f, w_new - lbw - dr);
            if (tw > 0.0f) t.edep += (double)((E_new - E_emit) * tw);
        }
        return;
    }
    const float dx = d.dx, dz = d.dz;
    const float xo = face == FACE_XP ? -dx * 0.5f : (face == FACE_XM ? dx * 0.5f : x_new);
    const int xsn = sub_bin(xo, dx, Lay::NX);
    const int zsn = face == FACE_ZM ? Lay::NZ - 1 : sub_bin(z_new, dz, Lay::NZ);
    const float dr = emit_component<Lay, PASS>(d, sc, par, cell, face, nb, 5, plan_of(d, pl), w_new, xsn, zsn, t);
    if (dr > 0.0f) { t.drop_w += (double)dr; t.drop_e += (double)(E_new * dr); }
    if (fold) {
        const float tw = fmaxf(0.0f, w_new - dr);
        if (tw > 0.0f) t.edep += (double)((E_new - E_emit) * tw);
    }
}

__device__ __forceinline__ int exit_face(float x, float z, float dx, float dz) {
    const float eps = 0.001f, hz = dz * 0.5f, hx = dx * 0.5f;
    if (z >= hz - eps) return FACE_ZP;
    if (z <= -hz + eps) return FACE_ZM;
    if (x >= hx - eps) return FACE_XP;
    if (x <= -hx + eps) return FACE_XM;
    return -1;
}

// One component of a listed cell gc of lane ln (lane-local index lc, which
// the random seeds use): local bin lidx of psi_in slot `slot` (sslot: the slot number
// the seeds use), entry bi of the bin list.  par selects the occupancy list
// of psi_out (par ^ 1).  The claim pass stores the step's outcome (new angle,
// energy, weight, raw position, lateral sigma, deposit, nuclear loss) in the
// bin's record; the deposit pass reads it back instead of repeating the
// physics, so both passes emit the same arithmetic's results.
//
// With the learned surrogate (expectation form, d.surr): the claim pass gives
// a K3 bin inside the network's domain a row of the surrogate's tables and
// emits no claims for it; after the network has run, the rows' claim pass
// (from_rec: the step's outcome from the record) and the deposit pass emit
// the bin's children from its row's table, or from the closed forms where
// the row fell back.
template <class Lay, int PASS, bool EXP>
__device__ void transport_bin(const Dev& d, int bi, int par, bool k3, int cell, int ln, int lc, uint32_t bid, int slot,
                              int sslot, int lidx, float w, unsigned salt, uint32_t tag, Tally& t,
                              bool from_rec = false) {
    const float dx = d.dx, dz = d.dz;
    int tl, El, xs, zs;
    Lay::dec(lidx, tl, El, xs, zs);
    int tbin = (int)(bid & 0xFFFu) * Lay::NT + tl;
    int Ebin = (int)((bid >> 12) & 0xFFFu) * Lay::NE + El;
    if (k3) {
        tbin = max(0, min(tbin, d.N_theta - 1));
        Ebin = max(0, min(Ebin, d.N_E - 1));
    }
    const float E = d.Ee[Ebin] + 1.0f * ((d.Ee[Ebin + 1] - d.Ee[Ebin]) * 0.5f);
    // the bins' weight and energy, the step's deposit and nuclear loss are
    // summed per cell by the tally kernel from the bin list and the step
    // records; the claim pass adds nothing either
    (void)t;
    if (w < (k3 ? d.prune_fine : d.prune_coarse)) {   // prune (k3:175-184, k2:172-177)
        t.drop_w += (double)w;
        t.drop_e += (double)(E * w);   // counted per cell by the tally (tally_cell)
        return;
    }
    const float tmin = d.th[0], tmax = d.th[d.N_theta];
    const float dth = (tmax - tmin) / (float)d.N_theta;
    const float theta = k3 ? d.th[tbin] + 0.5f * dth : tmin + ((float)tbin + 0.5f) * dth;
    if (E <= 0.1f) {
        t.w_cut += w;
        t.e_cut += (double)(E * w);
        return;
    }
    const float hx = dx * 0.5f, hz = dz * 0.5f;
    float theta_new, x_new, z_new, E_new, w_new, edep, w_rem = 0.0f, sigv;
    float s_th = 0.0f, s_E = 0.0f;   // expectation form: sigma_theta / dtheta, straggling sigma
    float4* rec = reinterpret_cast<float4*>(d.brec + 2 * (size_t)bi);
    int srow = -1;   // the bin's row of the surrogate's tables
    if (PASS != PASS_KEYS || (EXP && from_rec)) {
        const float4 r0 = __ldcs(rec), r1 = __ldcs(rec + 1);
        theta_new = r0.x; E_new = r0.y; w_new = r0.z; x_new = r0.w;
        z_new = r1.x; sigv = r1.y; edep = r1.z; w_rem = r1.w;
        if (EXP) {
            const float4 r2 = __ldcs(d.brec2 + bi);
            s_th = r2.x;
            s_E = r2.y;
            srow = __float_as_int(r2.z);
        }
    } else {
    const float xc = sub_offset(xs, Lay::NX, dx), zc = sub_offset(zs, Lay::NZ, dz);
    const int iz = lc / d.Nx;
    // slab phantom: paths below are geometric; energy loss, range limits,
    // straggling, nuclear attenuation and scattering thickness take the
    // water-equivalent path rho * step (rho = 1: the water arithmetic)
    const float rho = d.rho ? d.rho[iz] : 1.0f;
    float step, dE, sig_th, sig_x;
    unsigned ts;
    if (k3) {
        // K3_FineTransport body, k3_finetransport.cu:226-366
        const float mu0 = sm2d_cosf(theta), eta0 = sm2d_sinf(theta);
        const float szp = (mu0 > 0) ? (hz - zc) / mu0 : 1e30f;
        const float szm = (mu0 < 0) ? (-hz - zc) / mu0 : 1e30f;
        const float sxp = (eta0 > 0) ? (hx - xc) / eta0 : 1e30f;
        const float sxm = (eta0 < 0) ? (-hx - xc) / eta0 : 1e30f;
        const float sb = fmaxf(fminf(fminf(szp, szm), fminf(sxp, sxm)), 0.0f);
        const float RE = d.k2tab ? __ldg(d.k2tab + Ebin).x : lut_range(d, E);   // Ebin is clamped here
        step = fminf(fine_step_limit(E, RE) / rho, sb * 1.001f);
        const float mean_dE = lut_energy_loss(d, E, RE, rho * step);
        if (EXP) {   // the straggling distribution instead of a draw
            dE = mean_dE;
            s_E = d.straggle ? straggling_sigma(E, step, rho) : 0.0f;
        } else if (d.straggle) {
            unsigned seed = ((unsigned)(lc * 7 + sslot * 13 + lidx * 17) ^ 0xDEECE66Du) ^ salt;
            const float sE = straggling_sigma(E, step, rho);
            dE = sE <= 0.0f ? mean_dE : fmaxf(mean_dE + normal_draw(seed) * sE, 0.0f);
        } else {
            dE = mean_dE;
        }
        dE = fminf(dE, E);
        E_new = E - dE;
        edep = dE * w;
        w_new = w;
        if (d.nuclear) {
            const float surv = sm2d_expf(-nuclear_xs(E) * (rho * step));
            w_new = w * surv;
            w_rem = w - w_new;
        }
        const float sm = fmaxf(step, 0.0f);
        const float Ap = iz < d.Nz ? d.feA[(size_t)ln * d.Nz + iz] : 0.0f;
        const float Bp = iz < d.Nz ? d.feB[(size_t)ln * d.Nz + iz] : 0.0f;
        const float T = scatter_power(fmaxf(E - 0.5f * dE, d.lutEmin), sm, rho);
        sig_th = sqrtf(fmaxf(T * sm, 0.0f));
        const float dC = fmaxf(2.0f * Bp * sm + Ap * sm * sm + T * sm * sm * sm / 3.0f, 0.0f);
        sig_x = fmaxf(sqrtf(dC), 0.01f);
        const unsigned ps = (unsigned)fminf((float)iz * dz * 1000.0f, 4294967295.0f);
        ts = ((unsigned)(lc + 1) * 2654435761u) ^ ((unsigned)(sslot + 1) * 2246822519u) ^
             ((unsigned)(lidx + 1) * 3266489917u) ^ (unsigned)(Ebin + 17) ^ (ps * 747796405u) ^ salt;
    } else {
        // K2_CoarseTransport body, k2_coarsetransport.cu:186-350
        float lim = fminf(d.step_coarse, fminf(dx, dz));
        float rs = lim;
        bool split = false;
        // the table's values are this arithmetic's: the range for any row, the
        // rest for a density-1 row whose step does not split
        const bool inr = d.k2tab && Ebin < d.N_E;
        const bool tab = inr && rho == 1.0f;
        const float4 q = inr ? __ldg(d.k2tab + Ebin) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float RE = inr ? q.x : lut_range(d, E);
        if (E > d.E_fine_on + 1e-6f) {
            const float rtf = (RE - d.R_fine_on) / rho;   // geometric distance to the fine threshold
            if (rtf > 0.0f && rtf < rs) { rs = rtf; lim = rs; split = true; }
        }
        step = lim;
        const bool use = tab && !split;
        dE = use ? q.y : fminf(lut_energy_loss(d, E, RE, rho * rs), E);
        E_new = E - dE;
        edep = dE * w;
        const float surv = use ? q.z : sm2d_expf(-nuclear_xs(E) * (rho * rs));
        w_new = w * surv;
        w_rem = w - w_new;
        if (split && E_new > d.E_fine_on) {
            const float ex = E_new - d.E_fine_on;
            if (ex > 0.0f && w_new > 0.0f) edep += ex * w_new;
            E_new = d.E_fine_on;
        }
        const float p0 = fmaxf(0.0f, (float)iz * dz + (zc + 0.5f * dz));
        // scattering accumulated over the water-equivalent depth
        const float p0w = d.rho ? fmaxf(0.0f, d.wet[iz] + rho * (zc + 0.5f * dz)) : p0;
        const float sm = fmaxf(rs, 0.0f);
        const float s0 = p0 > 0.0f ? highland(E, p0w) : 0.0f;
        const float A0 = s0 * s0;
        const float B0 = 0.5f * A0 * p0;
        const float sx0 = d.sx0[ln];
        const float C0 = sx0 * sx0 + (A0 * p0 * p0) / 3.0f;
        const float T = use ? q.w : scatter_power(fmaxf(E - 0.5f * dE, d.lutEmin), sm, rho);
        const float A1 = fmaxf(A0 + T * sm, 0.0f);
        const float C1 = fmaxf(C0 + 2.0f * B0 * sm + A0 * sm * sm + (1.0f / 3.0f) * T * sm * sm * sm, 0.0f);
        sig_th = sqrtf(fmaxf(A1 - A0, 0.0f));
        const float dC = fmaxf(C1 - C0, 0.0f);
        const float uf = fminf(0.35f, 0.04f + 0.003f * p0);
        sig_x = fmaxf(sqrtf(fmaxf(dC + uf * C0, 0.0f)), 0.01f);
        const unsigned ps = (unsigned)fminf(p0 * 1000.0f, 4294967295.0f);
        ts = ((unsigned)(lc + 1) * 2654435761u) ^ ((unsigned)(sslot + 1) * 2246822519u) ^
             ((unsigned)(lidx + 1) * 3266489917u) ^ (unsigned)(Ebin + 17) ^ (ps * 747796405u) ^ salt;
    }
    float scat = 0.0f;
    if (EXP) s_th = sig_th / dth;   // the MCS distribution instead of a draw: geometry along theta
    else scat = sig_th <= 0.0f ? 0.0f : normal_draw(ts) * sig_th;
    theta_new = fmaxf(d.th[0], fminf(theta + scat, d.th[d.N_theta]));
    x_new = xc + sm2d_sinf(theta_new) * step;
    z_new = zc + sm2d_cosf(theta_new) * step;
    sigv = exit_face(x_new, z_new, dx, dz) >= 0
               ? (k3 ? 0.001f : fmaxf(sm2d_sinf(fminf(sig_th, 1.57f)) * fmaxf(step, 0.0f) / 1.7320508f, 0.01f))
               : sig_x;
    __stcg(rec, make_float4(theta_new, E_new, w_new, x_new));
    __stcg(rec + 1, make_float4(z_new, sigv, edep, w_rem));
    if (EXP) {
        // a K3 bin that stays above the cutoff with features inside the
        // network's domain gets a row of the surrogate's tables
        float4 q = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        if (d.surr && k3 && E_new > 0.1f && E_new > e_center(d, 0))
            q = surr_features(d, max(0, min(Ebin, d.N_E - 1)), s_th, E_new, s_E);
        if (q.w >= 0.0f) {
            const int row = atomicAdd(&d.gs->k3_rows, 1);
            if (row < d.k3_cap) {
                d.kfeat[row] = q;
                d.kbin[row] = bi;
                srow = row;
            } else {
                atomicAdd(&d.gs->k3_ovf, 1);
            }
        }
        __stcg(d.brec2 + bi, make_float4(s_th, s_E, __int_as_float(srow), 0.0f));
        if (srow >= 0) return;   // its claims follow the network (the rows' claim pass)
    }
    }
    const int face = exit_face(x_new, z_new, dx, dz);
    x_new = fmaxf(-hx, fminf(x_new, hx));
    z_new = fmaxf(-hz, fminf(z_new, hz));
    (void)edep;
    (void)w_rem;
    if (E_new <= 0.1f || ((d.esplit || d.floor_cutoff) && E_new <= e_center(d, 0))) {
        t.w_cut += w_new;
        t.e_cut += (double)(E_new * w_new);
        return;
    }
    const int my_cls = k3 ? 2 : 1;
    const Src sc{cell, slot, lidx, k3 ? 1 : 0, tag, E_new};
    if (EXP) {
        const int c0 = max(0, min(tbin, d.N_theta - 1)), j0 = max(0, min(Ebin, d.N_E - 1));
        // the surrogate's table where the network served the bin's row (the
        // rows' claim pass and the deposit pass), else the closed forms
        if (srow >= 0 && __ldcg(d.kfb + srow) == 0) {
            KidsT kt;
            make_kids_t(d, c0, j0, E_new, w_new, d.ktab + (size_t)srow * (SM2D_RD_NT * SM2D_RD_NE), kt);
            if (face >= 0)
                emit_cross<Lay, PASS>(d, sc, par, k3, cell, my_cls, face, kt, E_new, w_new, x_new, z_new, sigv, t);
            else
                emit_stay_kids<Lay, PASS>(d, sc, par, cell, kt, E_new, w_new, x_new, z_new, k3 ? 0.001f : sigv, sigv,
                                          t);
            return;
        }
        Kids kd;
        make_kids(d, c0, j0, s_th, E_new, s_E, w_new, kd);
        if (face >= 0)
            emit_cross<Lay, PASS>(d, sc, par, k3, cell, my_cls, face, kd, E_new, w_new, x_new, z_new, sigv, t);
        else
            emit_stay_kids<Lay, PASS>(d, sc, par, cell, kd, E_new, w_new, x_new, z_new, k3 ? 0.001f : sigv, sigv, t);
        return;
    }
    if (face >= 0) {
        emit_cross<Lay, PASS>(d, sc, par, k3, cell, my_cls, face, AngleEnergy{theta_new, E_new}, E_new, w_new, x_new,
                              z_new, sigv, t);
    } else {
        emit_stay<Lay, PASS>(d, sc, par, k3, cell, theta_new, E_new, w_new, x_new, z_new, k3 ? 0.001f : sigv, sigv, t);
    }
}

}  // namespace sm2d
