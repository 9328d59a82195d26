// sm2d_engine.cu -- kernels, device-resident iteration loop and C ABI of the
// SM_2D transport step on GB300 (sm_103a).
//
// One iteration (the body of the reference host loop k1k6_pipeline.cu:1606-2038)
// is four kernels that read every count from device memory:
//   k_classify   K1 active mask + per-block list counts (warp per occupied cell)
//   k_compact    ordered active/coarse lists, iteration bookkeeping, loop condition
//   k_transport  K2/K3 for every listed cell, warp per cell, with the K4 scatter
//                fused (direct mode) or written to DeviceOutflowBucket (bucket mode,
//                then k_bucket_gather = K4_BucketTransfer)
//   k_audit      K5 audit of the iteration, clear of the consumed buffer, K6 swap
// sm2d_run captures that body once into a CUDA graph whose while-conditional
// node repeats it on the device until no cell holds weight.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sm2d.h"
#include "sm2d_common.cuh"
#include "sm2d_device.cuh"
#include "sm2d_tables.h"
#include "sm2d_transport.cuh"

namespace sm2d {

// ------------------------------------------------------------------ injection
// LCG/Box-Muller of the source kernel (k1k6_pipeline.cu:433-447)
__device__ __forceinline__ float source_normal(unsigned& s) {
    s = 1664525u * s + 1013904223u;
    const float u1 = (float)(s >> 16) / 65536.0f;
    s = 1664525u * s + 1013904223u;
    const float u2 = (float)(s >> 16) / 65536.0f;
    const float r = sqrtf(-2.0f * logf(fmaxf(u1, 1e-10f)));
    const float th = (float)(2.0 * 3.14159265358979323846 * (double)u2);
    return r * cosf(th);
}

struct BeamArgs {
    float x0, z0, theta0, E0, W, sx, sth, sE, x_min, z_min;
    int n;
    unsigned seed;
};

// One source sample: inject_source_kernel's pencil branch
// (k1k6_pipeline.cu:325-343) or sample i of inject_gaussian_source_kernel
// (k1k6_pipeline.cu:451-551), placed as device_psic_inject_source does
// (device_psic.cuh:347-450: clamp into the cell, sub-cell bins, nearest
// global bins).  Returns false when the sample leaves the grid.
struct InjSample {
    int cell, l;
    uint32_t want;
    float w, E;
};
template <class Lay>
__device__ bool inject_sample(const Dev& d, const BeamArgs& b, int gaussian, int i, InjSample& o) {
    float theta, E, x, z;
    if (!gaussian) {
        const float xr = b.x0 - b.x_min, zr = b.z0 - b.z_min;
        int cx = (int)(xr / d.dx), cz = (int)(zr / d.dz);
        cx = cx < 0 ? 0 : (cx >= d.Nx ? d.Nx - 1 : cx);
        cz = cz < 0 ? 0 : (cz >= d.Nz ? d.Nz - 1 : cz);
        o.cell = cz * d.Nx + cx;
        theta = b.theta0;
        E = b.E0;
        o.w = b.W;
        x = xr - cx * d.dx;
        z = zr - cz * d.dz;
    } else {
        unsigned s = b.seed + (unsigned)i;
        const float xs = b.x0 + b.sx * source_normal(s);
        float ts = b.theta0 + b.sth * source_normal(s);
        float Es = b.E0 + b.sE * source_normal(s);
        Es = fmaxf(d.Ee[0], fminf(Es, d.Ee[d.N_E]));
        ts = fmaxf(d.th[0], fminf(ts, d.th[d.N_theta]));
        const float xr = xs - b.x_min, zr = b.z0 - b.z_min;
        const int ix = (int)(xr / d.dx), iz = (int)(zr / d.dz);
        o.w = b.W / b.n;
        o.E = Es;
        if (ix < 0 || ix >= d.Nx || iz < 0 || iz >= d.Nz) return false;
        o.cell = iz * d.Nx + ix;
        theta = ts;
        E = Es;
        x = xr - ix * d.dx;
        z = zr - iz * d.dz;
    }
    o.E = E;
    const float dx = d.dx, dz = d.dz;
    x = fmaxf(0.0f, fminf(x, dx));
    z = fmaxf(0.0f, fminf(z, dz));
    const int xs = sub_bin(x - dx * 0.5f, dx, Lay::NX), zs = sub_bin(z - dz * 0.5f, dz, Lay::NZ);
    const float tmin = d.th[0], tmax = d.th[d.N_theta];
    theta = fmaxf(tmin, fminf(theta, tmax));
    E = fmaxf(d.Ee[0], fminf(E, d.Ee[d.N_E]));
    const float cont = (theta - tmin) / ((tmax - tmin) / (float)d.N_theta);
    int tb = (int)cont;
    float ft = cont - (float)tb;
    int Eb = find_bin(d.Ee, d.N_E, E);
    const float lo = d.Ee[Eb], hi = d.Ee[Eb + 1];
    float fE = (hi - lo) > 1e-10f ? (E - lo) / (hi - lo) : 0.0f;
    if (tb >= d.N_theta - 1) { tb = d.N_theta - 1; ft = 0.0f; }
    if (Eb >= d.N_E - 1) { Eb = d.N_E - 1; fE = 0.0f; }
    if (ft >= 0.5f && tb < d.N_theta - 1) tb++;
    if (fE >= 0.5f && Eb < d.N_E - 1) Eb++;
    o.want = make_bid((uint32_t)(tb / Lay::NT), (uint32_t)(Eb / Lay::NE));
    o.l = Lay::enc(tb % Lay::NT, Eb % Lay::NE, xs, zs);
    return true;
}

// Opens an injection: one claim pass, refused (every sample booked as a
// source slot drop) when psi_in is not empty.
__global__ void k_inject_begin(IterState* it) {
    if (threadIdx.x || blockIdx.x) return;
    it->ctag += 1u;
    it->inj_skip = it->occ_n[it->parity] != 0 ? 1 : 0;
}

// Claim pass of the injection: each in-grid sample offers its block to its
// cell with its sample index as claim key.
template <class Lay>
__global__ void k_inject_keys(Dev d, const BeamArgs* bp, int gaussian) {
    const BeamArgs b = *bp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (gaussian ? b.n : 1) || d.it->inj_skip) return;
    InjSample o;
    if (!inject_sample<Lay>(d, b, gaussian, i, o) || !(o.w > 0.0f)) return;
    cand_insert(psi_row(d, o.cell), d.ccount + o.cell, d.it->ctag, o.want, (uint32_t)i, &d.it->cand_ovf);
    mark_occupied(d, d.it->parity, o.cell);
}

// Deposit pass of the injection: a sample whose block kept a slot adds its
// weight there; the others are source slot drops (the reference's claim
// without fallback).
template <class Lay>
__global__ void k_inject_deposit(Dev d, const BeamArgs* bp, int gaussian) {
    const BeamArgs b = *bp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (gaussian ? b.n : 1)) return;
    IterState* it = d.it;
    InjSample o;
    const bool in = inject_sample<Lay>(d, b, gaussian, i, o);
    if (!gaussian) {   // the pencil books W and E0 W in k_source_finalize
        if (in && !it->inj_skip && o.w > 0.0f) {
            const int s = cand_find(psi_row(d, o.cell), it->ctag, o.want);
            if (s >= 0 && d.bid[it->parity][(size_t)o.cell * kKb + s] == o.want)
                atomicAdd(d.val[it->parity] + ((size_t)o.cell * kKb + s) * Lay::L + o.l, o.w);
        }
        return;
    }
    if (!in) {
        atomicAdd(&it->src_oog_w, o.w);
        atomicAdd(&it->src_oog_e, (double)(o.E * o.w));
        return;
    }
    int s = -1;
    if (!it->inj_skip && o.w > 0.0f) s = cand_find(psi_row(d, o.cell), it->ctag, o.want);
    if (s >= 0 && d.bid[it->parity][(size_t)o.cell * kKb + s] == o.want) {
        atomicAdd(d.val[it->parity] + ((size_t)o.cell * kKb + s) * Lay::L + o.l, o.w);
        atomicAdd(&it->src_inj_w, o.w);
        atomicAdd(&it->src_inj_e, (double)(o.E * o.w));
    } else {
        atomicAdd(&it->src_slot_w, o.w);
        atomicAdd(&it->src_slot_e, (double)(o.E * o.w));
    }
}

// Weight and bin-centre energy of the w > 0 bins of buffer `buf`
// (compute_psic_total_weight_energy, k1k6_pipeline.cu:706-768); warp per
// occupied cell of that buffer.
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_totals(Dev d, int which) {
    const int buf = d.it->parity ^ which;
    const int n = d.it->occ_n[buf];
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double W = 0.0, E = 0.0;
    for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < n; wi += nw) {
        const int c = d.occ_list[buf][wi];
        const uint32_t b = d.bid[buf][(size_t)c * kKb + lane];
        unsigned used = __ballot_sync(kFull, b != kEmpty);
        while (used) {
            const int s = __ffs(used) - 1;
            used &= used - 1;
            const uint32_t bs = __shfl_sync(kFull, b, s);
            const float* v = d.val[buf] + ((size_t)c * kKb + s) * Lay::L;
            for (int l = lane; l < Lay::L; l += 32) {
                const float w = v[l];
                if (w <= 0.0f) continue;
                int Eb = (int)((bs >> 12) & 0xFFFu) * Lay::NE + (l / Lay::NT) % Lay::NE;
                Eb = max(0, min(Eb, d.N_E - 1));
                W += (double)w;
                E += (double)w * (double)e_center(d, Eb);
            }
        }
    }
    W = warp_sum(W);
    E = warp_sum(E);
    if (lane == 0 && (W != 0.0 || E != 0.0)) {
        atomicAdd(&d.it->tot_w, W);
        atomicAdd(&d.it->tot_e, E);
    }
}

// Sum N per-thread values over the block and add them to dst[0..N) with one
// atomic per value (dst: N consecutive IterState accumulators).
template <int N>
__device__ __forceinline__ void block_add(const double (&v)[N], double* dst) {
    __shared__ double s[N][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const double x = warp_sum(v[k]);
        if (lane == 0) s[k][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double a = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) a += s[threadIdx.x][w];
        if (a != 0.0) atomicAdd(dst + threadIdx.x, a);
    }
}

// ------------------------------------------------------------------ K1
// K1_ActiveMask (k1_activemask.cu:6-48) over the occupied cells of psi_in,
// warp per cell: the cell's class (active / coarse with w > 0,
// compact_coarse_list k1k6_pipeline.cu:625-665), its place in this
// iteration's cell list and bucket map, and, for a listed cell, its w > 0
// bins appended to the bin list (contiguous per cell) for the transport.
// The slot values are read as a flat run of float4s, eight loads in flight
// per lane.  The last block publishes the counts, applies the stopping
// rules, resets the per-iteration accumulators and sets the device loop
// condition.
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_classify(Dev d, cudaGraphConditionalHandle cond, int use_cond) {
    constexpr int Q = Lay::L / 4, NW = kThreads / 32, U = 8;
    __shared__ int s_cnt[2];
    __shared__ int s_last, s_halt, s_listed;
    __shared__ uint8_t s_slot[NW][kKb];   // r-th claimed slot of the warp's cell
    IterState* it = d.it;
    const int par = it->parity;
    const int nocc = it->occ_n[par];
    const unsigned long long g = it->gen + 1;   // number of this classification
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const unsigned lt = (1u << lane) - 1u;
    if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < nocc; wi += nw) {
        const int c = d.occ_list[par][wi];
        const uint32_t b = d.bid[par][(size_t)c * kKb + lane];
        const bool used = b != kEmpty;
        const uint32_t be = (b >> 12) & 0xFFFu;
        const bool c_on = __any_sync(kFull, used && be <= (uint32_t)d.b_on);
        const bool c_off = __any_sync(kFull, used && be <= (uint32_t)d.b_off);
        const unsigned um = __ballot_sync(kFull, used);
        __syncwarp();   // the previous cell's slot table is no longer read
        if (used) s_slot[wid][__popc(um & lt)] = (uint8_t)lane;
        __syncwarp();
        const int F = __popc(um) * Q;   // float4s of the claimed slots
        const float4* vc = reinterpret_cast<const float4*>(d.val[par] + (size_t)c * kKb * Lay::L);
        float ws = 0.0f;
        int nz = 0;
        for (int f0 = 0; f0 < F; f0 += 32 * U) {
            float4 r[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int f = f0 + 32 * u + lane;
                r[u] = f < F ? __ldcg(vc + (size_t)s_slot[wid][f / Q] * Q + f % Q) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ws += (r[u].x + r[u].y) + (r[u].z + r[u].w);
                nz += (r[u].x > 0.0f) + (r[u].y > 0.0f) + (r[u].z > 0.0f) + (r[u].w > 0.0f);
            }
        }
        ws = __shfl_sync(kFull, warp_sumf(ws), 0);
        for (int o = 16; o > 0; o >>= 1) nz += __shfl_xor_sync(kFull, nz, o);
        const bool hw = nz > 0;
        const bool prev = d.act_gen[c] == g - 1;
        const bool act = (c_on || (prev && c_off)) && ws > d.wmin;
        const int cls = act ? 2 : (hw ? 1 : 0);
        int base = 0;
        if (lane == 0) {
            d.cls[c] = (uint8_t)cls;
            if (act) d.act_gen[c] = g;
            if (cls) {
                const int idx = atomicAdd(&it->acc_listed, 1);
                atomicAdd(&it->acc_items, __popc(um));
                base = atomicAdd(&it->acc_bins, nz);
                d.listed[idx] = (uint32_t)c;
                d.c2b[c] = 4 * idx;
                atomicAdd(&s_cnt[act ? 0 : 1], 1);
            }
        }
        if (cls) {
            base = __shfl_sync(kFull, base, 0);
            if (base + nz > d.bins_cap) {   // no room: the last block stops the run
                if (lane == 0) atomicAdd(&it->bin_ovf, 1);
                continue;
            }
            // seed slot of each claimed slot: the rank of its block id
            int rk = 0;
            for (int t = 0; t < kKb; ++t) {
                const uint32_t bt = __shfl_sync(kFull, b, t);
                rk += (bt != kEmpty && bt < b) ? 1 : 0;
            }
            const uint32_t k3 = cls == 2 ? 1u : 0u;
            int off = base;
            for (int f0 = 0; f0 < F; f0 += 32 * U) {
                float4 r[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {   // all loads first (L2 hits of the first read)
                    const int f = f0 + 32 * u + lane;
                    r[u] = f < F ? __ldcg(vc + (size_t)s_slot[wid][f / Q] * Q + f % Q)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int f = f0 + 32 * u + lane;
                    const int s = f < F ? s_slot[wid][f / Q] : 0;
                    const int cnt = (r[u].x > 0.0f) + (r[u].y > 0.0f) + (r[u].z > 0.0f) + (r[u].w > 0.0f);
                    int inc = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int y = __shfl_up_sync(kFull, inc, o);
                        if (lane >= o) inc += y;
                    }
                    const uint32_t bs = __shfl_sync(kFull, b, s);
                    const uint32_t meta = (uint32_t)s | ((uint32_t)__shfl_sync(kFull, rk, s) << 5) | (k3 << 18);
                    int p = off + inc - cnt;
                    const float c4[4] = {r[u].x, r[u].y, r[u].z, r[u].w};
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (c4[k] > 0.0f)
                            d.bins[p++] = make_uint4((uint32_t)c, meta | ((uint32_t)(4 * (f % Q) + k) << 10),
                                                     __float_as_uint(c4[k]), bs);
                    off += __shfl_sync(kFull, inc, 31);
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_cnt[0]) atomicAdd(&it->acc_active, s_cnt[0]);
        if (s_cnt[1]) atomicAdd(&it->acc_coarse, s_cnt[1]);
        __threadfence();
        s_last = atomicAdd(&it->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    if (threadIdx.x == 0) {
        __threadfence();
        volatile IterState* v = it;
        int na = v->acc_active, nc = v->acc_coarse;
        const int nl = v->acc_listed, ni = v->acc_items, nb = v->acc_bins;
        it->acc_active = it->acc_coarse = it->acc_listed = it->acc_items = it->acc_bins = 0;
        it->gen = g;
        it->ctag += 1u;   // claim pass of this iteration
        // C1 stopping rule: in-flight weight (the last audit's W_out) below a
        // fraction of the injected weight ends the run; the rest is booked as
        // a terminal transport drop (k1k6_pipeline.cu:1677-1706 books it too)
        const bool light = d.stop_frac > 0.0f && it->iter > 0 && (na + nc) > 0 &&
                           it->last.W_out_total < d.stop_frac * it->src_inj_w;
        if (light) {
            it->transport_drop_w += it->last.W_out_total;
            it->transport_drop_e += it->last.E_out_total;
            na = nc = 0;
        }
        it->n_active = na;
        it->n_coarse = nc;
        const bool done = (na + nc) == 0;
        it->done = done ? 1 : 0;
        // a bin list that outgrew its capacity ends the run (reported by the
        // host API as SM2D_ERR_ALLOC)
        const bool halt = done || it->iter >= it->max_iter || v->bin_ovf != 0;
        it->halt = halt ? 1 : 0;
        it->n_listed = halt ? 0 : nl;
        it->n_items = halt ? 0 : ni;
        it->n_bins = halt ? 0 : nb;
        double* acc = &it->drop_w;   // the 14 per-iteration accumulators
        for (int k = 0; k < 14; ++k) acc[k] = 0.0;
        it->blocks_done = 0;
        if (!halt) {
            it->cell_steps += (double)(na + nc);
            it->slots_in += (double)ni;
        }
        if (use_cond) cudaGraphSetConditional(cond, (!halt && it->iter + 1 < it->max_iter) ? 1u : 0u);
        s_halt = halt ? 1 : 0;
        s_listed = nl;
    }
    __syncthreads();
    if (s_halt) {   // no transport or finalize follows: release this pass's cell marks
        for (int i = threadIdx.x; i < s_listed; i += blockDim.x) {
            const int c = (int)d.listed[i];
            d.cls[c] = 0;
            d.c2b[c] = -1;
        }
    }
}

// Ascending active and coarse lists from the classes of this iteration
// (the reference's ordered compaction); one block, on request of the
// stepping API.
__global__ void __launch_bounds__(1024) k_order_lists(Dev d) {
    __shared__ int s_w[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int base_a = 0, base_c = 0;
    for (int c0 = 0; c0 < d.Nc; c0 += 1024) {
        const int cell = c0 + (int)threadIdx.x;
        const int cls = cell < d.Nc ? d.cls[cell] : 0;
        const unsigned ba = __ballot_sync(kFull, cls == 2), bc = __ballot_sync(kFull, cls == 1);
        if (lane == 0) { s_w[0][wid] = __popc(ba); s_w[1][wid] = __popc(bc); }
        __syncthreads();
        int oa = base_a, oc = base_c, ta = 0, tc = 0;
        for (int w = 0; w < 32; ++w) {
            if (w < wid) { oa += s_w[0][w]; oc += s_w[1][w]; }
            ta += s_w[0][w];
            tc += s_w[1][w];
        }
        const unsigned lt = (1u << lane) - 1u;
        if (cls == 2) d.active[oa + __popc(ba & lt)] = (uint32_t)cell;
        if (cls == 1) d.coarse[oc + __popc(bc & lt)] = (uint32_t)cell;
        base_a += ta;
        base_c += tc;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ K2/K3
// Sum a per-lane value over runs of lanes with the same cell (the bin list
// keeps a cell's bins contiguous): afterwards the first lane of each run
// holds the run's total.
template <class T>
__device__ __forceinline__ T seg_sum(T v, const unsigned (&same)[5]) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const T n = __shfl_down_sync(kFull, v, 1 << i);
        if (same[i] & (1u << (threadIdx.x & 31))) v += n;
    }
    return v;
}

// One thread per w > 0 bin of the listed cells.  PASS_KEYS gathers the
// claim candidates; the deposit passes add the weights, book per-cell tally
// increments in the dl_* arrays (one atomic per cell run of a warp) and the
// audit sums per block.
template <class Lay, int PASS>
__global__ void __launch_bounds__(kThreads, 2) k_transport(Dev d) {
    IterState* it = d.it;
    if (it->halt) return;
    const int par = it->parity;
    const int n = it->n_bins;
    const uint32_t tag = it->ctag;
    const int lane = threadIdx.x & 31;
    const unsigned salt = d.salt ? (unsigned)it->iter * 0x9E3779B9u : 0u;
    double g[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // drop_w, drop_e, Win, Ein, Wout, Eout, -
    const int stride = gridDim.x * blockDim.x;
    for (int w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < n; w0 += stride) {
        const int i = w0 + lane;
        Tally t{};
        int cell = -1;
        if (i < n) {
            // the claim pass keeps the list in L2 for the deposit pass
            const uint4 r = PASS == PASS_KEYS ? __ldcg(d.bins + i) : __ldcs(d.bins + i);
            cell = (int)r.x;
            const int slot = (int)(r.y & 31u), sslot = (int)((r.y >> 5) & 31u), lidx = (int)((r.y >> 10) & 0xFFu);
            const bool k3 = ((r.y >> 18) & 1u) != 0;
            transport_bin<Lay, PASS>(d, par, k3, cell, r.w, slot, sslot, lidx, __uint_as_float(r.z), salt, tag, t);
        }
        if (PASS != PASS_KEYS) {
            unsigned same[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const int o = 1 << k;
                const int nc = __shfl_down_sync(kFull, cell, o);
                same[k] = __ballot_sync(kFull, lane + o < 32 && cell >= 0 && nc == cell);
            }
            const double edep = seg_sum(t.edep, same), ecut = seg_sum(t.e_cut, same), enuc = seg_sum(t.e_nuc, same),
                         ebnd = seg_sum(t.e_bnd, same);
            const float wcut = seg_sum(t.w_cut, same), wnuc = seg_sum(t.w_nuc, same), wbnd = seg_sum(t.w_bnd, same);
            const int prev_cell = __shfl_up_sync(kFull, cell, 1);
            if (cell >= 0 && (lane == 0 || prev_cell != cell)) {
                if (edep != 0.0) atomicAdd(d.dl_edep + cell, edep);
                if (ecut != 0.0) atomicAdd(d.dl_ecut + cell, ecut);
                if (enuc != 0.0) atomicAdd(d.dl_enuc + cell, enuc);
                if (ebnd != 0.0) atomicAdd(d.dl_ebnd + cell, ebnd);
                if (wcut != 0.0f) atomicAdd(d.dl_wcut + cell, wcut);
                if (wnuc != 0.0f) atomicAdd(d.dl_wnuc + cell, wnuc);
                if (wbnd != 0.0f) atomicAdd(d.dl_wbnd + cell, wbnd);
            }
            g[0] += t.drop_w; g[1] += t.drop_e; g[2] += t.Win; g[3] += t.Ein;
            g[4] += t.Wout; g[5] += t.Eout;
        }
    }
    if (PASS != PASS_KEYS) block_add<7>(g, &it->drop_w);
}

// ------------------------------------------------------------------ slot selection
// Selection of one claim-table row by one warp: the gathered ids ordered by
// claim key; the first 32 become slots 0..31 (written to kept[]), the rest
// fold into the nearest kept id (smallest bid_distance, lowest slot on
// ties).  Each entry's key is replaced by its slot for the deposit pass.
// Returns the number of kept ids.
struct SelScratch {
    uint32_t bid[kCand], key[kCand];
    uint8_t idx[kCand], rank[kCand];
    uint32_t kept[kKb];
};
__device__ int select_row(unsigned long long* row, int* count, uint32_t tag, SelScratch& sh, uint32_t* kept, int lane) {
    const unsigned lt = (1u << lane) - 1u;
    const bool any = *(volatile int*)count > 0;
    int n = 0;
    if (any) {
#pragma unroll
        for (int q = 0; q < kCand / 32; ++q) {
            const int i = q * 32 + lane;
            const unsigned long long tb = __ldcg(row + 2 * i);
            const bool cur = (uint32_t)(tb >> 32) == tag;
            const unsigned m = __ballot_sync(kFull, cur);
            if (cur) {
                const int p = n + __popc(m & lt);
                sh.bid[p] = (uint32_t)tb;
                sh.key[p] = (uint32_t)__ldcg(row + 2 * i + 1);
                sh.idx[p] = (uint8_t)i;
            }
            n += __popc(m);
        }
    }
    __syncwarp();
    for (int j = lane; j < n; j += 32) {
        const uint32_t kj = sh.key[j], bj = sh.bid[j];
        int r = 0;
        for (int m = 0; m < n; ++m) {
            const uint32_t km = sh.key[m];
            r += (km < kj || (km == kj && sh.bid[m] < bj)) ? 1 : 0;
        }
        sh.rank[j] = (uint8_t)r;
        if (r < kKb) sh.kept[r] = bj;
    }
    __syncwarp();
    const int nk = min(n, kKb);
    for (int j = lane; j < n; j += 32) {
        int slot = sh.rank[j];
        if (slot >= kKb) {
            const uint32_t want = sh.bid[j];
            int bd = 0x7fffffff;
            for (int k = 0; k < kKb; ++k) {
                const int dd = bid_distance(sh.kept[k], want);
                if (dd < bd) { bd = dd; slot = k; }
            }
        }
        row[2 * (int)sh.idx[j] + 1] = ((unsigned long long)(0xFFFFFFFFu - tag) << 32) | (uint32_t)slot;
    }
    if (kept) kept[lane] = lane < nk ? sh.kept[lane] : kEmpty;
    if (lane == 0 && any) *count = 0;
    __syncwarp();
    return nk;
}

// Buckets of this pass (warp per listed cell and face): select the kept
// ids, write them to the bucket (bucket mode: also clear its values), and
// offer them to the psi_out row of the cell behind the face in bucket-slot
// order, as K4 claims them.
template <class Lay, bool BUCKET>
__global__ void __launch_bounds__(kThreads) k_select_buckets(Dev d) {
    constexpr int NW = kThreads / 32;
    __shared__ SelScratch s_sel[NW];
    IterState* it = d.it;
    if (it->halt) return;
    const int out = it->parity ^ 1;
    const int n = 4 * it->n_listed;
    const uint32_t tag = it->ctag;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int wi = blockIdx.x * NW + wid; wi < n; wi += gridDim.x * NW) {
        const int face = wi & 3;
        const int src = (int)d.listed[wi >> 2];
        uint32_t* kept = d.bkt_ids + (size_t)wi * kKb;
        const int nk = select_row(bucket_row(d, wi), d.ccount + d.Nc + wi, tag, s_sel[wid], kept, lane);
        if (BUCKET) {
            unsigned char* b = d.buckets + (size_t)wi * d.bucket_bytes;
            bucket_ids(b)[lane] = lane < nk ? s_sel[wid].kept[lane] : kEmpty;
            reinterpret_cast<uint16_t*>(b + 128)[lane] = 0;
            float* v = bucket_vals(b);
            for (int k = lane; k < nk * Lay::L; k += 32) v[k] = 0.0f;
        }
        if (nk == 0) continue;
        const int ix = src % d.Nx, iz = src / d.Nx;
        int dst = -1;
        if (face == FACE_ZP && iz + 1 < d.Nz) dst = src + d.Nx;
        if (face == FACE_ZM && iz > 0) dst = src - d.Nx;
        if (face == FACE_XP && ix + 1 < d.Nx) dst = src + 1;
        if (face == FACE_XM && ix > 0) dst = src - 1;
        if (dst < 0) continue;
        const int k3 = d.cls[src] == 2 ? 1 : 0;
        if (lane < nk)
            cand_insert(psi_row(d, dst), d.ccount + dst, tag, s_sel[wid].kept[lane], k4_key(k3, face, lane),
                        &it->cand_ovf);
        if (lane == 0) mark_occupied(d, out, dst);
    }
}

// Occupied cells of psi_out (which = 1, a transport pass) or of psi_in
// (which = 0, an injection), warp per cell: select the kept ids into the
// cell's slot ids.
__global__ void __launch_bounds__(kThreads) k_select_psi(Dev d, int which) {
    constexpr int NW = kThreads / 32;
    __shared__ SelScratch s_sel[NW];
    IterState* it = d.it;
    if (which && it->halt) return;
    const int buf = it->parity ^ which;
    const int n = it->occ_n[buf];
    const uint32_t tag = it->ctag;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double kept_slots = 0.0;
    for (int wi = blockIdx.x * NW + wid; wi < n; wi += gridDim.x * NW) {
        const int cell = d.occ_list[buf][wi];
        const int nk = select_row(psi_row(d, cell), d.ccount + cell, tag, s_sel[wid], d.bid[buf] + (size_t)cell * kKb,
                                  lane);
        if (lane == 0) kept_slots += (double)nk;
    }
    if (which && lane == 0 && kept_slots != 0.0) atomicAdd(&it->slots_out_it, kept_slots);
}

// ------------------------------------------------------------------ bucket mode (reference structure)
// K4_BucketTransfer (k4_transfer.cu:174-333) driven from the source side:
// warp per (listed cell, face) moves that bucket into psi_out of the
// neighbour behind the face, each bucket slot into the slot its kept id
// resolved to (lidx remap when it folded into a nearer id).
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_bucket_push(Dev d) {
    IterState* it = d.it;
    if (it->halt) return;
    const int out = it->parity ^ 1;
    const int n = 4 * it->n_listed;
    const uint32_t tag = it->ctag;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double g[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // drop_w, drop_e, -, -, Wout, Eout, -
    for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < n; wi += nw) {
        const int face = wi & 3;
        const int src = (int)d.listed[wi >> 2];
        const int ix = src % d.Nx, iz = src / d.Nx;
        int dst = -1;
        if (face == FACE_ZP && iz + 1 < d.Nz) dst = src + d.Nx;
        if (face == FACE_ZM && iz > 0) dst = src - d.Nx;
        if (face == FACE_XP && ix + 1 < d.Nx) dst = src + 1;
        if (face == FACE_XM && ix > 0) dst = src - 1;
        if (dst < 0) continue;
        unsigned char* b = d.buckets + (size_t)wi * d.bucket_bytes;
        const uint32_t sb = bucket_ids(b)[lane];
        unsigned um = __ballot_sync(kFull, sb != kEmpty);
        const float* bv = bucket_vals(b);
        const uint32_t* kept = d.bid[out] + (size_t)dst * kKb;
        while (um) {
            const int s = __ffs(um) - 1;
            um &= um - 1;
            const uint32_t bid = __shfl_sync(kFull, sb, s);
            uint32_t sel = bid;
            const int os = resolve(d, psi_row(d, dst), kept, tag, bid, sel);
            const float* v = bv + (size_t)s * Lay::L;
            float* o = os >= 0 ? d.val[out] + ((size_t)dst * kKb + os) * Lay::L : nullptr;
            double eshift = 0.0;
            for (int l = lane; l < Lay::L; l += 32) {
                const float w = v[l];
                if (w <= 0.0f) continue;
                if (os < 0) {
                    g[0] += (double)w;
                    g[1] += (double)e_center(d, ebin_of<Lay>(d, bid, l)) * (double)w;
                    continue;
                }
                const int le = sel != bid ? remap_lidx<Lay>(l, bid, sel) : l;
                atomicAdd(o + le, w);
                const int Eb = ebin_of<Lay>(d, sel, le);
                if (sel != bid && d.esplit)
                    eshift += (double)((e_center(d, ebin_of<Lay>(d, bid, l)) - e_center(d, Eb)) * w);
                g[4] += (double)w;
                g[5] += (double)w * (double)e_center(d, Eb);
            }
            eshift = warp_sum(eshift);
            if (lane == 0 && eshift != 0.0) atomicAdd(d.dl_edep + src, eshift);
        }
    }
    block_add<7>(g, &it->drop_w);
}

// ------------------------------------------------------------------ K5 + clear + K6
__device__ void finalize_audit(Dev& d) {
    volatile IterState* v = d.it;
    IterState* it = d.it;
    sm2d_audit r;
    memset(&r, 0, sizeof r);
    r.W_in_total = (float)v->Win;
    r.W_out_total = (float)v->Wout;
    r.W_cutoff_total = (float)v->Wcut;
    r.W_nuclear_total = (float)v->Wnuc;
    r.W_boundary_total = (float)v->Wbnd;
    r.E_in_total = v->Ein;
    r.E_out_total = v->Eout;
    r.E_dep_total = v->Edep;
    r.E_cutoff_total = v->Ecut;
    r.E_nuclear_total = v->Enuc;
    r.E_boundary_total = v->Ebnd;
    const double dw = v->drop_w, de = v->drop_e;
    r.W_transport_drop_total = fmaxf(0.0f, (float)dw);
    r.E_transport_drop_total = fmax(0.0, de);
    if (v->include_source) {
        const float wso = fmaxf(0.0f, v->src_oog_w), wss = fmaxf(0.0f, v->src_slot_w);
        const double eso = fmax(0.0, v->src_oog_e), ess = fmax(0.0, v->src_slot_e);
        r.W_in_total += wso + wss;
        r.E_in_total += eso + ess;
        r.W_source_out_of_grid_total = wso;
        r.W_source_slot_drop_total = wss;
        r.E_source_out_of_grid_total = eso;
        r.E_source_slot_drop_total = ess;
    }
    r.processed_cells = d.Nc;
    const float Wr = r.W_out_total + r.W_cutoff_total + r.W_nuclear_total + r.W_boundary_total +
                     r.W_transport_drop_total + r.W_source_out_of_grid_total + r.W_source_slot_drop_total;
    const float We = fabsf(r.W_in_total - Wr) / fmaxf(r.W_in_total, 1e-20f);
    r.W_error = We;
    r.W_pass = (isfinite(We) && We < 1e-6f) ? 1 : 0;
    const double Er = r.E_out_total + r.E_dep_total + r.E_cutoff_total + r.E_nuclear_total + r.E_boundary_total +
                      r.E_transport_drop_total + r.E_source_out_of_grid_total + r.E_source_slot_drop_total;
    const float Ee_ = (float)(fabs(r.E_in_total - Er) / fmax(r.E_in_total, 1e-20));
    r.E_error = Ee_;
    r.E_pass = (isfinite(Ee_) && Ee_ < 1e-5f) ? 1 : 0;
    const double resid = r.E_in_total - Er;
    if (isfinite(resid)) it->audit_residual += resid;
    it->transport_drop_w += dw;
    it->transport_drop_e += de;
    it->slots_out += v->slots_out_it;
    const int k = it->iter;
    if (k < d.hist_cap) d.hist[k] = r;
    it->last = r;
    it->iter = k + 1;
    it->include_source = 0;
    it->occ_n[it->parity] = 0;   // the consumed buffer is empty again
    it->parity ^= 1;
    it->blocks_done = 0;
}

// Fold this iteration's increment of tally k of cell c into the cumulative
// tally; K5 books max(0, cumulative - previous) per cell (k5_audit.cu:93-99).
__device__ __forceinline__ double fold_tally(const Dev& d, int c, int k) {
    if (k < 4) {
        double* cum = k == 0 ? d.edep : (k == 1 ? d.e_cut : (k == 2 ? d.e_nuc : d.e_bnd));
        double* dl = k == 0 ? d.dl_edep : (k == 1 ? d.dl_ecut : (k == 2 ? d.dl_enuc : d.dl_ebnd));
        const double x = dl[c];
        if (x == 0.0) return 0.0;
        const double e0 = cum[c], e1 = e0 + x;
        cum[c] = e1;
        dl[c] = 0.0;
        return fmax(0.0, e1 - e0);
    }
    float* cum = k == 4 ? d.w_cut : (k == 5 ? d.w_nuc : d.w_bnd);
    float* dl = k == 4 ? d.dl_wcut : (k == 5 ? d.dl_wnuc : d.dl_wbnd);
    const float x = dl[c];
    if (x == 0.0f) return 0.0;
    const float w0 = cum[c], w1 = w0 + x;
    cum[c] = w1;
    dl[c] = 0.0f;
    return (double)fmaxf(0.0f, w1 - w0);
}

// K5 audit of the iteration and clear of the consumed buffer, warp per
// occupied cell of psi_in; the last block writes the audit record and swaps
// the buffers (K6).
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_finalize(Dev d) {
    constexpr int NW = kThreads / 32;
    __shared__ double s_acc[7][NW];
    __shared__ int s_last;
    IterState* it = d.it;
    if (it->halt) return;
    const int in = it->parity;
    const int nocc = it->occ_n[in];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = gridDim.x * NW;
    double part = 0.0;   // lane k < 7: audit share of tally k (edep, e_cut, e_nuc, e_bnd, w_cut, w_nuc, w_bnd)
    for (int wi = blockIdx.x * NW + wid; wi < nocc; wi += nw) {
        const int c = d.occ_list[in][wi];
        const int cls = d.cls[c];
        uint32_t* ids = d.bid[in] + (size_t)c * kKb;
        unsigned um = __ballot_sync(kFull, ids[lane] != kEmpty);
        while (um) {   // clear the consumed slots
            const int s = __ffs(um) - 1;
            um &= um - 1;
            float4* v = reinterpret_cast<float4*>(d.val[in] + ((size_t)c * kKb + s) * Lay::L);
            for (int q = lane; q < Lay::L / 4; q += 32) __stcs(v + q, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        if (cls && lane < 7) part += fold_tally(d, c, lane);
        ids[lane] = kEmpty;
        if (lane == 0) {
            d.occ[in][c] = 0;
            d.cls[c] = 0;
            if (cls) d.c2b[c] = -1;
        }
    }
    if (lane < 7) s_acc[lane][wid] = part;
    __syncthreads();
    if (threadIdx.x < 7) {
        double a = 0.0;
        for (int w = 0; w < NW; ++w) a += s_acc[threadIdx.x][w];
        if (a != 0.0) atomicAdd(&it->Edep + threadIdx.x, a);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&it->blocks_done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        finalize_audit(d);
    }
}

// ------------------------------------------------------------------ spot pipeline helpers
// Clear every claimed slot of both buffers (reset between spots).
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_clear_all(Dev d) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int b = 0; b < 2; ++b) {
        const int n = d.it->occ_n[b];
        for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < n; wi += nw) {
            const int c = d.occ_list[b][wi];
            uint32_t* ids = d.bid[b] + (size_t)c * kKb;
            const uint32_t x = ids[lane];
            unsigned um = __ballot_sync(kFull, x != kEmpty);
            while (um) {
                const int s = __ffs(um) - 1;
                um &= um - 1;
                float4* v = reinterpret_cast<float4*>(d.val[b] + ((size_t)c * kKb + s) * Lay::L);
                for (int q = lane; q < Lay::L / 4; q += 32) v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            ids[lane] = kEmpty;
            if (lane == 0) { d.occ[b][c] = 0; d.cls[c] = 0; }
        }
    }
}

__global__ void k_reset_state(IterState* it) {
    if (threadIdx.x || blockIdx.x) return;
    // the classification number runs on, one step past the last spot's, so
    // that no cell reads as active in a previous classification; the claim
    // pass number runs on too, and restarts after a wipe of the tables when
    // it nears its 32-bit limit
    const unsigned long long g = it->gen;
    uint32_t tag = it->ctag;
    const int ovf = it->cand_ovf, miss = it->cand_miss;
    int wipe = 0;
    if (tag >= 0xFFF00000u) {
        tag = 0;
        wipe = 1;
    }
    memset(it, 0, sizeof(IterState));
    it->gen = g + 1;
    it->ctag = tag;
    it->cand_ovf = ovf;
    it->cand_miss = miss;
    it->wipe = wipe;
    it->max_iter = INT_MAX;
}

// Clear every claim-table row when a tag wrap is pending (grid-stride).
__global__ void k_wipe(Dev d, size_t n_words, int n_counts) {
    if (!d.it->wipe) return;
    const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, st = (size_t)gridDim.x * blockDim.x;
    for (size_t i = i0; i < n_words; i += st) d.ctab[i] = ~0ull;
    for (size_t i = i0; i < (size_t)n_counts; i += st) d.ccount[i] = 0;
}

__global__ void k_set_iter_limit(IterState* it, int more) {
    if (threadIdx.x || blockIdx.x) return;
    const long long lim = (long long)it->iter + more;
    it->max_iter = lim > INT_MAX ? INT_MAX : (int)lim;
}

// Source accounting after injection (gpu_transport_wrapper.cu:339-460): the
// pencil path books W and E0*W; the represented energy comes from k_totals.
__global__ void k_source_finalize(IterState* it, const BeamArgs* b, int gaussian) {
    if (threadIdx.x || blockIdx.x) return;
    if (!gaussian) {
        it->src_inj_w = b->W;
        it->src_inj_e = (double)b->E0 * (double)b->W;
    }
    double loss = it->src_inj_e - it->tot_e;
    if (fabs(loss) < 1e-12) loss = 0.0;
    it->src_rep_loss = loss;
    it->include_source = 1;
    it->done = 0;
}

// Lateral MCS post-convolution of EdepC, one thread per output cell
// (gpu_transport_wrapper.cu:551-616; kernels built on the host at create).
__global__ void k_dose(const double* __restrict__ edep, const int* __restrict__ half, const double* __restrict__ ker,
                       int kstride, int Nx, int Nz, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nx * Nz) return;
    const int iz = i / Nx, ix = i - iz * Nx;
    const int h = half[iz];
    if (h == 0) { out[i] = edep[i]; return; }
    const double* k = ker + (size_t)iz * kstride;
    const double* row = edep + (size_t)iz * Nx;
    double acc = 0.0;
    for (int j = -h; j <= h; ++j) {
        const int x = ix + j;
        if (x >= 0 && x < Nx) acc += row[x] * k[j + h];
    }
    out[i] = acc;
}

// ================================================================== engine
struct Ctx {
    sm2d_problem p{};
    std::vector<float> th, Ee, feA, feB, feS;
    int L = 0, layout = 0;  // 0: LayoutRef, 1: LayoutB128
    Dev d{};
    IterState* it_host = nullptr;  // pinned mirror
    cudaStream_t s = nullptr;
    std::vector<void*> allocs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle cond{};
    cudaEvent_t ev[10] = {};   // 0..7 one iteration's stages, 8..9 a whole run
    float step_ms[7] = {};
    int grid_cell = 0, grid_transport = 0;   // warp-per-cell kernels, transport
    size_t ctab_words = 0;                   // claim-table size in 64-bit words
    bool injected = false;
    BeamArgs* beam_dev = nullptr;   // device copy of the current beam
    int* dose_half = nullptr;       // per-row half width of the lateral kernel
    double* dose_ker = nullptr;     // per-row kernel weights
    double* dose_dev = nullptr;     // convolved dose
    int dose_stride = 1;
    std::vector<cudaEvent_t> pev;   // event pool of the profiled replay
};

static int dalloc(Ctx& c, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(SM2D_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    c.allocs.push_back(*p);
    return 0;
}

template <class Lay>
struct Impl {
    // One iteration: K1 classify, (ascending lists on request), the claim
    // pass of K2/K3, bucket and psi_out slot selection, the deposit pass of
    // K2/K3 with the fused K4 scatter or the bucket pair, K5 finalize.
    // ev[0..7] bracket: classify, lists, claim pass, selection, deposit pass,
    // K4 bucket move, finalize.
    static int launch_body(Ctx& c, bool timed, bool use_cond, bool lists) {
        const int gc = c.grid_cell, gt = c.grid_transport;
        const bool bk = c.p.use_buckets != 0;
        auto rec = [&](int k) { return timed ? cudaEventRecord(c.ev[k], c.s) : cudaSuccess; };
        CK(rec(0));
        k_classify<Lay><<<gc, kThreads, 0, c.s>>>(c.d, c.cond, use_cond ? 1 : 0);
        CK(rec(1));
        if (lists) k_order_lists<<<1, 1024, 0, c.s>>>(c.d);
        CK(rec(2));
        k_transport<Lay, PASS_KEYS><<<gt, kThreads, 0, c.s>>>(c.d);
        CK(rec(3));
        if (bk) k_select_buckets<Lay, true><<<gc, kThreads, 0, c.s>>>(c.d);
        else k_select_buckets<Lay, false><<<gc, kThreads, 0, c.s>>>(c.d);
        k_select_psi<<<gc, kThreads, 0, c.s>>>(c.d, 1);
        CK(rec(4));
        if (bk) k_transport<Lay, PASS_BUCKET><<<gt, kThreads, 0, c.s>>>(c.d);
        else k_transport<Lay, PASS_DIRECT><<<gt, kThreads, 0, c.s>>>(c.d);
        CK(rec(5));
        if (bk) k_bucket_push<Lay><<<gc, kThreads, 0, c.s>>>(c.d);
        CK(rec(6));
        k_finalize<Lay><<<gc, kThreads, 0, c.s>>>(c.d);
        CK(rec(7));
        CK(cudaGetLastError());
        return 0;
    }
    static int transport_grid(Ctx& c, int sms) {
        int per_sm = 0;
        cudaError_t e = c.p.use_buckets
                            ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport<Lay, PASS_BUCKET>, kThreads, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport<Lay, PASS_DIRECT>, kThreads, 0);
        if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
        const long long items = (long long)c.d.bins_cap / 32;   // one warp per 32 bins at most
        const long long full = (long long)std::max(per_sm, 1) * std::max(sms, 1);
        c.grid_transport = (int)std::max(1LL, std::min(full, (items + kThreads / 32 - 1) / (kThreads / 32)));
        return 0;
    }
    static int clear_all(Ctx& c, int) {
        k_clear_all<Lay><<<c.grid_cell, kThreads, 0, c.s>>>(c.d);
        CK(cudaGetLastError());
        return 0;
    }
    // injection from the device beam description: claim pass, slot
    // selection, deposit pass
    static int inject_dev(Ctx& c, int n, bool gaussian) {
        const int blocks = gaussian ? (n + 255) / 256 : 1;
        k_inject_begin<<<1, 1, 0, c.s>>>(c.d.it);
        k_inject_keys<Lay><<<blocks, 256, 0, c.s>>>(c.d, c.beam_dev, gaussian ? 1 : 0);
        k_select_psi<<<c.grid_cell, kThreads, 0, c.s>>>(c.d, 0);
        k_inject_deposit<Lay><<<blocks, 256, 0, c.s>>>(c.d, c.beam_dev, gaussian ? 1 : 0);
        CK(cudaGetLastError());
        return 0;
    }
    static int totals(Ctx& c, int which) {
        k_totals<Lay><<<c.grid_cell, kThreads, 0, c.s>>>(c.d, which);
        CK(cudaGetLastError());
        return 0;
    }
};

#define DISPATCH(c, fn, ...) ((c).layout == 0 ? Impl<LayoutRef>::fn(c, __VA_ARGS__) : Impl<LayoutB128>::fn(c, __VA_ARGS__))

static int sync_state(Ctx& c) {
    CK(cudaMemcpyAsync(c.it_host, c.d.it, sizeof(IterState), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}
static int push_state(Ctx& c) {
    CK(cudaMemcpyAsync(c.d.it, c.it_host, sizeof(IterState), cudaMemcpyHostToDevice, c.s));
    return 0;
}

static int build_graph(Ctx& c) {
    if (c.exec) return 0;
    CK(cudaGraphCreate(&c.graph, 0));
    CK(cudaGraphConditionalHandleCreate(&c.cond, c.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = c.cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, c.graph, nullptr, nullptr, 0, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(c.s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = DISPATCH(c, launch_body, false, true, false);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(c.s, &captured);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    CK(cudaGraphInstantiate(&c.exec, c.graph, 0));
    return 0;
}

}  // namespace sm2d

using namespace sm2d;

struct sm2d_ctx : sm2d::Ctx {};

extern "C" {


int sm2d_create(const sm2d_problem* p, sm2d_handle* out) {
    if (!p || !out) return fail(SM2D_ERR_ARG, "null argument");
    *out = nullptr;
    if (p->Nx <= 0 || p->Nz <= 0 || p->N_theta <= 0 || p->N_E <= 1 || !p->theta_edges || !p->E_edges)
        return fail(SM2D_ERR_ARG, "invalid grid");
    if (!(p->dx > 0.0f) || !(p->dz > 0.0f)) return fail(SM2D_ERR_ARG, "cell size must be positive");
    // work items pack (cell << 5) | slot into 32 bits
    if ((long long)p->Nx * p->Nz > (1LL << 27)) return fail(SM2D_ERR_ARG, "grid too large (at most 2^27 cells)");
    int layout;
    if (p->nt_local == 4 && p->ne_local == 2 && p->nx_sub == 8 && p->nz_sub == 4) layout = 0;
    else if (p->nt_local == 8 && p->ne_local == 4 && p->nx_sub == 4 && p->nz_sub == 1) layout = 1;
    else return fail(SM2D_ERR_LAYOUT, "local layout (%d,%d,%d,%d) not compiled; use (4,2,8,4) or (8,4,4,1)",
                     p->nt_local, p->ne_local, p->nx_sub, p->nz_sub);
    if (p->N_theta / p->nt_local > 4095 || p->N_E / p->ne_local > 4095)
        return fail(SM2D_ERR_ARG, "grid exceeds the 12-bit block indices");
    sm2d_ctx* c = new sm2d_ctx();
    c->p = *p;
    c->layout = layout;
    c->L = p->nt_local * p->ne_local * p->nx_sub * p->nz_sub;
    c->th.assign(p->theta_edges, p->theta_edges + p->N_theta + 1);
    c->Ee.assign(p->E_edges, p->E_edges + p->N_E + 1);
    auto bail = [&](int rc) { sm2d_destroy(c); return rc; };
    if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(SM2D_ERR_CUDA, "no CUDA device"));
    for (auto& e : c->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return bail(fail(SM2D_ERR_CUDA, "event create"));
    const int N = p->N_E;
    std::vector<float> rep(N), R(N), S(N), lE(N), lR(N), lS(N);
    for (int i = 0; i < N; ++i) rep[i] = std::sqrt(c->Ee[i] * c->Ee[i + 1]);
    range_lut(N, rep.data(), R.data(), S.data(), lE.data(), lR.data(), lS.data());
    c->feA.resize(p->Nz);
    c->feB.resize(p->Nz);
    c->feS.resize(p->Nz);
    fermi_eyges_moments(p->E0, p->Nz, p->dz, p->sigma_x_initial, c->feA.data(), c->feB.data(), c->feS.data());
    Dev& d = c->d;
    d.Nx = p->Nx; d.Nz = p->Nz; d.Nc = p->Nx * p->Nz;
    d.dx = p->dx; d.dz = p->dz;
    d.N_theta = p->N_theta; d.N_E = N;
    d.lutN = N;
    d.lutEmin = p->E_min > 0.0f ? p->E_min : c->Ee[0];
    d.lutEmax = p->E_max > 0.0f ? p->E_max : c->Ee[N];
    d.E_fine_on = p->E_fine_on; d.wmin = p->weight_active_min;
    d.step_coarse = p->step_coarse; d.sx0 = p->sigma_x_initial;
    // compute_b_E_threshold: EnergyGrid::FindBin(E) / N_E_local
    auto find_bin_host = [&](float E) {
        if (E < c->Ee[0]) return 0;
        if (E >= c->Ee[N]) return N - 1;
        int lo = 0, hi = N;
        while (lo < hi) { int m = (lo + hi) / 2; if (c->Ee[m + 1] <= E) lo = m + 1; else hi = m; }
        return lo;
    };
    d.b_on = find_bin_host(p->E_fine_on) / p->ne_local;
    d.b_off = find_bin_host(p->E_fine_off) / p->ne_local;
    d.straggle = p->enable_straggling; d.nuclear = p->enable_nuclear;
    d.seed_mode = p->seed_slot_mode; d.esplit = p->energy_split;
    d.prune_coarse = p->prune_coarse > 0.0f ? p->prune_coarse : 1e-12f;
    d.prune_fine = p->prune_fine > 0.0f ? p->prune_fine : 1e-15f;
    d.split_min_w = p->split_min_weight;
    d.stop_frac = p->stop_weight_fraction;
    d.floor_cutoff = p->floor_cutoff;
    d.salt = p->seed_iteration_salt;
    const size_t Nc = (size_t)d.Nc, ns = Nc * kKb;
    void* q;
    int rc;
#define A(ptr, type, n)                                              \
    if ((rc = dalloc(*c, &q, sizeof(type) * (size_t)(n)))) return bail(rc); \
    ptr = reinterpret_cast<type*>(q)
    float *th_d, *Ee_d, *R_d, *lE_d, *lR_d, *fa, *fb;
    A(th_d, float, p->N_theta + 1);
    A(Ee_d, float, N + 1);
    A(R_d, float, N);
    A(lE_d, float, N);
    A(lR_d, float, N);
    A(fa, float, p->Nz);
    A(fb, float, p->Nz);
    d.th = th_d; d.Ee = Ee_d; d.R = R_d; d.logE = lE_d; d.logR = lR_d; d.feA = fa; d.feB = fb;
    for (int b = 0; b < 2; ++b) {
        A(d.bid[b], uint32_t, ns);
        A(d.val[b], float, ns * c->L);
        A(d.occ[b], int, Nc);
        A(d.occ_list[b], int, Nc);
    }
    A(d.edep, double, Nc); A(d.e_cut, double, Nc); A(d.e_nuc, double, Nc); A(d.e_bnd, double, Nc);
    A(d.w_cut, float, Nc); A(d.w_nuc, float, Nc); A(d.w_bnd, float, Nc);
    A(d.dl_edep, double, Nc); A(d.dl_ecut, double, Nc); A(d.dl_enuc, double, Nc); A(d.dl_ebnd, double, Nc);
    A(d.dl_wcut, float, Nc); A(d.dl_wnuc, float, Nc); A(d.dl_wbnd, float, Nc);
    A(d.act_gen, unsigned long long, Nc); A(d.cls, uint8_t, Nc);
    A(d.listed, uint32_t, Nc);
    // bin list: room for the w > 0 bins of four full slots per cell of the
    // grid on average (a listed cell holds at most 32); a run that needs
    // more stops with SM2D_ERR_ALLOC
    d.bins_cap = (int)std::min<size_t>((size_t)Nc * 4 * c->L, (size_t)INT_MAX);
    A(d.bins, uint4, d.bins_cap);
    A(d.active, uint32_t, Nc); A(d.coarse, uint32_t, Nc);
    A(d.it, IterState, 1);
    d.hist_cap = p->max_iterations > 0 ? p->max_iterations : 4096;
    A(d.hist, sm2d_audit, d.hist_cap);
    d.bucket_bytes = bucket_bytes_for(c->L);
    if (p->use_buckets) A(d.buckets, unsigned char, (size_t)Nc * 4 * d.bucket_bytes);
    A(d.c2b, int, Nc);
    c->ctab_words = (size_t)5 * Nc * 2 * kCand;
    A(d.ctab, unsigned long long, c->ctab_words);
    A(d.ccount, int, 5 * Nc);
    A(d.bkt_ids, uint32_t, (size_t)4 * Nc * kKb);
    if (cudaMemsetAsync(d.c2b, 0xFF, Nc * sizeof(int), c->s) != cudaSuccess ||
        cudaMemsetAsync(d.ctab, 0xFF, c->ctab_words * 8, c->s) != cudaSuccess ||
        cudaMemsetAsync(d.ccount, 0, 5 * Nc * sizeof(int), c->s) != cudaSuccess ||
        cudaMemsetAsync(d.bkt_ids, 0xFF, (size_t)4 * Nc * kKb * 4, c->s) != cudaSuccess)
        return bail(fail(SM2D_ERR_CUDA, "memset"));
    A(c->beam_dev, BeamArgs, 1);
    {   // lateral post-convolution kernels per depth row
        std::vector<int> half(p->Nz, 0);
        std::vector<double> k(p->Nx + 2);
        int hmax = 1;
        for (int iz = 0; iz < p->Nz; ++iz) {
            half[iz] = lateral_kernel(c->feS[iz], p->sigma_x_initial, p->dx, p->Nx, k.data());
            hmax = std::max(hmax, half[iz]);
        }
        c->dose_stride = 2 * hmax + 1;
        std::vector<double> ker((size_t)p->Nz * c->dose_stride, 0.0);
        for (int iz = 0; iz < p->Nz; ++iz)
            if (half[iz]) lateral_kernel(c->feS[iz], p->sigma_x_initial, p->dx, p->Nx, &ker[(size_t)iz * c->dose_stride]);
        A(c->dose_half, int, p->Nz);
        A(c->dose_ker, double, ker.size());
        A(c->dose_dev, double, Nc);
        if (cudaMemcpy(c->dose_half, half.data(), sizeof(int) * p->Nz, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(c->dose_ker, ker.data(), sizeof(double) * ker.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(SM2D_ERR_CUDA, "dose kernel upload"));
    }
#undef A
    if (cudaMallocHost(&c->it_host, sizeof(IterState)) != cudaSuccess) return bail(fail(SM2D_ERR_ALLOC, "pinned"));
    memset(c->it_host, 0, sizeof(IterState));
    c->it_host->max_iter = INT_MAX;
    cudaStream_t s = c->s;
    bool ok = cudaMemcpyAsync(th_d, c->th.data(), sizeof(float) * (p->N_theta + 1), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(Ee_d, c->Ee.data(), sizeof(float) * (N + 1), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(R_d, R.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(lE_d, lE.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(lR_d, lR.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(fa, c->feA.data(), sizeof(float) * p->Nz, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(fb, c->feB.data(), sizeof(float) * p->Nz, cudaMemcpyHostToDevice, s) == cudaSuccess;
    for (int b = 0; b < 2 && ok; ++b)
        ok = cudaMemsetAsync(d.bid[b], 0xFF, ns * 4, s) == cudaSuccess &&
             cudaMemsetAsync(d.val[b], 0, ns * c->L * 4, s) == cudaSuccess &&
             cudaMemsetAsync(d.occ[b], 0, Nc * 4, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(d.edep, 0, Nc * 8, s) == cudaSuccess && cudaMemsetAsync(d.e_cut, 0, Nc * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.e_nuc, 0, Nc * 8, s) == cudaSuccess && cudaMemsetAsync(d.e_bnd, 0, Nc * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.w_cut, 0, Nc * 4, s) == cudaSuccess && cudaMemsetAsync(d.w_nuc, 0, Nc * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.w_bnd, 0, Nc * 4, s) == cudaSuccess && cudaMemsetAsync(d.act_gen, 0, Nc * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.cls, 0, Nc, s) == cudaSuccess && cudaMemsetAsync(d.dl_edep, 0, Nc * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_ecut, 0, Nc * 8, s) == cudaSuccess && cudaMemsetAsync(d.dl_enuc, 0, Nc * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_ebnd, 0, Nc * 8, s) == cudaSuccess && cudaMemsetAsync(d.dl_wcut, 0, Nc * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_wnuc, 0, Nc * 4, s) == cudaSuccess && cudaMemsetAsync(d.dl_wbnd, 0, Nc * 4, s) == cudaSuccess;
    if (!ok) return bail(fail(SM2D_ERR_CUDA, "initial copies failed"));
    {   // grid origin of the beam description is fixed per problem
        BeamArgs origin{};
        origin.x_min = p->x_min;
        origin.z_min = p->z_min;
        if (cudaMemcpyAsync(c->beam_dev, &origin, sizeof origin, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return bail(fail(SM2D_ERR_CUDA, "beam origin upload"));
    }
    if (push_state(*c)) return bail(SM2D_ERR_CUDA);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    c->grid_cell = std::max(1, std::min((int)((Nc + kThreads / 32 - 1) / (kThreads / 32)), 4 * std::max(sms, 1)));
    if ((rc = DISPATCH(*c, transport_grid, sms))) return bail(rc);
    if (cudaStreamSynchronize(s) != cudaSuccess) return bail(fail(SM2D_ERR_CUDA, "create sync"));
    *out = c;
    return 0;
}

int sm2d_destroy(sm2d_handle h) {
    if (!h) return 0;
    if (h->s) cudaStreamSynchronize(h->s);
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : h->pev) cudaEventDestroy(e);
    if (h->it_host) cudaFreeHost(h->it_host);
    if (h->s) cudaStreamDestroy(h->s);
    delete h;
    return 0;
}

int sm2d_local_bins(sm2d_handle h) { return h ? h->L : SM2D_ERR_ARG; }

int sm2d_inject(sm2d_handle h, const sm2d_beam* b) {
    if (!h || !b) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    int rc = sync_state(c);
    if (rc) return rc;
    if (c.it_host->occ_n[c.it_host->parity] != 0)
        return fail(SM2D_ERR_STATE, "phase space not empty: call sm2d_reset before injecting");
    if ((rc = sm2d_inject_async(h, b))) return rc;
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

int sm2d_set_psi_in(sm2d_handle h, const uint32_t* bid, const float* val) {
    if (!h || !bid || !val) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    int rc = sync_state(c);
    if (rc) return rc;
    const int par = c.it_host->parity;
    const size_t ns = (size_t)c.d.Nc * kKb;
    std::vector<int> occ(c.d.Nc, 0), list;
    for (int cell = 0; cell < c.d.Nc; ++cell)
        for (int k = 0; k < kKb; ++k)
            if (bid[(size_t)cell * kKb + k] != kEmpty) {
                occ[cell] = 1;
                list.push_back(cell);
                break;
            }
    CK(cudaMemcpyAsync(c.d.bid[par], bid, ns * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(c.d.val[par], val, ns * c.L * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(c.d.occ[par], occ.data(), sizeof(int) * occ.size(), cudaMemcpyHostToDevice, c.s));
    if (!list.empty())
        CK(cudaMemcpyAsync(c.d.occ_list[par], list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, c.s));
    c.it_host->occ_n[par] = (int)list.size();
    c.it_host->done = 0;
    if ((rc = push_state(c))) return rc;
    CK(cudaStreamSynchronize(c.s));
    c.injected = true;
    return 0;
}

int sm2d_get_psi_in(sm2d_handle h, uint32_t* bid, float* val) {
    if (!h || !bid) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    int rc = sync_state(c);
    if (rc) return rc;
    const int par = c.it_host->parity;
    const size_t ns = (size_t)c.d.Nc * kKb;
    CK(cudaMemcpyAsync(bid, c.d.bid[par], ns * 4, cudaMemcpyDeviceToHost, c.s));
    if (val) CK(cudaMemcpyAsync(val, c.d.val[par], ns * c.L * 4, cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

int sm2d_step(sm2d_handle h, int* n_active, int* n_coarse) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space: call sm2d_inject or sm2d_set_psi_in first");
    int rc = DISPATCH(c, launch_body, true, false, true);
    if (rc) return rc;
    if ((rc = sync_state(c))) return rc;
    if (c.it_host->bin_ovf) return fail(SM2D_ERR_ALLOC, "bin list capacity (%d bins) exceeded", c.d.bins_cap);
    // classify, lists, claim pass, selection, deposit pass, K4 bucket move, finalize
    for (int k = 0; k < 7; ++k) CK(cudaEventElapsedTime(&c.step_ms[k], c.ev[k], c.ev[k + 1]));
    if (n_active) *n_active = c.it_host->done ? 0 : c.it_host->n_active;
    if (n_coarse) *n_coarse = c.it_host->done ? 0 : c.it_host->n_coarse;
    return 0;
}

static int run_impl(Ctx& c, int max_it, int* done_iters, float* ms) {
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space: call sm2d_inject or sm2d_set_psi_in first");
    if (max_it <= 0) return fail(SM2D_ERR_ARG, "max_iterations must be positive");
    int rc = build_graph(c);
    if (rc) return rc;
    if ((rc = sync_state(c))) return rc;
    const int start = c.it_host->iter;
    c.it_host->max_iter = start + max_it;
    if ((rc = push_state(c))) return rc;
    if (ms) CK(cudaEventRecord(c.ev[8], c.s));
    CK(cudaGraphLaunch(c.exec, c.s));
    if (ms) CK(cudaEventRecord(c.ev[9], c.s));
    CK(cudaStreamSynchronize(c.s));
    if (ms) CK(cudaEventElapsedTime(ms, c.ev[8], c.ev[9]));
    if ((rc = sync_state(c))) return rc;
    c.it_host->max_iter = INT_MAX;
    if ((rc = push_state(c))) return rc;
    CK(cudaStreamSynchronize(c.s));
    if (done_iters) *done_iters = c.it_host->iter - start;
    if (c.it_host->bin_ovf) return fail(SM2D_ERR_ALLOC, "bin list capacity (%d bins) exceeded", c.d.bins_cap);
    return 0;
}

int sm2d_run(sm2d_handle h, int max_it, int* done_iters) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    return run_impl(*h, max_it, done_iters, nullptr);
}

int sm2d_run_timed(sm2d_handle h, int max_it, int* done_iters, float* ms) {
    if (!h || !ms) return fail(SM2D_ERR_ARG, "null argument");
    return run_impl(*h, max_it, done_iters, ms);
}

int sm2d_get_mask(sm2d_handle h, uint8_t* mask) {
    if (!h || !mask) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    std::vector<unsigned long long> g(h->d.Nc);
    CK(cudaMemcpyAsync(g.data(), h->d.act_gen, sizeof(unsigned long long) * g.size(), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    const unsigned long long cur = h->it_host->gen;
    for (int i = 0; i < h->d.Nc; ++i) mask[i] = (cur != 0 && g[i] == cur) ? 1 : 0;
    return 0;
}

int sm2d_get_lists(sm2d_handle h, uint32_t* active, int* na, uint32_t* coarse, int* nc) {
    if (!h || !na || !nc) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    *na = h->it_host->done ? 0 : h->it_host->n_active;
    *nc = h->it_host->done ? 0 : h->it_host->n_coarse;
    if (active && *na) CK(cudaMemcpyAsync(active, h->d.active, sizeof(uint32_t) * *na, cudaMemcpyDeviceToHost, h->s));
    if (coarse && *nc) CK(cudaMemcpyAsync(coarse, h->d.coarse, sizeof(uint32_t) * *nc, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int sm2d_get_tallies(sm2d_handle h, double* edep, float* w_cut, double* e_cut, float* w_nuc, double* e_nuc,
                     float* w_bnd, double* e_bnd) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    const size_t n = (size_t)h->d.Nc;
    const Dev& d = h->d;
    if (edep) CK(cudaMemcpyAsync(edep, d.edep, n * 8, cudaMemcpyDeviceToHost, h->s));
    if (w_cut) CK(cudaMemcpyAsync(w_cut, d.w_cut, n * 4, cudaMemcpyDeviceToHost, h->s));
    if (e_cut) CK(cudaMemcpyAsync(e_cut, d.e_cut, n * 8, cudaMemcpyDeviceToHost, h->s));
    if (w_nuc) CK(cudaMemcpyAsync(w_nuc, d.w_nuc, n * 4, cudaMemcpyDeviceToHost, h->s));
    if (e_nuc) CK(cudaMemcpyAsync(e_nuc, d.e_nuc, n * 8, cudaMemcpyDeviceToHost, h->s));
    if (w_bnd) CK(cudaMemcpyAsync(w_bnd, d.w_bnd, n * 4, cudaMemcpyDeviceToHost, h->s));
    if (e_bnd) CK(cudaMemcpyAsync(e_bnd, d.e_bnd, n * 8, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int sm2d_get_audit(sm2d_handle h, sm2d_audit* out) {
    if (!h || !out) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    *out = h->it_host->last;
    return 0;
}

int sm2d_get_audit_history(sm2d_handle h, sm2d_audit* out, int max_entries, int* n) {
    if (!h || !out || !n) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    *n = std::min(std::min(h->it_host->iter, h->d.hist_cap), max_entries);
    if (*n > 0) CK(cudaMemcpyAsync(out, h->d.hist, sizeof(sm2d_audit) * *n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int sm2d_get_scalars(sm2d_handle h, double* o) {
    if (!h || !o) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    const IterState& it = *h->it_host;
    o[0] = it.transport_drop_w; o[1] = it.transport_drop_e; o[2] = it.audit_residual;
    o[3] = it.src_inj_w; o[4] = it.src_inj_e; o[5] = it.src_oog_w; o[6] = it.src_oog_e;
    o[7] = it.src_slot_w; o[8] = it.src_slot_e; o[9] = it.src_rep_loss;
    o[10] = it.iter; o[11] = it.cell_steps; o[12] = it.slots_in; o[13] = it.slots_out;
    o[14] = it.cand_ovf; o[15] = it.cand_miss; o[16] = it.bin_ovf;
    return 0;
}

int sm2d_get_fe(sm2d_handle h, float* A, float* B, float* S) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    const size_t n = h->feA.size();
    if (A) memcpy(A, h->feA.data(), n * 4);
    if (B) memcpy(B, h->feB.data(), n * 4);
    if (S) memcpy(S, h->feS.data(), n * 4);
    return 0;
}

static int enqueue_dose(Ctx& c) {
    const int n = c.d.Nc;
    k_dose<<<(n + 255) / 256, 256, 0, c.s>>>(c.d.edep, c.dose_half, c.dose_ker, c.dose_stride, c.d.Nx, c.d.Nz,
                                             c.dose_dev);
    CK(cudaGetLastError());
    return 0;
}

int sm2d_get_dose(sm2d_handle h, double* dose) {
    if (!h || !dose) return fail(SM2D_ERR_ARG, "null argument");
    int rc = enqueue_dose(*h);
    if (rc) return rc;
    CK(cudaMemcpyAsync(dose, h->dose_dev, sizeof(double) * h->d.Nc, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

void* sm2d_stream(sm2d_handle h) { return h ? (void*)h->s : nullptr; }

int sm2d_reset(sm2d_handle h) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    int rc = DISPATCH(c, clear_all, 0);
    if (rc) return rc;
    const size_t n = (size_t)c.d.Nc;
    CK(cudaMemsetAsync(c.d.edep, 0, n * 8, c.s));
    CK(cudaMemsetAsync(c.d.e_cut, 0, n * 8, c.s));
    CK(cudaMemsetAsync(c.d.e_nuc, 0, n * 8, c.s));
    CK(cudaMemsetAsync(c.d.e_bnd, 0, n * 8, c.s));
    CK(cudaMemsetAsync(c.d.w_cut, 0, n * 4, c.s));
    CK(cudaMemsetAsync(c.d.w_nuc, 0, n * 4, c.s));
    CK(cudaMemsetAsync(c.d.w_bnd, 0, n * 4, c.s));
    CK(cudaMemsetAsync(c.d.cls, 0, n, c.s));
    k_reset_state<<<1, 1, 0, c.s>>>(c.d.it);
    k_wipe<<<c.grid_cell, kThreads, 0, c.s>>>(c.d, c.ctab_words, 5 * c.d.Nc);
    CK(cudaGetLastError());
    c.injected = false;
    return 0;
}

int sm2d_inject_async(sm2d_handle h, const sm2d_beam* b) {
    if (!h || !b) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    const bool gaussian = (b->n_samples > 1) || (b->sigma_x > 0.0f) || (b->sigma_theta > 0.0f);
    if (gaussian && b->n_samples <= 0) return fail(SM2D_ERR_ARG, "n_samples must be positive");
    // the beam travels as-is (host struct -> device); x_min/z_min come from the problem
    static_assert(sizeof(sm2d_beam) == 10 * 4, "beam layout");
    CK(cudaMemcpyAsync(c.beam_dev, b, 8 * sizeof(float), cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(reinterpret_cast<char*>(c.beam_dev) + offsetof(BeamArgs, n), &b->n_samples,
                       sizeof(int) + sizeof(unsigned), cudaMemcpyHostToDevice, c.s));
    CK(cudaMemsetAsync(&c.d.it->src_inj_w, 0, offsetof(IterState, last) - offsetof(IterState, src_inj_w), c.s));
    int rc = DISPATCH(c, inject_dev, b->n_samples, gaussian);
    if (rc) return rc;
    if ((rc = DISPATCH(c, totals, 0))) return rc;
    k_source_finalize<<<1, 1, 0, c.s>>>(c.d.it, c.beam_dev, gaussian ? 1 : 0);
    CK(cudaGetLastError());
    c.injected = true;
    return 0;
}

int sm2d_run_async(sm2d_handle h, int max_it) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space: call sm2d_inject or sm2d_set_psi_in first");
    if (max_it <= 0) return fail(SM2D_ERR_ARG, "max_iterations must be positive");
    int rc = build_graph(c);
    if (rc) return rc;
    k_set_iter_limit<<<1, 1, 0, c.s>>>(c.d.it, max_it);
    CK(cudaGetLastError());
    CK(cudaGraphLaunch(c.exec, c.s));
    return 0;
}

int sm2d_dose_async(sm2d_handle h, double* host_dose) {
    if (!h || !host_dose) return fail(SM2D_ERR_ARG, "null argument");
    int rc = enqueue_dose(*h);
    if (rc) return rc;
    CK(cudaMemcpyAsync(host_dose, h->dose_dev, sizeof(double) * h->d.Nc, cudaMemcpyDeviceToHost, h->s));
    return 0;
}

int sm2d_run_profiled(sm2d_handle h, int n, int* done_iters, float* ms7, int* launches) {
    if (!h || !ms7 || n <= 0) return fail(SM2D_ERR_ARG, "invalid argument");
    Ctx& c = *h;
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space");
    int rc = sync_state(c);
    if (rc) return rc;
    const int start = c.it_host->iter;
    constexpr int E = 8;   // events per iteration
    const size_t need = (size_t)E * n;
    while (c.pev.size() < need) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        c.pev.push_back(e);
    }
    cudaEvent_t saved[E];
    memcpy(saved, c.ev, sizeof saved);
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < E; ++k) c.ev[k] = c.pev[(size_t)E * i + k];
        if ((rc = DISPATCH(c, launch_body, true, false, false))) break;
    }
    memcpy(c.ev, saved, sizeof saved);
    if (rc) return rc;
    if ((rc = sync_state(c))) return rc;
    const int done = c.it_host->iter - start;
    for (int k = 0; k < E - 1; ++k) ms7[k] = 0.0f;
    for (int i = 0; i < done; ++i)
        for (int k = 0; k < E - 1; ++k) {
            float t = 0.0f;
            CK(cudaEventElapsedTime(&t, c.pev[(size_t)E * i + k], c.pev[(size_t)E * i + k + 1]));
            ms7[k] += t;
        }
    if (done_iters) *done_iters = done;
    if (launches) *launches = done * (c.p.use_buckets ? 7 : 6);
    return 0;
}

int sm2d_get_step_timing(sm2d_handle h, float* ms7) {
    if (!h || !ms7) return fail(SM2D_ERR_ARG, "null argument");
    memcpy(ms7, h->step_ms, sizeof h->step_ms);
    return 0;
}

}  // extern "C"
