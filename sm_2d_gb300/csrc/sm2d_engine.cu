// sm2d_engine.cu -- kernels, device-resident iteration loop and C ABI of the
// SM_2D transport step on GB300 (sm_103a).
//
// The engine holds B lanes, B independent spots stacked in one set of arrays
// (gc = lane * Nc + cell).  One pass of the iteration -- the body of the
// reference host loop k1k6_pipeline.cu:1606-2038 -- transports every lane
// that still has work, with these kernels, all counts read from device
// memory:
//   k_classify         K1 mask and classes of the occupied cells, cell list,
//                      the w > 0 bins of the listed cells copied into the bin
//                      list (psi_in is cleared as it is read), stopping rules,
//                      device loop condition
//   k_transport<KEYS>  K2/K3 per bin: the block ids each emission claims,
//                      with their sequential claim keys
//   k_select_buckets   bucket slots, then K4's claims on psi_out
//   k_select_psi       psi_out slots
//   k_transport<...>   K2/K3 per bin again, depositing into psi_out (fused K4)
//                      or into the DeviceOutflowBucket array (then
//                      k_bucket_push = K4_BucketTransfer)
//   k_finalize         K5 audit per lane, K6 swap
// sm2d_run and the batch entries capture the pass once into a CUDA graph
// whose while-conditional node repeats it on the device until no lane has
// work.  The single-spot entries drive lane 0 of a one-lane engine.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sm2d.h"
#include "sm2d_common.cuh"
#include "sm2d_device.cuh"
#include "sm2d_tables.h"
#include "sm2d_transport.cuh"

namespace sm2d {


// Per-lane sums of a block staged in shared memory, flushed with one atomic
// per (lane, value) at the end of the block.
template <int N>
struct LaneSums {
    double v[kMaxLanes][N];
    __device__ void zero(int B) {
        for (int i = threadIdx.x; i < B * N; i += blockDim.x) (&v[0][0])[i] = 0.0;
    }
    __device__ void flush(const Dev& d, int first) {   // into LaneState doubles starting at `first`
        for (int i = threadIdx.x; i < d.B * N; i += blockDim.x) {
            const double x = (&v[0][0])[i];
            if (x != 0.0) atomicAdd(reinterpret_cast<double*>(d.ls + i / N) + first + i % N, x);
        }
    }
};
// index of a LaneState double member, for LaneSums::flush
#define LANE_DOUBLE(member) ((int)(offsetof(LaneState, member) / sizeof(double)))

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

__device__ __forceinline__ bool beam_gaussian(const BeamArgs& b) {   // gpu_transport_wrapper.cu:246
    return b.kind == 0 && (b.n > 1 || b.sx > 0.0f || b.sth > 0.0f);
}
__device__ __forceinline__ int beam_samples(const BeamArgs& b) {
    return b.kind == 1 ? b.n : beam_gaussian(b) ? max(b.n, 0) : 1;
}

// The quadrature source's angular nodes and weights, the reference's own
// 7-point table (k1k6_pipeline.cu:316-318).
__constant__ float kGhAbscissa[7] = {-2.65f, -1.67f, -0.82f, 0.0f, 0.82f, 1.67f, 2.65f};
__constant__ float kGhWeight[7] = {0.0105f, 0.0769f, 0.2448f, 0.3357f, 0.2448f, 0.0769f, 0.0105f};

// One source sample: inject_source_kernel's pencil branch
// (k1k6_pipeline.cu:325-343), sample i of inject_gaussian_source_kernel
// (k1k6_pipeline.cu:451-551) or sample i of inject_source_kernel's
// distributed branch (k1k6_pipeline.cu:345-427: i = angle node * cells +
// cell, the kernel's loop order), placed as device_psic_inject_source does
// (device_psic.cuh:347-450: clamp into the cell, sub-cell bins, nearest
// global bins).  Returns false when the sample leaves the grid.
struct InjSample {
    int cell, l;   // lane-local cell
    uint32_t want;
    float w, E;
};
template <class Lay>
__device__ bool inject_sample(const Dev& d, const BeamArgs& b, float x_min, float z_min, int i, InjSample& o) {
    float theta, E, x, z;
    if (b.kind == 1) {
        // Gaussian weight of each cell centre over the cell range, normalised
        // by their float sum in cell order; angle nodes when sigma_theta > 1e-4
        const int it = i / b.q_nx, ix = b.q_ix0 + i % b.q_nx;
        float total = 0.0f;
        for (int k = b.q_ix0; k < b.q_ix0 + b.q_nx; ++k) {
            const float dxb = (x_min + ((float)k + 0.5f) * d.dx) - b.x0;
            total += sm2d_expf(-0.5f * dxb * dxb / (b.sx * b.sx)) * d.dx;
        }
        if (total <= 0.0f) total = 1.0f;
        const float dxb = (x_min + ((float)ix + 0.5f) * d.dx) - b.x0;
        const float w_x = (sm2d_expf(-0.5f * dxb * dxb / (b.sx * b.sx)) * d.dx) / total;
        const bool ang = b.sth > 0.0001f;
        theta = ang ? b.theta0 + kGhAbscissa[it] * b.sth : b.theta0;
        const float w_t = ang ? kGhWeight[it] : 1.0f;
        const float zr = b.z0 - z_min;
        int cz = (int)(zr / d.dz);
        cz = cz < 0 ? 0 : (cz >= d.Nz ? d.Nz - 1 : cz);
        o.cell = cz * d.Nx + ix;
        o.w = b.W * w_t * w_x;
        E = b.E0;
        x = d.dx * 0.5f;
        z = zr - cz * d.dz;
    } else if (!beam_gaussian(b)) {
        const float xr = b.x0 - x_min, zr = b.z0 - z_min;
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
        const float xr = xs - x_min, zr = b.z0 - z_min;
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
    int Eb = find_ebin(d, E);
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

// Opens an injection into the lanes whose beam has samples: one claim pass.
// check_empty (single-lane engines) refuses an injection into an occupied
// phase space: every sample is then booked as a source slot drop.  The
// injected cells are appended to psi_in's occupancy list from occ_mark on.
__global__ void k_inject_begin(Dev d, int check_empty) {
    if (threadIdx.x || blockIdx.x) return;
    d.gs->ctag += 1u;
    d.gs->occ_mark = d.gs->occ_n[d.gs->parity];
    d.ls[0].inj_skip = (check_empty && d.gs->occ_n[d.gs->parity] != 0) ? 1 : 0;
}

// Claim pass of the injection: each in-grid sample offers its block to its
// cell with its sample index as claim key (the reference's source kernels
// claim in sample order when run one sample at a time).  Blocks (x, lane),
// grid-stride over the lane's samples; with refill_only, only the lanes a
// plan refills.
template <class Lay>
__global__ void k_inject_keys(Dev d, const BeamArgs* beams, float x_min, float z_min, int refill_only) {
    const int lane = blockIdx.y;
    if ((refill_only && !d.ls[lane].refill) || d.ls[lane].inj_skip) return;
    const BeamArgs b = beams[lane];
    const int ns = beam_samples(b);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        InjSample o;
        if (!inject_sample<Lay>(d, b, x_min, z_min, i, o) || !(o.w > 0.0f)) continue;
        const int gc = lane * d.Nc + o.cell;
        cand_insert(psi_row(d, gc), d.ccount + gc, d.gs->ctag, o.want, (uint32_t)i, &d.gs->cand_ovf);
        mark_occupied(d, d.gs->parity, gc);
    }
}

// Deposit pass of the injection: a sample whose block kept a slot adds its
// weight there; the others are source slot drops (the reference's claim
// without fallback).  The pencil books W and E0 W in k_source_finalize.
template <class Lay>
__global__ void k_inject_deposit(Dev d, const BeamArgs* beams, float x_min, float z_min, int refill_only) {
    const int lane = blockIdx.y;
    LaneState& L = d.ls[lane];
    if (refill_only && !L.refill) return;
    const BeamArgs b = beams[lane];
    const int ns = beam_samples(b);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        InjSample o;
        const bool in = inject_sample<Lay>(d, b, x_min, z_min, i, o);
        const int gc = lane * d.Nc + o.cell;
        int s = -1;
        if (in && !L.inj_skip && o.w > 0.0f) {
            uint32_t sel;
            s = cand_find(psi_row(d, gc), d.gs->ctag, o.want, sel);
            if (s >= 0 && sel != o.want) s = -1;   // folded into another block: a slot drop
        }
        if (s >= 0) vadd(d, page_of<true>(d, gc, s), Lay::L, o.l, o.w);
        if (!beam_gaussian(b)) continue;
        if (!in) {
            atomicAdd(&L.src_oog_w, o.w);
            atomicAdd(&L.src_oog_e, (double)(o.E * o.w));
        } else if (s >= 0) {
            atomicAdd(&L.src_inj_w, o.w);
            atomicAdd(&L.src_inj_e, (double)(o.E * o.w));
        } else {
            atomicAdd(&L.src_slot_w, o.w);
            atomicAdd(&L.src_slot_e, (double)(o.E * o.w));
        }
    }
}

// Weight and bin-centre energy of the w > 0 bins of the cells the last
// injection put on psi_in's occupancy list (compute_psic_total_weight_energy,
// k1k6_pipeline.cu:706-768), per lane; warp per cell.
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_totals(Dev d) {
    const int k = d.gs->parity;
    const int n = d.gs->occ_n[k];
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int wi = d.gs->occ_mark + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); wi < n; wi += nw) {
        const int gc = d.occ_list[k][wi];
        const uint32_t b = d.bid[(size_t)gc * kKb + lane];
        unsigned used = __ballot_sync(kFull, b != kEmpty);
        double W = 0.0, E = 0.0;
        while (used) {
            const int s = __ffs(used) - 1;
            used &= used - 1;
            const uint32_t bs = __shfl_sync(kFull, b, s);
            const float* v = d.val + page_of<true>(d, gc, s) * Lay::L;
            for (int l = lane; l < Lay::L; l += 32) {
                const float w = v[l];
                if (w <= 0.0f) continue;
                int Eb = (int)((bs >> 12) & 0xFFFu) * Lay::NE + (l / Lay::NT) % Lay::NE;
                Eb = max(0, min(Eb, d.N_E - 1));
                W += (double)w;
                E += (double)w * (double)e_center(d, Eb);
            }
        }
        W = warp_sum(W);
        E = warp_sum(E);
        if (lane == 0 && (W != 0.0 || E != 0.0)) {
            LaneState& L = d.ls[lane_of(d, gc)];
            atomicAdd(&L.tot_w, W);
            atomicAdd(&L.tot_e, E);
        }
    }
}

// Source accounting after an injection (gpu_transport_wrapper.cu:339-460):
// the pencil books W and E0 W; the represented energy comes from k_totals.
// Thread per lane (the refilled lanes only, with refill_only).
__global__ void k_source_finalize(Dev d, const BeamArgs* beams, int refill_only) {
    const int lane = blockIdx.x * blockDim.x + threadIdx.x;
    if (lane >= d.B) return;
    LaneState& L = d.ls[lane];
    if (refill_only && !L.refill) return;
    L.refill = 0;
    const BeamArgs b = beams[lane];
    if (!beam_gaussian(b)) {
        L.src_inj_w = b.W;
        L.src_inj_e = (double)b.E0 * (double)b.W;
    }
    double loss = L.src_inj_e - L.tot_e;
    if (fabs(loss) < 1e-12) loss = 0.0;
    L.src_rep_loss = loss;
    L.include_source = 1;
    L.done = 0;
    L.light = 0;
}

// Sum N per-thread values over the block and add them to dst[0..N) with one
// atomic per value.
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
// compact_coarse_list k1k6_pipeline.cu:625-665), its place in this pass's
// cell list and bucket map, and, for a listed cell, its w > 0 bins appended
// to the bin list (contiguous per cell, by slot and local bin).  Only the
// float4s the slots' occupancy masks mark are read (the others hold zeros):
// each lane lists its slot's marked float4s in the warp's shared list, and
// the warp then reads the list as a flat run, U loads in flight per lane.
// The marked float4s and the masks are then cleared, so that the storage
// can receive psi_out.  A lane whose stopping rule was met consumes its
// cells without transport.  The last block publishes the counts, settles
// each lane, resets the per-lane accumulators and sets the device loop
// condition; in a spot plan it also lists the lanes whose spot just
// finished and sets the refill condition.
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_classify(Dev d, cudaGraphConditionalHandle cond,
                                                       cudaGraphConditionalHandle rcond, int use_cond) {
    constexpr int Q = Lay::L / 4, NW = kThreads / 32, U = 4;
    static_assert(Q <= 64, "a slot's occupancy mask has 64 bits");
    __shared__ int s_cnt[kMaxLanes][3];   // listed active, listed coarse, their slots
    __shared__ int s_last;
    __shared__ uint16_t s_f4[NW][kKb * Q];   // the warp's cell: marked float4s, slot << 6 | float4
    IterGlobal* gs = d.gs;
    if (gs->pass >= gs->max_pass) {   // paused: leave the phase space as it is
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            gs->halt = 1;
            if (use_cond) {
                cudaGraphSetConditional(cond, 0u);
                cudaGraphSetConditional(rcond, 0u);
            }
        }
        return;
    }
    const int par = gs->parity;
    const int nocc = gs->occ_n[par];
    const unsigned long long g = gs->gen + 1;   // number of this classification
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    uint16_t* fl = s_f4[wid];
    for (int i = threadIdx.x; i < d.B * 3; i += blockDim.x) (&s_cnt[0][0])[i] = 0;
    __syncthreads();
    for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < nocc; wi += nw) {
        const int c = d.occ_list[par][wi];
        // the cell's value pages: slot s in page pg0 + s (pages past the
        // cell's own run belong to other cells or to the overflow pages, and
        // only the used slots' masks and values are taken)
        const int pg0 = __ldcg(d.occ_pg[par] + wi);
        const int ln = lane_of(d, c);
        const bool light = d.ls[ln].light != 0;
        uint32_t* ids = d.bid + (size_t)c * kKb;
        const int page = pg0 + lane;
        const uint32_t b = ids[lane];
        const uint2 mw = __ldcg(d.vmask + page);
        const bool used = b != kEmpty;
        const unsigned long long mk = used ? ((unsigned long long)mw.y << 32) | mw.x : 0ull;
        const uint32_t be = (b >> 12) & 0xFFFu;
        const bool c_on = __any_sync(kFull, used && be <= (uint32_t)d.b_on);
        const bool c_off = __any_sync(kFull, used && be <= (uint32_t)d.b_off);
        const unsigned um = __ballot_sync(kFull, used);
        // the marked float4s of the cell as one list, by slot and float4
        const int nm = __popcll(mk);
        int pm = nm;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, pm, o);
            if (lane >= o) pm += y;
        }
        const int M = __shfl_sync(kFull, pm, 31);
        pm -= nm;
        __syncwarp();   // the previous cell's list is no longer read
        for (unsigned long long m = mk; m;) {
            const int q = __ffsll((long long)m) - 1;
            m &= m - 1;
            fl[pm++] = (uint16_t)((lane << 6) | q);
        }
        __syncwarp();
        const float4* vc = reinterpret_cast<const float4*>(d.val) + (size_t)pg0 * Q;
        float ws = 0.0f;
        int nz = 0;
        for (int f0 = 0; f0 < M; f0 += 32 * U) {
            float4 r[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int f = f0 + 32 * u + lane;
                const int e = f < M ? fl[f] : 0;
                r[u] = f < M ? __ldcg(vc + (e >> 6) * Q + (e & 63)) : z4;
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
        const bool act = !light && (c_on || (prev && c_off)) && ws > d.wmin;
        const int cls = light ? 0 : (act ? 2 : (hw ? 1 : 0));
        int base = 0, in_list = 0;
        if (lane == 0) {
            d.cls[c] = (uint8_t)cls;
            if (act) d.act_gen[c] = g;
            if (cls) {
                // the cell's list position and its first bin in one reservation
                const unsigned long long o = atomicAdd(&gs->acc_lb, (1ull << 32) | (unsigned)nz);
                const int idx = (int)(o >> 32);
                base = (int)(uint32_t)o;
                if (idx < d.listed_cap) {
                    d.listed[idx] = (uint32_t)c;
                    d.c2b[c] = 4 * idx;
                    d.cell_bins[idx] = make_int2(base, nz);
                    in_list = 1;
                }
                atomicAdd(&s_cnt[ln][act ? 0 : 1], 1);
                atomicAdd(&s_cnt[ln][2], __popc(um));
            }
        }
        if (cls) {
            const int idx_ok = __shfl_sync(kFull, in_list, 0);
            base = __shfl_sync(kFull, base, 0);
            if (!idx_ok || base + nz > d.bins_cap) {   // no room: the last block stops the run
                if (lane == 0) atomicAdd(&gs->bin_ovf, 1);
            } else {
                // seed slot of each claimed slot: the rank of its block id
                // (seed_slot_mode 1), or the storage slot itself as the
                // reference's seeds take it (0)
                int rk = 0;
                for (int t = 0; t < kKb; ++t) {
                    const uint32_t bt = __shfl_sync(kFull, b, t);
                    rk += (bt != kEmpty && bt < b) ? 1 : 0;
                }
                if (!d.seed_mode) rk = lane;
                const uint32_t k3 = cls == 2 ? 1u : 0u;
                int off = base;
                for (int f0 = 0; f0 < M; f0 += 32 * U) {
                    float4 r[U];
                    int e[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {   // all loads first (L2 hits of the first read)
                        const int f = f0 + 32 * u + lane;
                        e[u] = f < M ? fl[f] : 0;
                        r[u] = f < M ? __ldcg(vc + (e[u] >> 6) * Q + (e[u] & 63)) : z4;
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int s = e[u] >> 6, q = e[u] & 63;
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
                                d.bins[p++] = make_uint4((uint32_t)c, meta | ((uint32_t)(4 * q + k) << 10),
                                                         __float_as_uint(c4[k]), bs);
                        off += __shfl_sync(kFull, inc, 31);
                    }
                }
            }
        }
        // psi_in of the cell is consumed: its pages return to zeros
        float4* vw = reinterpret_cast<float4*>(d.val) + (size_t)page * Q;
        for (unsigned long long m = mk; m;) {
            const int q = __ffsll((long long)m) - 1;
            m &= m - 1;
            __stcs(vw + q, z4);
        }
        if (used && (mw.x | mw.y)) d.vmask[page] = make_uint2(0u, 0u);
        ids[lane] = kEmpty;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < d.B; i += blockDim.x) {
        if (s_cnt[i][0]) atomicAdd(&d.ls[i].acc_active, s_cnt[i][0]);
        if (s_cnt[i][1]) atomicAdd(&d.ls[i].acc_coarse, s_cnt[i][1]);
        if (s_cnt[i][2]) atomicAdd(&d.ls[i].acc_slots, s_cnt[i][2]);
    }
    // the block's writes before its count (one fence after the barrier, by
    // the thread that counts: the barrier orders the others' writes before it)
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&gs->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // settle each lane: counts, C1 stopping rule, accumulators
    __shared__ int s_work, s_items;
    __shared__ uint8_t s_fin[kMaxLanes];
    const bool plan = gs->plan_n > 0;
    if (threadIdx.x == 0) s_work = s_items = 0;
    __syncthreads();
    for (int ln = threadIdx.x; ln < d.B; ln += blockDim.x) {
        LaneState& L = d.ls[ln];
        volatile LaneState* v = &L;
        const bool was_running = v->done == 0;
        const int na = v->acc_active, nc = v->acc_coarse, nsl = v->acc_slots;
        L.acc_active = L.acc_coarse = L.acc_slots = 0;
        if (nsl) atomicAdd(&s_items, nsl);
        // every psi_in page of the lane is cleared: its region starts again
        atomicMax(&gs->pool_peak, L.pool_top);
        L.pool_top = 0;
        if (L.light) {
            // in-flight weight below a fraction of the injected weight ends
            // the spot; the rest is booked as a terminal transport drop
            // (k1k6_pipeline.cu:1677-1706 books it too)
            L.transport_drop_w += L.last.W_out_total;
            L.transport_drop_e += L.last.E_out_total;
            L.light = 0;
        }
        L.n_active = na;
        L.n_coarse = nc;
        const bool work = (na + nc) > 0;
        L.done = work ? 0 : 1;
        L.work = work ? 1 : 0;
        s_fin[ln] = (plan && was_running && !work) ? 1 : 0;
        double* acc = &L.drop_w;   // the 14 per-iteration accumulators
        for (int k = 0; k < 14; ++k) acc[k] = 0.0;
        if (work) {
            L.cell_steps += (double)(na + nc);
            L.slots_in += (double)nsl;
            atomicAdd(&s_work, 1);
        }
    }
    __syncthreads();
    // the finished lanes, ascending (warp 0, 32 lanes a step)
    if (threadIdx.x >= 32) return;
    int nf = 0;
    for (int l0 = 0; l0 < d.B; l0 += 32) {
        const int ln = l0 + (int)threadIdx.x;
        const bool f = ln < d.B && s_fin[ln];
        const unsigned m = __ballot_sync(kFull, f);
        if (f) gs->fin[nf + __popc(m & ((1u << threadIdx.x) - 1u))] = ln;
        nf += __popc(m);
    }
    if (threadIdx.x != 0) return;
    volatile IterGlobal* v = gs;
    const unsigned long long lb = v->acc_lb;
    const int nl = (int)(lb >> 32), ni = s_items, nb = (int)(uint32_t)lb;
    gs->acc_lb = 0ull;
    gs->gen = g;
    gs->ctag += 1u;   // claim pass of this iteration
    gs->n_fin = nf;
    // a cell or bin list that outgrew its capacity ends the run (reported by
    // the host API as SM2D_ERR_ALLOC); a plan runs on while a spot finished
    // (its lane is refilled at the end of this pass)
    const bool halt = (s_work == 0 && nf == 0) || v->bin_ovf != 0;
    gs->halt = halt ? 1 : 0;
    gs->n_listed = halt ? 0 : min(nl, d.listed_cap);
    gs->n_items = halt ? 0 : ni;
    gs->n_bins = halt ? 0 : nb;
    gs->k3_total += (unsigned long long)min(max(v->k3_rows, 0), d.k3_cap);   // the last pass's surrogate rows
    gs->k3_rows = 0;
    if (!halt) gs->bins_total += (unsigned long long)nb;
    gs->blocks_done = 0;
    if (use_cond) {
        cudaGraphSetConditional(cond, (!halt && gs->pass + 1 < gs->max_pass) ? 1u : 0u);
        cudaGraphSetConditional(rcond, (!halt && nf > 0) ? 1u : 0u);
    }
}

// The claims of the bins that took a surrogate row in the claim pass, from
// the network's table of each row (or the closed forms where the row fell
// back), thread per row.  The claim keys are the bins' own sequential keys,
// so the claim tables end as if the claim pass had emitted them.
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_surr_keys(Dev d) {
    IterGlobal* gs = d.gs;
    if (gs->halt) return;
    const int par = gs->parity;
    const int n = min(gs->k3_rows, d.k3_cap);
    const uint32_t tag = gs->ctag;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        const unsigned am = __activemask();
        const unsigned fbm = __ballot_sync(am, __ldcg(d.kfb + row) != 0);
        if ((threadIdx.x & 31) == __ffs(am) - 1 && fbm) atomicAdd(&gs->k3_fb, (unsigned long long)__popc(fbm));
        const int i = __ldcg(d.kbin + row);
        const uint4 r = __ldcg(d.bins + i);
        const int cell = (int)r.x;
        const int ln = lane_of(d, cell);
        const int slot = (int)(r.y & 31u), sslot = (int)((r.y >> 5) & 31u), lidx = (int)((r.y >> 10) & 0xFFu);
        const bool k3 = ((r.y >> 18) & 1u) != 0;
        const unsigned salt = d.salt ? (unsigned)d.ls[ln].iter * 0x9E3779B9u : 0u;
        Tally t{};
        transport_bin<Lay, PASS_KEYS, true>(d, i, par, k3, cell, ln, cell - ln * d.Nc, r.w, slot, sslot, lidx,
                                            __uint_as_float(r.z), salt, tag, t, true);
    }
}

// Ascending active and coarse lists of lane 0 from the classes of this pass
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
    if (!__any_sync(kFull, v != T(0))) return v;   // all zero: the sums are zero
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
// per-lane drop sums (staged per block in shared memory); psi_out's weight
// and energy for the audit are summed by the finalize kernel.  Resident blocks
// per SM: five for the claim passes (48 registers, no spills; 27.2 -> 24.1 ms
// per wave of 80 spots against four) and for the sampled form's deposit pass,
// which spills 88 bytes and still gains from the warps (175.1 -> 170.2 us a
// pass at 512 lanes; 196 at three blocks); four for the expectation form's
// and the bucket mode's deposit passes (five would spill 0.7-1 KB).
template <class Lay, int PASS, bool EXP = false>
__global__ void __launch_bounds__(kThreads, (PASS == PASS_KEYS || (PASS == PASS_DIRECT && !EXP)) ? 5 : 4) k_transport(Dev d) {
    __shared__ LaneSums<2> s_sum;   // drop_w, drop_e
    IterGlobal* gs = d.gs;
    if (gs->halt) return;
    const int par = gs->parity;
    const int n = gs->n_bins;
    const uint32_t tag = gs->ctag;
    const int lane = threadIdx.x & 31;
    if (PASS != PASS_KEYS) {
        s_sum.zero(d.B);
        __syncthreads();
    }
    const int stride = gridDim.x * blockDim.x;
    for (int w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < n; w0 += stride) {
        const int i = w0 + lane;
        Tally t{};
        int cell = -1;
        if (i < n) {
            // the claim pass keeps the list in L2 for the deposit pass
            const uint4 r = PASS == PASS_KEYS ? __ldcg(d.bins + i) : __ldcs(d.bins + i);
            cell = (int)r.x;
            const int ln = lane_of(d, cell);
            const int slot = (int)(r.y & 31u), sslot = (int)((r.y >> 5) & 31u), lidx = (int)((r.y >> 10) & 0xFFu);
            const bool k3 = ((r.y >> 18) & 1u) != 0;
            const unsigned salt = d.salt ? (unsigned)d.ls[ln].iter * 0x9E3779B9u : 0u;
            transport_bin<Lay, PASS, EXP>(d, i, par, k3, cell, ln, cell - ln * d.Nc, r.w, slot, sslot, lidx,
                                          __uint_as_float(r.z), salt, tag, t);
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
            const double dw = seg_sum(t.drop_w, same), de = seg_sum(t.drop_e, same);
            const int prev_cell = __shfl_up_sync(kFull, cell, 1);
            if (cell >= 0 && (lane == 0 || prev_cell != cell)) {
                if (edep != 0.0) atomicAdd(d.dl_edep + cell, edep);
                if (ecut != 0.0) atomicAdd(d.dl_ecut + cell, ecut);
                if (enuc != 0.0) atomicAdd(d.dl_enuc + cell, enuc);
                if (ebnd != 0.0) atomicAdd(d.dl_ebnd + cell, ebnd);
                if (wcut != 0.0f) atomicAdd(d.dl_wcut + cell, wcut);
                if (wnuc != 0.0f) atomicAdd(d.dl_wnuc + cell, wnuc);
                if (wbnd != 0.0f) atomicAdd(d.dl_wbnd + cell, wbnd);
                if (dw != 0.0 || de != 0.0) {
                    double* ls = s_sum.v[lane_of(d, cell)];
                    atomicAdd(ls + 0, dw);
                    atomicAdd(ls + 1, de);
                }
            }
        }
    }
    if (PASS != PASS_KEYS) {
        __syncthreads();
        s_sum.flush(d, LANE_DOUBLE(drop_w));
    }
}

// Per-cell tallies of the transported bins of listed cell idx (its
// contiguous run of the bin list), by one warp: the psi_in weight and
// bin-centre energy of every bin, and for the bins that took a step (past the
// prune and cutoff checks) the deposit and the nuclear loss from their step
// records.  One warp reduction per cell instead of one per 32 bins in the
// deposit pass; the bucket selection runs it for each cell's first face.
template <class Lay, int NS>
__device__ __forceinline__ void tally_cell(const Dev& d, int idx, int lane, LaneSums<NS>& s_sum, double* s_prune) {
    const int2 r = d.cell_bins[idx];
    const int c = (int)d.listed[idx];
    const float4* rec = reinterpret_cast<const float4*>(d.brec);
    double Wi = 0.0, Ei = 0.0, ed = 0.0, en = 0.0, pw = 0.0, pe = 0.0;
    float wn = 0.0f;
    int pn = 0, k3c = 0;
    // U bins per lane in flight: their list entries and step records
    // together, then the bin-centre energies (sums in bin order per lane)
    constexpr int U = 4;
    const int end = r.x + r.y;
    for (int i0 = r.x + lane; i0 < end; i0 += 32 * U) {
        uint4 bb[U];
        float4 rr[U];   // z, sigma, deposit, nuclear weight
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + 32 * u;
            bb[u] = i < end ? __ldcg(d.bins + i) : make_uint4(0u, 0u, 0u, 0u);
            rr[u] = i < end ? __ldcg(rec + 2 * (size_t)i + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (i0 + 32 * u >= end) continue;
            const uint4 b = bb[u];
            const bool k3 = ((b.y >> 18) & 1u) != 0;
            const int lidx = (int)((b.y >> 10) & 0xFFu);
            const float w = __uint_as_float(b.z);
            int tl, El, xs, zs;
            Lay::dec(lidx, tl, El, xs, zs);
            int Ebin = (int)((b.w >> 12) & 0xFFFu) * Lay::NE + El;
            if (k3) Ebin = max(0, min(Ebin, d.N_E - 1));
            const float E = d.Ee[Ebin] + 1.0f * ((d.Ee[Ebin + 1] - d.Ee[Ebin]) * 0.5f);
            Wi += (double)w;
            Ei += (double)w * (double)E;
            if (w < (k3 ? d.prune_fine : d.prune_coarse)) {   // the transport's prune drop
                pw += (double)w;
                pe += (double)(E * w);
                ++pn;
                k3c = k3;
                continue;
            }
            if (E <= 0.1f) continue;
            ed += (double)rr[u].z;
            wn += rr[u].w;
            en += (double)(rr[u].w * E);
        }
    }
    Wi = warp_sum(Wi);
    Ei = warp_sum(Ei);
    ed = warp_sum(ed);
    en = warp_sum(en);
    wn = warp_sumf(wn);
    if (__any_sync(kFull, pn != 0)) {   // a cell is of one class: K2 or K3
        const int st = __reduce_max_sync(kFull, (unsigned)k3c);
        pw = warp_sum(pw);
        pe = warp_sum(pe);
        pn = (int)__reduce_add_sync(kFull, (unsigned)pn);
        if (lane == 0) {
            atomicAdd(s_prune + 3 * st, (double)pn);
            atomicAdd(s_prune + 3 * st + 1, pw);
            atomicAdd(s_prune + 3 * st + 2, pe);
        }
    }
    if (lane == 0) {
        if (ed != 0.0) atomicAdd(d.dl_edep + c, ed);
        if (en != 0.0) atomicAdd(d.dl_enuc + c, en);
        if (wn != 0.0f) atomicAdd(d.dl_wnuc + c, wn);
        double* ls = s_sum.v[lane_of(d, c)];
        atomicAdd(ls + 0, Wi);
        atomicAdd(ls + 1, Ei);
    }
}

// ------------------------------------------------------------------ slot selection
// Selection of one claim-table row by one warp: the gathered ids ordered by
// claim key; the first 32 become slots 0..31 (written to kept[]), the rest
// fold into the nearest kept id (smallest bid_distance, lowest slot on
// ties).  Each entry's key is replaced by its slot for the deposit pass.
// Returns the number of kept ids.
struct SelScratch {
    unsigned long long kb[kCand];   // claim key << 32 | block id: the order of the row's ids
    uint8_t idx[kCand], rank[kCand];
    uint32_t kept[kKb];
};
__device__ int select_row(unsigned long long* row, int* count, uint32_t tag, SelScratch& sh, uint32_t* kept, int lane) {
    const unsigned lt = (1u << lane) - 1u;
    // every entry's id and key words in one 16-byte load, all in flight
    // together with the row's count (entries of earlier passes carry older
    // tags and are skipped)
    ulonglong2 e[kCand / 32];
#pragma unroll
    for (int q = 0; q < kCand / 32; ++q) e[q] = __ldcg(reinterpret_cast<const ulonglong2*>(row + 2 * (q * 32 + lane)));
    const bool any = *(volatile int*)count > 0;
    int n = 0;
    if (any) {
#pragma unroll
        for (int q = 0; q < kCand / 32; ++q) {
            const int i = q * 32 + lane;
            const bool cur = (uint32_t)(e[q].x >> 32) == tag;
            const unsigned m = __ballot_sync(kFull, cur);
            if (cur) {
                const int p = n + __popc(m & lt);
                sh.kb[p] = ((unsigned long long)(uint32_t)e[q].y << 32) | (uint32_t)e[q].x;
                sh.idx[p] = (uint8_t)i;
            }
            n += __popc(m);
        }
    }
    __syncwarp();
    // the rank of each gathered id by (key, id): every entry is read once
    // (one 8-byte broadcast load) and compared with the lane's entries held in
    // registers, four a lane a round
    for (int j0 = 0; j0 < n; j0 += 128) {
        unsigned long long c[4];
        int r[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = j0 + 32 * u + lane;
            c[u] = j < n ? sh.kb[j] : ~0ull;
            r[u] = 0;
        }
        for (int m = 0; m < n; ++m) {
            const unsigned long long x = sh.kb[m];
#pragma unroll
            for (int u = 0; u < 4; ++u) r[u] += x < c[u] ? 1 : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = j0 + 32 * u + lane;
            if (j < n) {
                sh.rank[j] = (uint8_t)r[u];
                if (r[u] < kKb) sh.kept[r[u]] = (uint32_t)c[u];
            }
        }
    }
    __syncwarp();
    const int nk = min(n, kKb);
    for (int j = lane; j < n; j += 32) {
        int slot = sh.rank[j];
        if (slot >= kKb) {
            const uint32_t want = (uint32_t)sh.kb[j];
            int bd = 0x7fffffff;
            for (int k = 0; k < kKb; ++k) {
                const int dd = bid_distance(sh.kept[k], want);
                if (dd < bd) { bd = dd; slot = k; }
            }
        }
        // the slot and the id it holds: a found id resolves in one probe
        const uint32_t sel = sh.rank[j] < kKb ? (uint32_t)sh.kb[j] : sh.kept[slot];
        row[2 * (int)sh.idx[j] + 1] =
            ((unsigned long long)(0xFFFFFFFFu - tag) << 32) | (uint32_t)slot | ((sel & 0xFFFFFFu) << 5);
    }
    if (kept) kept[lane] = lane < nk ? sh.kept[lane] : kEmpty;
    if (lane == 0 && any) *count = 0;
    __syncwarp();
    return nk;
}

// Buckets of this pass (warp per listed cell and face): select the kept
// ids, write them to the bucket (bucket mode: also clear its values), and
// offer them to the psi_out row of the cell behind the face in bucket-slot
// order, as K4 claims them; and the per-cell tallies of the step records.
template <class Lay, bool BUCKET>
__global__ void __launch_bounds__(kThreads) k_select_buckets(Dev d) {
    constexpr int NW = kThreads / 32;
    __shared__ SelScratch s_sel[NW];
    __shared__ LaneSums<2> s_tal;   // Win, Ein of the cell tallies
    __shared__ double s_prune[6];   // pruned components, weight, energy of K2 and K3
    IterGlobal* gs = d.gs;
    if (gs->halt) return;
    const int out = gs->parity ^ 1;
    const int n = 4 * gs->n_listed;
    const uint32_t tag = gs->ctag;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    s_tal.zero(d.B);
    if (threadIdx.x < 6) s_prune[threadIdx.x] = 0.0;
    __syncthreads();
    for (int wi = blockIdx.x * NW + wid; wi < n; wi += gridDim.x * NW) {
        const int face = wi & 3;
        const int src = (int)d.listed[wi >> 2];
        // the warp of the cell's -z face (usually without emissions) takes
        // the cell's tallies
        if (face == FACE_ZM) tally_cell<Lay>(d, wi >> 2, lane, s_tal, s_prune);
        uint32_t* kept = d.bkt_ids + (size_t)wi * kKb;
        const int nk = select_row(bucket_row(d, wi), d.ccount + (size_t)d.B * d.Nc + wi, tag, s_sel[wid], kept, lane);
        if (BUCKET) {
            unsigned char* b = d.buckets + (size_t)wi * d.bucket_bytes;
            bucket_ids(b)[lane] = lane < nk ? s_sel[wid].kept[lane] : kEmpty;
            reinterpret_cast<uint16_t*>(b + 128)[lane] = 0;
            float* v = bucket_vals(b);
            for (int k = lane; k < nk * Lay::L; k += 32) v[k] = 0.0f;
        }
        if (nk == 0) continue;
        const int ix = src % d.Nx, iz = (src / d.Nx) % d.Nz;
        int dst = -1;
        if (face == FACE_ZP && iz + 1 < d.Nz) dst = src + d.Nx;
        if (face == FACE_ZM && iz > 0) dst = src - d.Nx;
        if (face == FACE_XP && ix + 1 < d.Nx) dst = src + 1;
        if (face == FACE_XM && ix > 0) dst = src - 1;
        if (dst < 0) continue;
        const int k3 = d.cls[src] == 2 ? 1 : 0;
        if (lane < nk)
            cand_insert(psi_row(d, dst), d.ccount + dst, tag, s_sel[wid].kept[lane], k4_key(k3, face, lane),
                        &gs->cand_ovf);
        if (lane == 0) mark_occupied(d, out, dst);
    }
    __syncthreads();
    s_tal.flush(d, LANE_DOUBLE(Win));
    if (threadIdx.x < 2 && s_prune[3 * threadIdx.x] != 0.0) {
        const int st = threadIdx.x;
        atomicAdd(&gs->drops.n[st][DROP_PRUNE], (unsigned long long)s_prune[3 * st]);
        atomicAdd(&gs->drops.w[st][DROP_PRUNE], s_prune[3 * st + 1]);
        atomicAdd(&gs->drops.e[st][DROP_PRUNE], s_prune[3 * st + 2]);
    }
}

// Occupied cells of psi_out (which = 1, a transport pass) or the cells an
// injection put on psi_in's list (which = 0), warp per cell: select the kept
// ids into the cell's slot ids.  In a transport pass the warp then resolves
// the kept ids of the four bucket rows that lead into the cell (the K4 step
// of the fused deposit) to the cell's slots, once per pass instead of once
// per emitted component.
__global__ void __launch_bounds__(kThreads) k_select_psi(Dev d, int which) {
    constexpr int NW = kThreads / 32;
    __shared__ SelScratch s_sel[NW];
    __shared__ LaneSums<1> s_sum;
    IterGlobal* gs = d.gs;
    if (which && gs->halt) return;
    const int k = gs->parity ^ which;
    const int n = gs->occ_n[k];
    const uint32_t tag = gs->ctag;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    s_sum.zero(d.B);
    __syncthreads();
    for (int wi = (which ? 0 : gs->occ_mark) + blockIdx.x * NW + wid; wi < n; wi += gridDim.x * NW) {
        const int gc = d.occ_list[k][wi];
        const int nk = select_row(psi_row(d, gc), d.ccount + gc, tag, s_sel[wid], d.bid + (size_t)gc * kKb, lane);
        int pb = 0;
        if (lane == 0) {   // one page per kept slot, consecutive, from the lane's region
            const int ln = lane_of(d, gc);
            pb = d.pool_lane * d.B;   // no slot, or the region is full: the overflow pages
            if (nk > 0) {
                const int p0 = atomicAdd(&d.ls[ln].pool_top, nk);
                if (p0 + nk <= d.pool_lane) pb = ln * d.pool_lane + p0;
                else atomicAdd(&gs->bin_ovf, 1);
            }
            d.pbase[gc] = pb;
            d.occ_pg[k][wi] = pb;
        }
        if (!which) continue;
        if (lane == 0) atomicAdd(&s_sum.v[lane_of(d, gc)][0], (double)nk);
        // the four bucket rows that lead into the cell, resolved side by
        // side (each step's loads of the four in flight together): the
        // source cells' bucket bases, the rows' kept ids, their first probes
        // in this cell's claim row; the kept ids of this cell come from the
        // selection just made (shuffles, not loads)
        const int ix = gc % d.Nx, iz = (gc / d.Nx) % d.Nz;
        int src[4];
        src[FACE_ZP] = iz > 0 ? gc - d.Nx : -1;
        src[FACE_ZM] = iz + 1 < d.Nz ? gc + d.Nx : -1;
        src[FACE_XP] = ix > 0 ? gc - 1 : -1;
        src[FACE_XM] = ix + 1 < d.Nx ? gc + 1 : -1;
        int base[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) base[f] = src[f] >= 0 ? __ldcg(d.c2b + src[f]) : -1;
        uint32_t id[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) id[f] = base[f] >= 0 ? __ldcg(d.bkt_ids + (size_t)(base[f] + f) * kKb + lane) : kEmpty;
        const unsigned long long* row = psi_row(d, gc);
        ulonglong2 pr[4];
#pragma unroll
        for (int f = 0; f < 4; ++f)
            pr[f] = id[f] != kEmpty ? __ldcg(reinterpret_cast<const ulonglong2*>(row + 2 * cand_hash(id[f])))
                                    : make_ulonglong2(0ull, 0ull);
        const uint32_t kp = lane < nk ? s_sel[wid].kept[lane] : kEmpty;   // this cell's kept ids
        int os[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const unsigned long long tb = ((unsigned long long)tag << 32) | id[f];
            os[f] = -1;
            if (id[f] != kEmpty) {
                if (pr[f].x == tb) os[f] = (int)((uint32_t)pr[f].y & 31u);
                else if ((uint32_t)(pr[f].x >> 32) == tag) os[f] = cand_find(row, tag, id[f]);   // probe on
            }
            // an id the row did not gather: the nearest kept id (resolve)
            const bool miss = id[f] != kEmpty && os[f] < 0;
            if (__any_sync(kFull, miss)) {
                if (miss) atomicAdd(&d.gs->cand_miss, 1);
                int bd = 0x7fffffff;
                for (int k = 0; k < kKb; ++k) {
                    const uint32_t x = __shfl_sync(kFull, kp, k);
                    if (!miss || x == kEmpty) continue;
                    const int dd = bid_distance(x, id[f]);
                    if (dd < bd) { bd = dd; os[f] = k; }
                }
            }
        }
        pb = __shfl_sync(kFull, pb, 0);   // the cell's first page (lane 0's allocation)
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const uint32_t sel = __shfl_sync(kFull, kp, os[f] >= 0 ? os[f] : 0);
            if (base[f] >= 0)
                d.bkt_os[(size_t)(base[f] + f) * kKb + lane] =
                    bkt_slot_pack(os[f] >= 0 ? pb + os[f] : -1, os[f] >= 0 ? sel : (id[f] != kEmpty ? id[f] : kEmpty));
        }
    }
    __syncthreads();
    if (which) s_sum.flush(d, LANE_DOUBLE(slots_out_it));
}

// ------------------------------------------------------------------ bucket mode (reference structure)
// K4_BucketTransfer (k4_transfer.cu:174-333) driven from the source side:
// warp per (listed cell, face) moves that bucket into psi_out of the
// neighbour behind the face, each bucket slot into the slot its kept id
// resolved to (lidx remap when it folded into a nearer id).
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_bucket_push(Dev d) {
    __shared__ LaneSums<2> s_sum;   // drop_w, drop_e
    IterGlobal* gs = d.gs;
    if (gs->halt) return;
    const int n = 4 * gs->n_listed;
    const uint32_t tag = gs->ctag;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    s_sum.zero(d.B);
    __syncthreads();
    for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < n; wi += nw) {
        const int face = wi & 3;
        const int src = (int)d.listed[wi >> 2];
        const int ix = src % d.Nx, iz = (src / d.Nx) % d.Nz;
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
        const uint32_t* kept = d.bid + (size_t)dst * kKb;
        double g[2] = {0.0, 0.0};
        while (um) {
            const int s = __ffs(um) - 1;
            um &= um - 1;
            const uint32_t bid = __shfl_sync(kFull, sb, s);
            uint32_t sel = bid;
            const int os = resolve(d, psi_row(d, dst), kept, tag, bid, sel);
            const float* v = bv + (size_t)s * Lay::L;
            const size_t pg = os >= 0 ? page_of<true>(d, dst, os) : 0;
            float* o = os >= 0 ? d.val + pg * Lay::L : nullptr;
            double eshift = 0.0;
            for (int l = lane; l < Lay::L; l += 32) {
                const float w = v[l];
                if (w <= 0.0f) continue;
                if (os < 0) {
                    const double e = (double)e_center(d, ebin_of<Lay>(d, bid, l)) * (double)w;
                    g[0] += (double)w;
                    g[1] += e;
                    count_drop(d.gs, 2, DROP_SLOT, (double)w, e);
                    continue;
                }
                const int le = sel != bid ? remap_lidx<Lay>(l, bid, sel) : l;
                atomicAdd(o + le, w);
                vmark(d, pg, le);
                if (sel != bid && d.esplit)
                    eshift += (double)((e_center(d, ebin_of<Lay>(d, bid, l)) - e_center(d, ebin_of<Lay>(d, sel, le))) * w);
            }
            eshift = warp_sum(eshift);
            if (lane == 0 && eshift != 0.0) atomicAdd(d.dl_edep + src, eshift);
        }
        double* ls = s_sum.v[lane_of(d, src)];
        if (__any_sync(kFull, g[0] != 0.0 || g[1] != 0.0)) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const double x = warp_sum(g[k]);
                if (lane == 0 && x != 0.0) atomicAdd(ls + k, x);
            }
        }
    }
    __syncthreads();
    s_sum.flush(d, LANE_DOUBLE(drop_w));
}

// ------------------------------------------------------------------ K5 + K6
// Audit record of one lane's iteration (k5_audit.cu:22-167) from its
// accumulators, and the lane's bookkeeping.
__device__ void finalize_lane(const Dev& d, int ln) {
    volatile LaneState* v = d.ls + ln;
    LaneState& L = d.ls[ln];
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
    if (isfinite(resid)) L.audit_residual += resid;
    L.transport_drop_w += dw;
    L.transport_drop_e += de;
    L.slots_out += v->slots_out_it;
    const int k = L.iter;
    if (k < d.hist_cap) d.hist[(size_t)ln * d.hist_cap + k] = r;
    L.last = r;
    L.w_fail += r.W_pass ? 0 : 1;
    L.e_fail += r.E_pass ? 0 : 1;
    L.iter = k + 1;
    L.include_source = 0;
    // C1 stopping rule, applied by the next classification: in-flight
    // weight below a fraction of the injected weight
    L.light = (d.stop_frac > 0.0f && r.W_out_total < d.stop_frac * L.src_inj_w) ? 1 : 0;
    // a plan's spot at its iteration limit ends the same way, unfinished
    // (the terminal residual of k1k6_pipeline.cu:1677-1706)
    if (!L.light && d.gs->plan_n > 0 && k + 1 >= d.gs->lane_max_it) {
        L.light = 1;
        L.stopped = 1;
    }
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
    // the precision form books the increment itself (its rounding is its own,
    // not the cumulative tally's)
    return (double)fmaxf(0.0f, d.precise ? x : w1 - w0);
}

// K5 audit of the iteration, warp per cell of psi_in's list (whose storage
// the classify kernel already cleared); the last block writes each working
// lane's audit record and swaps the occupancy lists (K6).
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_finalize(Dev d) {
    constexpr int NW = kThreads / 32;
    __shared__ LaneSums<7> s_sum;   // Edep, Ecut, Enuc, Ebnd, Wcut, Wnuc, Wbnd
    __shared__ float s_out[kMaxLanes][2];   // psi_out weight and bin-centre energy
    __shared__ int s_last;
    IterGlobal* gs = d.gs;
    if (gs->halt) return;
    const int in = gs->parity;
    const int nocc = gs->occ_n[in];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = gridDim.x * NW;
    s_sum.zero(d.B);
    for (int i = threadIdx.x; i < 2 * d.B; i += blockDim.x) (&s_out[0][0])[i] = 0.0f;
    __syncthreads();
    // psi_out's weight and bin-centre energy per lane, from the values the
    // deposit pass left (K5_ConservationAudit's psi_out sums,
    // k5_audit.cu:22-167): warp per occupied psi_out cell, lane per slot, the
    // float4s its occupancy mask marks, U loads in flight.  The four values of
    // a float4 lie in one energy bin of the slot's block (NT is a multiple of
    // 4).  Float sums per slot, per cell and per block (FP64 is a scarce pipe
    // on this part), converted to double once per block.
    static_assert(Lay::NT % 4 == 0 && Lay::NE <= 4 && Lay::L / 4 <= 64, "a float4 lies in one local energy bin");
    constexpr int Q = Lay::L / 4, U = 4;
    const int nout = gs->occ_n[in ^ 1];
    for (int wi = blockIdx.x * NW + wid; wi < nout; wi += nw) {
        const int gc = d.occ_list[in ^ 1][wi];
        const size_t page = (size_t)__ldcg(d.occ_pg[in ^ 1] + wi) + lane;
        const uint32_t bs = d.bid[(size_t)gc * kKb + lane];
        const uint2 mw = __ldcg(d.vmask + page);
        unsigned long long m = bs != kEmpty ? ((unsigned long long)mw.y << 32) | mw.x : 0ull;
        float W = 0.0f, E = 0.0f;
        if (m) {
            const float4* v = reinterpret_cast<const float4*>(d.val) + page * Q;
            const int eb0 = (int)((bs >> 12) & 0xFFFu) * Lay::NE;
            float ec[Lay::NE];
#pragma unroll
            for (int e = 0; e < Lay::NE; ++e) ec[e] = e_center(d, max(0, min(eb0 + e, d.N_E - 1)));
            while (m) {
                float4 r[U];
                int qq[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    qq[u] = __ffsll((long long)m) - 1;
                    m &= m - 1;
                    r[u] = qq[u] >= 0 ? __ldcg(v + qq[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    float w = 0.0f;
                    if (r[u].x > 0.0f) w += r[u].x;
                    if (r[u].y > 0.0f) w += r[u].y;
                    if (r[u].z > 0.0f) w += r[u].z;
                    if (r[u].w > 0.0f) w += r[u].w;
                    const int e = ((4 * max(qq[u], 0)) / Lay::NT) % Lay::NE;
                    float ce = ec[0];
#pragma unroll
                    for (int k = 1; k < Lay::NE; ++k)
                        if (e == k) ce = ec[k];
                    W += w;
                    E += w * ce;
                }
            }
        }
        W = warp_sumf(W);
        E = warp_sumf(E);
        if (lane == 0 && W != 0.0f) {
            float* ls = s_out[lane_of(d, gc)];
            atomicAdd(ls + 0, W);
            atomicAdd(ls + 1, E);
        }
    }
    for (int wi = blockIdx.x * NW + wid; wi < nocc; wi += nw) {
        const int c = d.occ_list[in][wi];
        const int cls = d.cls[c];
        if (cls && lane < 7) {
            const double x = fold_tally(d, c, lane);
            if (x != 0.0) atomicAdd(&s_sum.v[lane_of(d, c)][lane], x);
        }
        if (lane == 0) {
            d.occ[in][c] = 0;
            d.cls[c] = 0;
            if (cls) d.c2b[c] = -1;
        }
    }
    __syncthreads();
    s_sum.flush(d, LANE_DOUBLE(Edep));
    for (int i = threadIdx.x; i < 2 * d.B; i += blockDim.x) {
        const float x = (&s_out[0][0])[i];
        if (x != 0.0f) atomicAdd(reinterpret_cast<double*>(d.ls + i / 2) + LANE_DOUBLE(Wout) + i % 2, (double)x);
    }
    // the block's writes before its count (one fence after the barrier, by
    // the thread that counts: the barrier orders the others' writes before it)
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&gs->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int ln = threadIdx.x; ln < d.B; ln += blockDim.x)
        if (d.ls[ln].work) finalize_lane(d, ln);
    __syncthreads();
    if (threadIdx.x == 0) {
        gs->occ_n[in] = 0;   // the consumed list is empty again
        gs->parity = in ^ 1;
        gs->pass += 1;
        gs->blocks_done = 0;
    }
}

// ------------------------------------------------------------------ spot pipeline helpers
// Clear the phase space of every listed cell of both occupancy lists (reset
// between spots).
template <class Lay>
__global__ void __launch_bounds__(kThreads) k_clear_all(Dev d) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = 0; k < 2; ++k) {
        const int n = d.gs->occ_n[k];
        for (int wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < n; wi += nw) {
            const int c = d.occ_list[k][wi];
            const size_t pg0 = (size_t)d.occ_pg[k][wi];
            uint32_t* ids = d.bid + (size_t)c * kKb;
            const uint32_t x = ids[lane];
            unsigned um = __ballot_sync(kFull, x != kEmpty);
            const unsigned used = um;
            while (um) {
                const int s = __ffs(um) - 1;
                um &= um - 1;
                float4* v = reinterpret_cast<float4*>(d.val + (pg0 + s) * Lay::L);
                for (int q = lane; q < Lay::L / 4; q += 32) v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            ids[lane] = kEmpty;
            if (used & (1u << lane)) d.vmask[pg0 + lane] = make_uint2(0u, 0u);
            if (lane == 0) { d.occ[k][c] = 0; d.cls[c] = 0; d.c2b[c] = -1; }
        }
    }
    // the overflow pages (written only by a run that ran out of pages), and
    // every lane's region starts again
    const size_t sink = (size_t)d.pool_lane * d.B;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)kKb * Lay::L / 4;
         i += (size_t)gridDim.x * blockDim.x) {
        reinterpret_cast<float4*>(d.val + sink * Lay::L)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < kKb) d.vmask[sink + i] = make_uint2(0u, 0u);
    }
    for (int ln = blockIdx.x * blockDim.x + threadIdx.x; ln < d.B; ln += gridDim.x * blockDim.x) d.ls[ln].pool_top = 0;
}

// Occupancy masks of slots 0..n-1 of a single-lane engine from the values a
// caller wrote, in pages numbered like the slots (pbase[gc] = 32 gc); thread
// per slot, an empty slot's mask is zero.
template <class Lay>
__global__ void k_vmask_build(Dev d, size_t n) {
    constexpr int Q = Lay::L / 4;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        unsigned long long m = 0ull;
        if (d.bid[i] != kEmpty) {
            const float4* v = reinterpret_cast<const float4*>(d.val) + i * Q;
            for (int q = 0; q < Q; ++q) {
                const float4 x = v[q];
                if (x.x != 0.0f || x.y != 0.0f || x.z != 0.0f || x.w != 0.0f) m |= 1ull << q;
            }
        }
        d.vmask[i] = make_uint2((uint32_t)m, (uint32_t)(m >> 32));
    }
}

// psi_in values of lane 0 in the dense layout [Nc][32][L] (zeros for an
// empty slot), gathered from the cells' pages; thread per value.
template <class Lay>
__global__ void k_gather_psi(Dev d, float* out) {
    const size_t n = (size_t)d.Nc * kKb * Lay::L;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t slot = i / Lay::L;
        const int l = (int)(i % Lay::L);
        float x = 0.0f;
        if (d.bid[slot] != kEmpty) x = d.val[page_of(d, (int)(slot / kKb), (int)(slot % kKb)) * Lay::L + l];
        out[i] = x;
    }
}
// Pages numbered like the slots for a phase space a caller wrote (single
// lane: pbase[gc] = 32 gc, the occupancy list's pages likewise).
__global__ void k_pages_identity(Dev d, int list_k, int n_listed) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.Nc; i += gridDim.x * blockDim.x) {
        d.pbase[i] = i * kKb;
        if (i < n_listed) d.occ_pg[list_k][i] = d.occ_list[list_k][i] * kKb;
    }
}

// New spots in every lane: zero the iteration and lane states.  The
// classification number runs on, one step past the last spot's, so that no
// cell reads as active in a previous classification; the claim pass number
// runs on too, and restarts after a wipe of the claim tables when it nears
// its 32-bit limit.
__global__ void k_reset_state(Dev d) {
    // every lane's state, a thread per lane
    for (int ln = blockIdx.x * blockDim.x + threadIdx.x; ln < d.B; ln += gridDim.x * blockDim.x) {
        memset(&d.ls[ln], 0, sizeof(LaneState));
        d.ls[ln].done = 1;
        d.ls[ln].spot = -1;
    }
    if (threadIdx.x || blockIdx.x) return;
    IterGlobal* gs = d.gs;
    const unsigned long long g = gs->gen;
    uint32_t tag = gs->ctag;
    const int ovf = gs->cand_ovf, miss = gs->cand_miss;
    int wipe = 0;
    if (tag >= 0xFFF00000u) {
        tag = 0;
        wipe = 1;
    }
    memset(gs, 0, sizeof(IterGlobal));
    gs->gen = g + 1;
    gs->ctag = tag;
    gs->cand_ovf = ovf;
    gs->cand_miss = miss;
    gs->wipe = wipe;
    gs->max_pass = INT_MAX;
}

// Clear every claim-table row when a tag wrap is pending (grid-stride).
__global__ void k_wipe(Dev d, size_t n_words, size_t n_counts) {
    if (!d.gs->wipe) return;
    const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, st = (size_t)gridDim.x * blockDim.x;
    for (size_t i = i0; i < n_words; i += st) d.ctab[i] = ~0ull;
    for (size_t i = i0; i < n_counts; i += st) d.ccount[i] = 0;
}

__global__ void k_set_pass_limit(IterGlobal* gs, int more) {
    if (threadIdx.x || blockIdx.x) return;
    const long long lim = (long long)gs->pass + more;
    gs->max_pass = lim > INT_MAX ? INT_MAX : (int)lim;
}

// Lateral post-convolution kernel of one depth row (the kernel of
// gpu_transport_wrapper.cu:551-616): a Gaussian of sigma^2 = sigma_total^2 -
// sigma_x0^2, in cells, over +-ceil(3 sigma) cells (at most Nx/2),
// normalised.  Half width 0 leaves the row as it is.
__device__ __forceinline__ int lateral_half(float st, float s0, float dx, int Nx, double* sc) {
    const float msq = st * st - s0 * s0;
    if (msq <= 1e-6f) return 0;
    const float c = sqrtf(msq) / dx;
    *sc = (double)c;
    const int h = (int)ceilf(3.0f * c);
    return max(1, min(h, Nx / 2));
}
__device__ __forceinline__ double lateral_tap(int j, double sc) { return exp(-0.5 * ((double)j * j) / (sc * sc)); }

// The row kernels of every lane from its sigma_total(z) and initial sigma_x;
// thread per (lane, row).
__global__ void k_dose_tables(const float* __restrict__ feS, const float* __restrict__ sx0, float dx, int Nx, int Nz,
                              int B, int stride, int* __restrict__ half, double* __restrict__ ker) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * Nz) return;
    double sc = 0.0;
    const int h = lateral_half(feS[i], sx0[i / Nz], dx, Nx, &sc);
    half[i] = h;
    if (h == 0) return;
    double* k = ker + (size_t)i * stride;
    double sum = 0.0;
    for (int j = -h; j <= h; ++j) {
        k[j + h] = lateral_tap(j, sc);
        sum += k[j + h];
    }
    for (int j = 0; j <= 2 * h; ++j) k[j] /= sum;
}

// Lateral MCS post-convolution of EdepC, one thread per output cell of each
// lane, with that lane's row kernels.
__global__ void k_dose(const double* __restrict__ edep, const int* __restrict__ half, const double* __restrict__ ker,
                       int kstride, int Nx, int Nz, int B, double* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nc = (long long)Nx * Nz;
    if (i >= nc * B) return;
    const int lc = (int)(i % nc);
    const long long ln = i / nc;
    const int iz = lc / Nx, ix = lc - iz * Nx;
    const int h = half[ln * Nz + iz];
    if (h == 0) { out[i] = edep[i]; return; }
    const double* k = ker + (size_t)(ln * Nz + iz) * kstride;
    const double* row = edep + (i - lc) + (size_t)iz * Nx;
    double acc = 0.0;
    for (int j = -h; j <= h; ++j) {
        const int x = ix + j;
        if (x >= 0 && x < Nx) acc += row[x] * k[j + h];
    }
    out[i] = acc;
}

// lut_range(E) of the device LUT, once (the fine-threshold range of K2)
__global__ void k_eval_range(Dev d, float E, float* out) {
    if (threadIdx.x || blockIdx.x) return;
    *out = lut_range(d, E);
}

// K2's physics per energy bin at density 1 over the coarse step (Dev::k2tab):
// the expressions of the K2 branch of transport_bin with rho = 1
__global__ void k_k2_table(Dev d, float4* tab) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.N_E) return;
    const float E = d.Ee[b] + 1.0f * ((d.Ee[b + 1] - d.Ee[b]) * 0.5f);
    const float rs = fminf(d.step_coarse, fminf(d.dx, d.dz));
    const float rho = 1.0f;
    const float RE = lut_range(d, E);
    const float dE = fminf(lut_energy_loss(d, E, RE, rho * rs), E);
    const float surv = sm2d_expf(-nuclear_xs(E) * (rho * rs));
    const float T = scatter_power(fmaxf(E - 0.5f * dE, d.lutEmin), fmaxf(rs, 0.0f), rho);
    tab[b] = make_float4(RE, dE, surv, T);
}

// ------------------------------------------------------------------ spot plan
// Outcome of a lane's spot (sm2d_spot_result).
__host__ __device__ inline void lane_result(const LaneState& L, sm2d_spot_result& r) {
    r.iterations = L.iter;
    r.finished = (L.done && !L.stopped) ? 1 : 0;
    r.weight_audit_failures = L.w_fail;
    r.energy_audit_failures = L.e_fail;
    r.injected_weight = L.src_inj_w;
    r.injected_energy = L.src_inj_e;
    r.source_out_of_grid_weight = L.src_oog_w;
    r.source_slot_dropped_weight = L.src_slot_w;
    r.transport_dropped_weight = L.transport_drop_w;
    r.transport_dropped_energy = L.transport_drop_e;
    r.audit_residual_energy = L.audit_residual;
    r.representation_loss_energy = L.src_rep_loss;
    r.cell_steps = L.cell_steps;
    r.slots_in = L.slots_in;
    r.slots_out = L.slots_out;
    r.last = L.last;
}

// Opens a plan of n spots, each limited to max_it iterations.
__global__ void k_plan_begin(Dev d, const BeamArgs* beams, const float* fe, double* dose, sm2d_spot_result* res, int n,
                             int max_it, int lane_limit, const int* order) {
    if (threadIdx.x || blockIdx.x) return;
    IterGlobal* gs = d.gs;
    gs->plan_n = n;
    gs->plan_order = order;
    gs->lane_limit = lane_limit;
    gs->plan_next = 0;
    gs->lane_max_it = max_it;
    gs->refills = 0;
    gs->n_fin = 0;
    gs->plan_beams = beams;
    gs->plan_fe = fe;
    gs->plan_dose = dose;
    gs->plan_res = res;
    gs->max_pass = INT_MAX;
}
__global__ void k_plan_end(Dev d) {
    if (threadIdx.x || blockIdx.x) return;
    d.gs->plan_n = 0;
}

// Each lane whose spot finished at this classification: the lateral
// post-convolution of its dose into the plan's dose map of the spot, with
// the kernel k_dose_tables builds, then its tallies cleared for the next
// spot.  Block per (depth row, finished lane).
__global__ void __launch_bounds__(128) k_lane_complete(Dev d) {
    extern __shared__ double s_k[];
    __shared__ double s_sum;
    const IterGlobal* gs = d.gs;
    if ((int)blockIdx.y >= gs->n_fin) return;
    const int ln = gs->fin[blockIdx.y];
    const int iz = blockIdx.x;
    const size_t row = (size_t)ln * d.Nc + (size_t)iz * d.Nx;
    const int spot = d.ls[ln].spot;
    double* out = gs->plan_dose;
    if (out && spot >= 0) {
        double sc = 0.0;
        const int h = lateral_half(d.feS[(size_t)ln * d.Nz + iz], d.sx0[ln], d.dx, d.Nx, &sc);
        double* dst = out + (size_t)spot * d.Nc + (size_t)iz * d.Nx;
        if (h == 0) {
            for (int ix = threadIdx.x; ix < d.Nx; ix += blockDim.x) dst[ix] = d.edep[row + ix];
        } else {
            for (int j = threadIdx.x; j <= 2 * h; j += blockDim.x) s_k[j] = lateral_tap(j - h, sc);
            __syncthreads();
            if (threadIdx.x == 0) {
                double sum = 0.0;
                for (int j = 0; j <= 2 * h; ++j) sum += s_k[j];
                s_sum = sum;
            }
            __syncthreads();
            for (int j = threadIdx.x; j <= 2 * h; j += blockDim.x) s_k[j] /= s_sum;
            __syncthreads();
            for (int ix = threadIdx.x; ix < d.Nx; ix += blockDim.x) {
                double acc = 0.0;
                for (int j = -h; j <= h; ++j) {
                    const int x = ix + j;
                    if (x >= 0 && x < d.Nx) acc += d.edep[row + x] * s_k[j + h];
                }
                dst[ix] = acc;
            }
        }
    }
    __syncthreads();
    for (int ix = threadIdx.x; ix < d.Nx; ix += blockDim.x) {
        d.edep[row + ix] = 0.0; d.e_cut[row + ix] = 0.0; d.e_nuc[row + ix] = 0.0; d.e_bnd[row + ix] = 0.0;
        d.w_cut[row + ix] = 0.0f; d.w_nuc[row + ix] = 0.0f; d.w_bnd[row + ix] = 0.0f;
    }
}

// Results of the finished spots, then the plan's next spots into the idle
// lanes in lane order: lane state cleared, beam and Fermi-Eyges tables of
// the spot, refill flag for the injection kernels that follow.  One block.
__global__ void __launch_bounds__(256) k_lane_assign(Dev d) {
    __shared__ int s_cnt[256];
    IterGlobal* gs = d.gs;
    const int tid = threadIdx.x;
    // results of the lanes whose spot just finished
    for (int j = tid; j < gs->n_fin; j += blockDim.x) {
        LaneState& L = d.ls[gs->fin[j]];
        if (L.spot >= 0 && gs->plan_res) lane_result(L, gs->plan_res[L.spot]);
        L.spot = -1;
    }
    __syncthreads();
    // idle lanes in lane order take the plan's next spots: thread t looks at
    // the lanes t * per .. t * per + per - 1, a block scan orders them
    const int lim = gs->lane_limit > 0 ? min(gs->lane_limit, d.B) : d.B;
    const int per = (lim + blockDim.x - 1) / blockDim.x;
    int mine = 0;
    for (int k = 0; k < per; ++k) {
        const int ln = tid * per + k;
        if (ln < lim && d.ls[ln].done && d.ls[ln].spot < 0) ++mine;
    }
    s_cnt[tid] = mine;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {   // inclusive scan
        const int y = tid >= o ? s_cnt[tid - o] : 0;
        __syncthreads();
        s_cnt[tid] += y;
        __syncthreads();
    }
    const int next = gs->plan_next, left = max(gs->plan_n - next, 0);
    const int total = min(s_cnt[blockDim.x - 1], left);
    int r = s_cnt[tid] - mine;
    for (int k = 0; k < per && r < total; ++k) {
        const int ln = tid * per + k;
        if (ln < lim && d.ls[ln].done && d.ls[ln].spot < 0) {
            gs->fill_lane[r] = ln;
            gs->fill_spot[r] = gs->plan_order ? gs->plan_order[next + r] : next + r;
            ++r;
        }
    }
    __syncthreads();
    if (tid == 0) {
        gs->n_fin = 0;
        gs->n_fill = total;
        gs->plan_next = next + total;
        gs->refills += 1;
    }
}

// The lanes the refill assigned: state cleared, the spot's tables and beam
// copied, marked for the injection; a grid over (lane, element).
__global__ void __launch_bounds__(256) k_lane_fill(Dev d, BeamArgs* beams) {
    const IterGlobal* gs = d.gs;
    const int n = gs->n_fill, Nz = d.Nz;
    constexpr int NW = (int)(sizeof(LaneState) / 4);
    const int per = NW + Nz;   // LaneState words, then the depth rows of the tables
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x, st = gridDim.x * blockDim.x;
    for (int i = i0; i < n * per; i += st) {
        const int k = i / per, e = i % per, ln = gs->fill_lane[k], sp = gs->fill_spot[k];
        if (e < NW) {
            int v = 0;
            if (e == (int)(offsetof(LaneState, spot) / 4)) v = sp;
            if (e == (int)(offsetof(LaneState, refill) / 4)) v = 1;
            if (e == (int)(offsetof(LaneState, done) / 4)) v = 1;
            reinterpret_cast<int*>(d.ls + ln)[e] = v;
            continue;
        }
        const int z = e - NW;
        const float* fe = gs->plan_fe + (size_t)sp * (3 * Nz + 1);
        d.feA[(size_t)ln * Nz + z] = fe[z];
        d.feB[(size_t)ln * Nz + z] = fe[Nz + z];
        d.feS[(size_t)ln * Nz + z] = fe[2 * Nz + z];
        if (z == 0) {
            d.sx0[ln] = fe[3 * Nz];
            beams[ln] = gs->plan_beams[sp];
        }
    }
}

// ================================================================== engine
struct Ctx {
    sm2d_problem p{};
    std::vector<float> th, Ee, feA, feB, feS;   // Fermi-Eyges tables of the problem's E0 and sigma_x
    // per-lane Fermi-Eyges tables: host copy [feA B*Nz | feB B*Nz | feS B*Nz |
    // sigma_x B] of fe_dev, and the (E0, sigma_x) each lane's tables are for
    std::vector<float> fe_host, fe_E0, fe_sx;
    std::vector<float> rho_host;    // slab phantom: density per depth row (empty: water)
    float* fe_dev = nullptr;
    int fe_lo = 0, fe_hi = -1;      // lanes whose tables changed since the last upload
    int L = 0, layout = 0;  // 0: LayoutRef, 1: LayoutB128
    int B = 1;
    Dev d{};
    IterGlobal* gs_host = nullptr;  // pinned mirrors
    LaneState* ls_host = nullptr;
    cudaStream_t s = nullptr;
    std::vector<void*> allocs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle cond{};    // device loop: another pass
    cudaGraphConditionalHandle rcond{};   // spot plan: refill after this pass
    cudaEvent_t ev[10] = {};   // 0..7 one iteration's stages, 8..9 a whole run
    float step_ms[7] = {};
    int grid_cell = 0, grid_transport = 0, grid_keys = 0;   // warp-per-cell kernels, deposit pass, claim pass
    int shape[4] = {8, 4, 0, 0};   // blocks per SM: warp-per-cell kernels, finalize, claim pass, deposit
                                   // pass (0: every resident block)
    int sms = 1;
    int lanes_in_flight = 0;   // a plan fills lanes 0 .. lanes_in_flight - 1 (0: every lane)
    int grid_fin = 0;   // finalize: four blocks per SM (its per-block flushes of per-lane sums are atomics on a
                        // few addresses; 13.2 ms per wave of 80 spots against 14.2 at eight, 14.8 at three)
    size_t pages = 0;                        // value pages (every lane's region and the overflow pages)
    size_t ctab_words = 0;                   // claim-table size in 64-bit words
    size_t ccount_n = 0;
    bool injected = false;
    BeamArgs* beams_dev = nullptr;  // device beams, one per lane
    BeamArgs* beams_host = nullptr; // pinned staging
    int* dose_half = nullptr;       // per-lane, per-row half width of the lateral kernel [B][Nz]
    double* dose_ker = nullptr;     // its weights [B][Nz][dose_stride]
    double* dose_dev = nullptr;     // convolved dose [B][Nc]
    int dose_stride = 1;            // 2 (Nx/2) + 1: the widest kernel
    std::vector<cudaEvent_t> pev;   // event pool of the profiled replay
    // spot plan: device copies of the plan's beams, Fermi-Eyges tables,
    // results and dose maps (grown on demand), and their host staging
    int plan_n = 0, plan_max_it = 0;
    bool plan_dose_on = false;
    int plan_max_n = 1024;          // sizes the injection grid of a refill
    size_t plan_cap = 0, plan_dose_cap = 0;
    BeamArgs* plan_beams_dev = nullptr;
    float* plan_fe_dev = nullptr;
    sm2d_spot_result* plan_res_dev = nullptr;
    int* plan_order_dev = nullptr;    // the order lanes take the plan's spots
    std::vector<int> plan_order_host;
    double* plan_dose_dev = nullptr;
    double* plan_dose_ext = nullptr;  // sm2d_batch_run: the caller's pinned host maps, written by the device
    std::vector<BeamArgs> plan_beams_host;
    std::vector<float> plan_fe_host;
    // the learned surrogate in the expectation form's K3 (sm2d_set_surrogate)
    sm2d_mlp_handle mlp = nullptr;
    float mlp_tol = 0.0f;
    int mlp_method = 0;
    size_t k3_alloc = 0;   // rows of the buffers below
    int grid_rows = 0;
};

static int dalloc(Ctx& c, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(SM2D_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    c.allocs.push_back(*p);
    return 0;
}

static BeamArgs beam_args(const sm2d_beam& b) {
    return BeamArgs{b.x0, b.z0, b.theta0, b.E0, b.W_total, b.sigma_x, b.sigma_theta, b.sigma_E, b.n_samples, b.seed};
}
static bool host_gaussian(const sm2d_beam& b) {   // gpu_transport_wrapper.cu:246
    return (b.n_samples > 1) || (b.sigma_x > 0.0f) || (b.sigma_theta > 0.0f);
}

template <class Lay>
struct Impl {
    // One iteration: K1 classify, (ascending lists on request), the claim
    // pass of K2/K3, bucket and psi_out slot selection (with the per-cell
    // tallies of the claim pass's step records), the deposit pass of K2/K3
    // with the fused K4 scatter or the bucket pair, K5 finalize.  ev[0..7]
    // bracket: classify, lists, claim pass, selection + tallies, deposit
    // pass, K4 bucket move, finalize.
    static int launch_body(Ctx& c, bool timed, bool use_cond, bool lists) {
        const int gc = c.grid_cell, gt = c.grid_transport, gk = c.grid_keys;
        const bool bk = c.p.use_buckets != 0;
        auto rec = [&](int k) { return timed ? cudaEventRecord(c.ev[k], c.s) : cudaSuccess; };
        CK(rec(0));
        k_classify<Lay><<<gc, kThreads, 0, c.s>>>(c.d, c.cond, c.rcond, use_cond ? 1 : 0);
        CK(rec(1));
        if (lists) k_order_lists<<<1, 1024, 0, c.s>>>(c.d);
        CK(rec(2));
        // the expectation form (direct scatter only) has kernels of its own,
        // so the sampled form's keep their registers
        if (c.d.expect) k_transport<Lay, PASS_KEYS, true><<<gk, kThreads, 0, c.s>>>(c.d);
        else k_transport<Lay, PASS_KEYS><<<gk, kThreads, 0, c.s>>>(c.d);
        if (c.d.surr) {   // the network over the claim pass's surrogate rows, then their claims
            const int rc = mlp_transport_rows(c.mlp, c.s, c.d.kfeat, &c.d.gs->k3_rows, c.d.k3_cap, c.mlp_tol,
                                              c.mlp_method, c.d.ktab, c.d.kfb);
            if (rc) return rc;
            k_surr_keys<Lay><<<c.grid_rows, kThreads, 0, c.s>>>(c.d);
        }
        CK(rec(3));
        if (bk) k_select_buckets<Lay, true><<<gc, kThreads, 0, c.s>>>(c.d);
        else k_select_buckets<Lay, false><<<gc, kThreads, 0, c.s>>>(c.d);
        k_select_psi<<<gc, kThreads, 0, c.s>>>(c.d, 1);
        CK(rec(4));
        if (bk) k_transport<Lay, PASS_BUCKET><<<gt, kThreads, 0, c.s>>>(c.d);
        else if (c.d.expect) k_transport<Lay, PASS_DIRECT, true><<<gt, kThreads, 0, c.s>>>(c.d);
        else k_transport<Lay, PASS_DIRECT><<<gt, kThreads, 0, c.s>>>(c.d);
        CK(rec(5));
        if (bk) k_bucket_push<Lay><<<gc, kThreads, 0, c.s>>>(c.d);
        CK(rec(6));
        k_finalize<Lay><<<c.grid_fin, kThreads, 0, c.s>>>(c.d);
        CK(rec(7));
        CK(cudaGetLastError());
        return 0;
    }
    // grids of the two transport passes: every resident block once (the
    // kernels stride over the bin list)
    static int transport_grid(Ctx& c, int sms) {
        int per_sm = 0, per_sm_keys = 0;
        cudaError_t e =
            c.p.use_buckets ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport<Lay, PASS_BUCKET>, kThreads, 0)
            : c.d.expect    ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport<Lay, PASS_DIRECT, true>, kThreads, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_transport<Lay, PASS_DIRECT>, kThreads, 0);
        if (e == cudaSuccess)
            e = c.d.expect ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_keys, k_transport<Lay, PASS_KEYS, true>, kThreads, 0)
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_keys, k_transport<Lay, PASS_KEYS>, kThreads, 0);
        if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
        const long long blocks_for_cap = ((long long)c.d.bins_cap + kThreads - 1) / kThreads;
        const long long s = std::max(sms, 1);
        if (c.shape[3] > 0) per_sm = std::min(per_sm, c.shape[3]);
        if (c.shape[2] > 0) per_sm_keys = std::min(per_sm_keys, c.shape[2]);
        c.grid_transport = (int)std::max(1LL, std::min((long long)std::max(per_sm, 1) * s, blocks_for_cap));
        c.grid_keys = (int)std::max(1LL, std::min((long long)std::max(per_sm_keys, 1) * s, blocks_for_cap));
        return 0;
    }
    // grid of the surrogate rows' claim pass: every resident block once
    static int rows_grid(Ctx& c, int sms) {
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_surr_keys<Lay>, kThreads, 0);
        if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
        const long long blocks_for_cap = ((long long)c.d.k3_cap + kThreads - 1) / kThreads;
        c.grid_rows = (int)std::max(1LL, std::min((long long)std::max(per_sm, 1) * std::max(sms, 1), blocks_for_cap));
        return 0;
    }
    static int clear_all(Ctx& c, int) {
        k_clear_all<Lay><<<c.grid_cell, kThreads, 0, c.s>>>(c.d);
        CK(cudaGetLastError());
        return 0;
    }
    static int build_masks(Ctx& c, size_t n) {
        k_vmask_build<Lay><<<(unsigned)std::min<size_t>((n + 255) / 256, 8192), 256, 0, c.s>>>(c.d, n);
        CK(cudaGetLastError());
        return 0;
    }
    static int gather_psi(Ctx& c, float* out) {
        const size_t n = (size_t)c.d.Nc * kKb * c.L;
        k_gather_psi<Lay><<<(unsigned)std::min<size_t>((n + 255) / 256, 16384), 256, 0, c.s>>>(c.d, out);
        CK(cudaGetLastError());
        return 0;
    }
    // injection of the beams in beams_dev (one per lane; the kernels stride
    // over a lane's samples, max_n sizes the grid): claim pass, slot
    // selection, deposit pass, source accounting.  refill_only: the lanes
    // a plan refills.
    static int inject(Ctx& c, int max_n, bool check_empty, bool refill_only) {
        const int gx = std::min((std::max(max_n, 1) + 255) / 256, 16);
        const dim3 grid((unsigned)gx, (unsigned)c.B);
        const int ro = refill_only ? 1 : 0;
        k_inject_begin<<<1, 1, 0, c.s>>>(c.d, check_empty ? 1 : 0);
        k_inject_keys<Lay><<<grid, 256, 0, c.s>>>(c.d, c.beams_dev, c.p.x_min, c.p.z_min, ro);
        k_select_psi<<<c.grid_cell, kThreads, 0, c.s>>>(c.d, 0);
        k_inject_deposit<Lay><<<grid, 256, 0, c.s>>>(c.d, c.beams_dev, c.p.x_min, c.p.z_min, ro);
        k_totals<Lay><<<c.grid_cell, kThreads, 0, c.s>>>(c.d);
        k_source_finalize<<<(c.B + 255) / 256, 256, 0, c.s>>>(c.d, c.beams_dev, ro);
        CK(cudaGetLastError());
        return 0;
    }
    // refill of a spot plan: finished lanes' dose and results, next spots
    // into the idle lanes, their injection
    static int refill(Ctx& c, int) {
        const size_t smem = sizeof(double) * (size_t)c.dose_stride;
        k_lane_complete<<<dim3((unsigned)c.d.Nz, (unsigned)c.B), 128, smem, c.s>>>(c.d);
        k_lane_assign<<<1, 256, 0, c.s>>>(c.d);
        k_lane_fill<<<(unsigned)std::min(c.B * 4, 2048), 256, 0, c.s>>>(c.d, c.beams_dev);
        CK(cudaGetLastError());
        return inject(c, c.plan_max_n, false, true);
    }
};

#define DISPATCH(c, fn, ...) ((c).layout == 0 ? Impl<LayoutRef>::fn(c, __VA_ARGS__) : Impl<LayoutB128>::fn(c, __VA_ARGS__))

static int sync_state(Ctx& c) {
    CK(cudaMemcpyAsync(c.gs_host, c.d.gs, sizeof(IterGlobal), cudaMemcpyDeviceToHost, c.s));
    CK(cudaMemcpyAsync(c.ls_host, c.d.ls, sizeof(LaneState) * c.B, cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}
static int push_state(Ctx& c) {
    CK(cudaMemcpyAsync(c.d.gs, c.gs_host, sizeof(IterGlobal), cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(c.d.ls, c.ls_host, sizeof(LaneState) * c.B, cudaMemcpyHostToDevice, c.s));
    return 0;
}

// grids of the pass kernels from the launch shape (blocks per SM)
static int apply_shape(Ctx& c) {
    const long long NcB = (long long)c.B * c.d.Nc;
    const long long cells = std::max(1LL, (NcB + kThreads / 32 - 1) / (kThreads / 32));
    c.grid_cell = (int)std::max(1LL, std::min(cells, (long long)c.shape[0] * c.sms));
    c.grid_fin = (int)std::max(1LL, std::min((long long)c.grid_cell, (long long)c.shape[1] * c.sms));
    int rc = DISPATCH(c, transport_grid, c.sms);
    if (!rc && c.d.surr) rc = DISPATCH(c, rows_grid, c.sms);
    return rc;
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
    CK(cudaGraphConditionalHandleCreate(&c.rcond, body, 0, 0));
    CK(cudaStreamBeginCaptureToGraph(c.s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = DISPATCH(c, launch_body, false, true, false);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(c.s, &captured);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    // the refill of a spot plan: an if-node after the pass's last kernel
    size_t nn = 0;
    CK(cudaGraphGetNodes(body, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn), sinks;
    CK(cudaGraphGetNodes(body, nodes.data(), &nn));
    for (cudaGraphNode_t n : nodes) {
        size_t nd = 0;
        CK(cudaGraphNodeGetDependentNodes(n, nullptr, nullptr, &nd));
        if (nd == 0) sinks.push_back(n);
    }
    cudaGraphNodeParams ip{};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = c.rcond;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t ifn;
    CK(cudaGraphAddNode(&ifn, body, sinks.data(), nullptr, sinks.size(), &ip));
    cudaGraph_t rbody = ip.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(c.s, rbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    rc = DISPATCH(c, refill, 0);
    e = cudaStreamEndCapture(c.s, &captured);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "refill capture: %s", cudaGetErrorString(e));
    CK(cudaGraphInstantiate(&c.exec, c.graph, 0));
    return 0;
}

// Zero the per-cell tallies and mask history of every lane and the lane
// and iteration states (the phase space itself: clear_all).
static int reset_lanes(Ctx& c) {
    int rc = DISPATCH(c, clear_all, 0);
    if (rc) return rc;
    const size_t n = (size_t)c.B * c.d.Nc;
    const Dev& d = c.d;
    CK(cudaMemsetAsync(d.edep, 0, n * 8, c.s));
    CK(cudaMemsetAsync(d.e_cut, 0, n * 8, c.s));
    CK(cudaMemsetAsync(d.e_nuc, 0, n * 8, c.s));
    CK(cudaMemsetAsync(d.e_bnd, 0, n * 8, c.s));
    CK(cudaMemsetAsync(d.w_cut, 0, n * 4, c.s));
    CK(cudaMemsetAsync(d.w_nuc, 0, n * 4, c.s));
    CK(cudaMemsetAsync(d.w_bnd, 0, n * 4, c.s));
    CK(cudaMemsetAsync(d.cls, 0, n, c.s));
    k_reset_state<<<(unsigned)((c.B + 127) / 128), 128, 0, c.s>>>(c.d);
    k_wipe<<<c.grid_cell, kThreads, 0, c.s>>>(c.d, c.ctab_words, c.ccount_n);
    CK(cudaGetLastError());
    c.injected = false;
    return 0;
}

static int enqueue_dose(Ctx& c) {
    const long long n = (long long)c.B * c.d.Nc;
    k_dose<<<(unsigned)((n + 255) / 256), 256, 0, c.s>>>(c.d.edep, c.dose_half, c.dose_ker, c.dose_stride, c.d.Nx,
                                                         c.d.Nz, c.B, c.dose_dev);
    CK(cudaGetLastError());
    return 0;
}

// Fermi-Eyges tables of lane ln for a beam of energy E0 and width sigma_x
// (gpu_transport_wrapper.cu:273-276 hands the beam's E0 and sigma_x to the
// precompute of k1k6_pipeline.cu:1061-1206); recomputed only when they change.
static void set_lane_fe(Ctx& c, int ln, float E0, float sx) {
    if (c.fe_E0[ln] == E0 && c.fe_sx[ln] == sx) return;
    const int Nz = c.d.Nz;
    const size_t BN = (size_t)c.B * Nz;
    float* A = c.fe_host.data() + (size_t)ln * Nz;
    fermi_eyges_moments(E0, Nz, c.d.dz, sx, A, A + BN, A + 2 * BN, c.rho_host.empty() ? nullptr : c.rho_host.data());
    c.fe_host[3 * BN + ln] = sx;
    c.fe_E0[ln] = E0;
    c.fe_sx[ln] = sx;
    c.fe_lo = std::min(c.fe_lo, ln);
    c.fe_hi = std::max(c.fe_hi, ln);
}

// Upload the changed lanes' tables and rebuild their lateral dose kernels.
// The copies are from pageable memory, which the copy call has read by the
// time it returns, so fe_host may change right after.
static int upload_lane_fe(Ctx& c) {
    if (c.fe_hi < c.fe_lo) return 0;
    const int Nz = c.d.Nz, lo = c.fe_lo, n = c.fe_hi - c.fe_lo + 1;
    const size_t BN = (size_t)c.B * Nz;
    for (int k = 0; k < 3; ++k)
        CK(cudaMemcpyAsync(c.fe_dev + k * BN + (size_t)lo * Nz, c.fe_host.data() + k * BN + (size_t)lo * Nz,
                           sizeof(float) * (size_t)n * Nz, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(c.fe_dev + 3 * BN + lo, c.fe_host.data() + 3 * BN + lo, sizeof(float) * n,
                       cudaMemcpyHostToDevice, c.s));
    const int rows = n * Nz;
    k_dose_tables<<<(rows + 127) / 128, 128, 0, c.s>>>(c.fe_dev + 2 * BN + (size_t)lo * Nz, c.fe_dev + 3 * BN + lo,
                                                      c.d.dx, c.d.Nx, Nz, n, c.dose_stride,
                                                      c.dose_half + (size_t)lo * Nz,
                                                      c.dose_ker + (size_t)lo * Nz * c.dose_stride);
    CK(cudaGetLastError());
    c.fe_lo = c.B;
    c.fe_hi = -1;
    return 0;
}

// Beams into the device (lane 0 = *b for a single spot; empty beams elsewhere)
static int stage_beams(Ctx& c, const sm2d_beam* beams, int n, int* max_n) {
    int mx = 1;
    for (int ln = 0; ln < c.B; ++ln) {
        if (ln < n) {
            c.beams_host[ln] = beam_args(beams[ln]);
            if (host_gaussian(beams[ln])) mx = std::max(mx, beams[ln].n_samples);
        } else {
            c.beams_host[ln] = BeamArgs{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0, 0u};
        }
    }
    CK(cudaMemcpyAsync(c.beams_dev, c.beams_host, sizeof(BeamArgs) * c.B, cudaMemcpyHostToDevice, c.s));
    *max_n = mx;
    return 0;
}

// Search tables of slot_of: for each slot of float patterns between lo and
// hi (top bits above kSlotShift), the result of `search` at the slot's
// smallest value.
template <class F>
static std::vector<int> slot_table(float lo, float hi, uint32_t* base, F search) {
    uint32_t ulo, uhi;
    memcpy(&ulo, &lo, 4);
    memcpy(&uhi, &hi, 4);
    *base = ulo >> kSlotShift;
    const uint32_t last = uhi >> kSlotShift;
    std::vector<int> t(last - *base + 1);
    for (uint32_t j = 0; j < t.size(); ++j) {
        const uint32_t u = (*base + j) << kSlotShift;
        float v;
        memcpy(&v, &u, 4);
        t[j] = search(v);
    }
    return t;
}

}  // namespace sm2d

using namespace sm2d;

struct sm2d_ctx : sm2d::Ctx {};

namespace sm2d {
// The device view of a handle's grids and R-LUT and its stream, for the
// redistribution tables of sm2d_surrogate.cu (the transport's own per-bin
// physics evaluated outside a transport pass).
int handle_dev(sm2d_handle h, Dev* d, cudaStream_t* s) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    *d = h->d;
    *s = h->s;
    return 0;
}
}  // namespace sm2d

extern "C" {

int sm2d_create(const sm2d_problem* p, sm2d_handle* out) {
    if (!p || !out) return fail(SM2D_ERR_ARG, "null argument");
    *out = nullptr;
    if (p->Nx <= 0 || p->Nz <= 0 || p->N_theta <= 0 || p->N_E <= 1 || !p->theta_edges || !p->E_edges)
        return fail(SM2D_ERR_ARG, "invalid grid");
    if (!(p->dx > 0.0f) || !(p->dz > 0.0f)) return fail(SM2D_ERR_ARG, "cell size must be positive");
    const int B = p->lanes > 1 ? p->lanes : 1;
    if (B > kMaxLanes) return fail(SM2D_ERR_ARG, "at most %d lanes", kMaxLanes);
    // bin records and claim tables index cells of all lanes with 32 bits
    if ((long long)p->Nx * p->Nz * B > (1LL << 30)) return fail(SM2D_ERR_ARG, "grid x lanes too large (at most 2^30 cells)");
    int layout;
    if (p->nt_local == 4 && p->ne_local == 2 && p->nx_sub == 8 && p->nz_sub == 4) layout = 0;
    else if (p->nt_local == 8 && p->ne_local == 4 && p->nx_sub == 4 && p->nz_sub == 1) layout = 1;
    else return fail(SM2D_ERR_LAYOUT, "local layout (%d,%d,%d,%d) not compiled; use (4,2,8,4) or (8,4,4,1)",
                     p->nt_local, p->ne_local, p->nx_sub, p->nz_sub);
    if (p->N_theta / p->nt_local > 4095 || p->N_E / p->ne_local > 4095)
        return fail(SM2D_ERR_ARG, "grid exceeds the 12-bit block indices");
    if (p->density_z)
        for (int iz = 0; iz < p->Nz; ++iz)
            if (!(p->density_z[iz] > 0.0f) || !std::isfinite(p->density_z[iz]))
                return fail(SM2D_ERR_ARG, "density of row %d must be positive", iz);
    if (p->expectation && !p->energy_split)
        return fail(SM2D_ERR_ARG, "the expectation form needs the energy split (energy_split = 1)");
    if (p->expectation && p->use_buckets)
        return fail(SM2D_ERR_ARG, "the expectation form runs the direct neighbour scatter (use_buckets = 0)");
    sm2d_ctx* c = new sm2d_ctx();
    c->p = *p;
    c->layout = layout;
    c->B = B;
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
    if (p->density_z) c->rho_host.assign(p->density_z, p->density_z + p->Nz);
    c->feA.resize(p->Nz);
    c->feB.resize(p->Nz);
    c->feS.resize(p->Nz);
    fermi_eyges_moments(p->E0, p->Nz, p->dz, p->sigma_x_initial, c->feA.data(), c->feB.data(), c->feS.data(),
                        p->density_z ? c->rho_host.data() : nullptr);
    Dev& d = c->d;
    d.Nx = p->Nx; d.Nz = p->Nz; d.Nc = p->Nx * p->Nz; d.B = B;
    d.dx = p->dx; d.dz = p->dz;
    d.N_theta = p->N_theta; d.N_E = N;
    d.lutN = N;
    d.lutEmin = p->E_min > 0.0f ? p->E_min : c->Ee[0];
    d.lutEmax = p->E_max > 0.0f ? p->E_max : c->Ee[N];
    d.E_fine_on = p->E_fine_on; d.wmin = p->weight_active_min;
    d.step_coarse = p->step_coarse;
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
    d.expect = p->expectation ? 1 : 0;
    d.precise = p->precision_form ? 1 : 0;
    const size_t Nc = (size_t)d.Nc, NcB = Nc * B, ns = NcB * kKb;
    void* q;
    int rc;
#define A(ptr, type, n)                                              \
    if ((rc = dalloc(*c, &q, sizeof(type) * (size_t)(n)))) return bail(rc); \
    ptr = reinterpret_cast<type*>(q)
    float *th_d, *Ee_d, *R_d, *lE_d, *lR_d;
    A(th_d, float, p->N_theta + 1);
    A(Ee_d, float, N + 1);
    A(R_d, float, N);
    A(lE_d, float, N);
    A(lR_d, float, N);
    // search tables: the energy bin (binary search of device_find_bin_edges)
    // and the R-LUT lower bound at each slot's smallest value
    const std::vector<float>& Eh = c->Ee;
    const std::vector<int> et = slot_table(Eh[0], Eh[N], &d.e_base, [&](float v) {
        if (v <= Eh[0]) return 0;
        if (v >= Eh[N]) return N - 1;
        int lo = 0, hi = N;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (Eh[mid + 1] <= v) lo = mid + 1; else hi = mid;
        }
        return lo;
    });
    const std::vector<int> rt = slot_table(std::max(R[0], 1e-30f), std::max(R[N - 1], 1e-30f), &d.r_base,
                                           [&](float v) { return (int)(std::lower_bound(R.begin(), R.end(), v) - R.begin()); });
    d.e_nslot = (int)et.size();
    d.r_nslot = (int)rt.size();
    int *e_slot, *r_slot;
    A(e_slot, int, et.size());
    A(r_slot, int, rt.size());
    d.e_slot = e_slot;
    d.r_slot = r_slot;
    // slab phantom: density and water-equivalent depth of each row's upper face
    std::vector<float> wet;
    float *rho_d = nullptr, *wet_d = nullptr;
    if (!c->rho_host.empty()) {
        wet.resize(p->Nz);
        float acc = 0.0f;
        for (int iz = 0; iz < p->Nz; ++iz) {
            wet[iz] = acc;
            acc += c->rho_host[iz] * p->dz;
        }
        A(rho_d, float, p->Nz);
        A(wet_d, float, p->Nz);
    }
    d.rho = rho_d;
    d.wet = wet_d;
    const size_t BN = (size_t)B * p->Nz;
    A(c->fe_dev, float, 3 * BN + B);
    d.th = th_d; d.Ee = Ee_d; d.R = R_d; d.logE = lE_d; d.logR = lR_d;
    d.feA = c->fe_dev; d.feB = c->fe_dev + BN; d.feS = c->fe_dev + 2 * BN; d.sx0 = c->fe_dev + 3 * BN;
    // value pages: a single lane has one per slot of every cell; a lane of a
    // batch has slot_pages_per_lane, by default 32 MB of values (32768 pages of
    // 256 values, 65536 of 128: the widest 70 MeV spot of the 512-spot plan
    // peaks at 4422 slots on the reference grids and at about 20000 on the
    // 256 log-E / 512 theta grid), plus 32 overflow pages after the last region
    const size_t def_pages = ((size_t)8 << 20) / (size_t)c->L;
    d.pool_lane = B == 1 ? (int)(Nc * kKb)
                         : (int)std::min<size_t>(Nc * kKb, p->slot_pages_per_lane > 0 ? (size_t)p->slot_pages_per_lane : def_pages);
    if ((size_t)d.pool_lane * B + kKb > (size_t)INT_MAX) return bail(fail(SM2D_ERR_ARG, "too many value pages"));
    c->pages = (size_t)d.pool_lane * B + kKb;
    A(d.bid, uint32_t, ns);
    A(d.val, float, c->pages * c->L);
    A(d.vmask, uint2, c->pages);
    A(d.pbase, int, NcB);
    for (int k = 0; k < 2; ++k) {
        A(d.occ[k], int, NcB);
        A(d.occ_list[k], int, NcB);
        A(d.occ_pg[k], int, NcB);
    }
    A(d.edep, double, NcB); A(d.e_cut, double, NcB); A(d.e_nuc, double, NcB); A(d.e_bnd, double, NcB);
    A(d.w_cut, float, NcB); A(d.w_nuc, float, NcB); A(d.w_bnd, float, NcB);
    A(d.dl_edep, double, NcB); A(d.dl_ecut, double, NcB); A(d.dl_enuc, double, NcB); A(d.dl_ebnd, double, NcB);
    A(d.dl_wcut, float, NcB); A(d.dl_wnuc, float, NcB); A(d.dl_wbnd, float, NcB);
    A(d.act_gen, unsigned long long, NcB); A(d.cls, uint8_t, NcB); A(d.c2b, int, NcB);
    // cell list: every cell of a single lane; 2048 cells per lane of a batch,
    // shared by its lanes (a plan spot lists about a hundred cells a pass)
    d.listed_cap = B == 1 ? (int)Nc : (int)std::min<size_t>(NcB, (size_t)B * std::min<size_t>(Nc, 2048));
    A(d.listed, uint32_t, d.listed_cap);
    // bin list: the w > 0 bins of one full slot per cell of a single lane on
    // average; per lane of a batch 32 per value page, shared by the lanes (a
    // plan spot transports about 4000 a pass on average); a pass that needs
    // more stops with SM2D_ERR_ALLOC
    d.bins_cap = (int)std::min<size_t>((B == 1 ? Nc * c->L : (size_t)B * std::min<size_t>(Nc * c->L / 4, (size_t)d.pool_lane * 32)),
                                       (size_t)INT_MAX);
    A(d.bins, uint4, d.bins_cap);
    A(d.cell_bins, int2, d.listed_cap);
    A(d.brec, uint4, 2 * (size_t)d.bins_cap);
    if (d.expect) A(d.brec2, float4, (size_t)d.bins_cap);
    A(d.active, uint32_t, Nc); A(d.coarse, uint32_t, Nc);
    A(d.gs, IterGlobal, 1);
    A(d.ls, LaneState, B);
    d.hist_cap = p->max_iterations > 0 ? p->max_iterations : 4096;
    A(d.hist, sm2d_audit, std::max(1, B * d.hist_cap));
    d.bucket_bytes = bucket_bytes_for(c->L);
    if (p->use_buckets) A(d.buckets, unsigned char, (size_t)4 * d.listed_cap * d.bucket_bytes);
    c->ctab_words = ((size_t)NcB + (size_t)4 * d.listed_cap) * 2 * kCand;
    c->ccount_n = (size_t)NcB + (size_t)4 * d.listed_cap;
    A(d.ctab, unsigned long long, c->ctab_words);
    A(d.ccount, int, c->ccount_n);
    A(d.bkt_ids, uint32_t, (size_t)4 * d.listed_cap * kKb);
    A(d.bkt_os, uint2, (size_t)4 * d.listed_cap * kKb);
    A(c->beams_dev, BeamArgs, B);
    // lateral post-convolution kernels per lane and depth row: half widths
    // are at most Nx/2
    c->dose_stride = 2 * std::max(1, p->Nx / 2) + 1;
    if (sizeof(double) * c->dose_stride > 48 * 1024 &&
        cudaFuncSetAttribute(k_lane_complete, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double) * c->dose_stride)) != cudaSuccess)
        return bail(fail(SM2D_ERR_ARG, "Nx too large for the dose kernel"));
    A(c->dose_half, int, BN);
    A(c->dose_ker, double, BN * c->dose_stride);
    A(c->dose_dev, double, NcB);
#undef A
    if (cudaMallocHost(&c->gs_host, sizeof(IterGlobal)) != cudaSuccess ||
        cudaMallocHost(&c->ls_host, sizeof(LaneState) * B) != cudaSuccess ||
        cudaMallocHost(&c->beams_host, sizeof(BeamArgs) * B) != cudaSuccess)
        return bail(fail(SM2D_ERR_ALLOC, "pinned host state"));
    memset(c->gs_host, 0, sizeof(IterGlobal));
    memset(c->ls_host, 0, sizeof(LaneState) * B);
    c->gs_host->max_pass = INT_MAX;
    for (int ln = 0; ln < B; ++ln) c->ls_host[ln].done = 1;
    cudaStream_t s = c->s;
    bool ok = cudaMemcpyAsync(th_d, c->th.data(), sizeof(float) * (p->N_theta + 1), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(Ee_d, c->Ee.data(), sizeof(float) * (N + 1), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(R_d, R.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(lE_d, lE.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(lR_d, lR.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(e_slot, et.data(), sizeof(int) * et.size(), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(r_slot, rt.data(), sizeof(int) * rt.size(), cudaMemcpyHostToDevice, s) == cudaSuccess;
    if (ok && rho_d)
        ok = cudaMemcpyAsync(rho_d, c->rho_host.data(), sizeof(float) * p->Nz, cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaMemcpyAsync(wet_d, wet.data(), sizeof(float) * p->Nz, cudaMemcpyHostToDevice, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(d.bid, 0xFF, ns * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.val, 0, c->pages * c->L * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.vmask, 0, c->pages * sizeof(uint2), s) == cudaSuccess &&
         cudaMemsetAsync(d.pbase, 0, NcB * 4, s) == cudaSuccess;
    for (int k = 0; k < 2 && ok; ++k) ok = cudaMemsetAsync(d.occ[k], 0, NcB * 4, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(d.edep, 0, NcB * 8, s) == cudaSuccess && cudaMemsetAsync(d.e_cut, 0, NcB * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.e_nuc, 0, NcB * 8, s) == cudaSuccess && cudaMemsetAsync(d.e_bnd, 0, NcB * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.w_cut, 0, NcB * 4, s) == cudaSuccess && cudaMemsetAsync(d.w_nuc, 0, NcB * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.w_bnd, 0, NcB * 4, s) == cudaSuccess && cudaMemsetAsync(d.act_gen, 0, NcB * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.cls, 0, NcB, s) == cudaSuccess && cudaMemsetAsync(d.c2b, 0xFF, NcB * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_edep, 0, NcB * 8, s) == cudaSuccess && cudaMemsetAsync(d.dl_ecut, 0, NcB * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_enuc, 0, NcB * 8, s) == cudaSuccess && cudaMemsetAsync(d.dl_ebnd, 0, NcB * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_wcut, 0, NcB * 4, s) == cudaSuccess && cudaMemsetAsync(d.dl_wnuc, 0, NcB * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.dl_wbnd, 0, NcB * 4, s) == cudaSuccess &&
         cudaMemsetAsync(d.ctab, 0xFF, c->ctab_words * 8, s) == cudaSuccess &&
         cudaMemsetAsync(d.ccount, 0, c->ccount_n * sizeof(int), s) == cudaSuccess &&
         cudaMemsetAsync(d.bkt_ids, 0xFF, (size_t)4 * d.listed_cap * kKb * 4, s) == cudaSuccess;
    if (!ok) return bail(fail(SM2D_ERR_CUDA, "initial copies failed"));
    {   // the fine-threshold range, evaluated by the device LUT itself
        void* q1 = nullptr;
        if ((rc = dalloc(*c, &q1, sizeof(float)))) return bail(rc);
        float* rf = static_cast<float*>(q1);
        k_eval_range<<<1, 1, 0, s>>>(d, fmaxf(p->E_fine_on, d.lutEmin), rf);
        if (cudaMemcpyAsync(&d.R_fine_on, rf, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return bail(fail(SM2D_ERR_CUDA, "LUT setup"));
        // the range below which the precision form inverts the LUT in double
        k_eval_range<<<1, 1, 0, s>>>(d, fmaxf(10.0f, d.lutEmin), rf);
        if (cudaMemcpyAsync(&d.R_prec, rf, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return bail(fail(SM2D_ERR_CUDA, "LUT setup"));
        void* q2 = nullptr;
        if ((rc = dalloc(*c, &q2, sizeof(float4) * (size_t)d.N_E))) return bail(rc);
        k_k2_table<<<(d.N_E + 255) / 256, 256, 0, s>>>(d, static_cast<float4*>(q2));
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
            return bail(fail(SM2D_ERR_CUDA, "K2 table setup"));
        d.k2tab = static_cast<const float4*>(q2);
    }
    // every lane starts with the problem's tables
    c->fe_host.assign(3 * BN + B, 0.0f);
    c->fe_E0.assign(B, -1.0f);
    c->fe_sx.assign(B, -1.0f);
    c->fe_lo = B;
    c->fe_hi = -1;
    for (int ln = 0; ln < B; ++ln) {
        if (ln == 0) set_lane_fe(*c, 0, p->E0, p->sigma_x_initial);
        else {
            for (int k = 0; k < 3; ++k)
                std::copy_n(c->fe_host.data() + k * BN, p->Nz, c->fe_host.data() + k * BN + (size_t)ln * p->Nz);
            c->fe_host[3 * BN + ln] = p->sigma_x_initial;
            c->fe_E0[ln] = p->E0;
            c->fe_sx[ln] = p->sigma_x_initial;
            c->fe_hi = ln;
        }
    }
    if (upload_lane_fe(*c)) return bail(SM2D_ERR_CUDA);
    if (push_state(*c)) return bail(SM2D_ERR_CUDA);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // warp-per-cell kernels: 8 blocks per SM (the selection kernels are
    // latency-bound and gain from the warps in flight; finalize's last-block
    // step grows with the grid beyond that)
    c->sms = std::max(sms, 1);
    if ((rc = apply_shape(*c))) return bail(rc);
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
    if (h->gs_host) cudaFreeHost(h->gs_host);
    if (h->ls_host) cudaFreeHost(h->ls_host);
    if (h->beams_host) cudaFreeHost(h->beams_host);
    for (void* p : {(void*)h->plan_beams_dev, (void*)h->plan_fe_dev, (void*)h->plan_res_dev, (void*)h->plan_dose_dev,
                    (void*)h->plan_order_dev})
        if (p) cudaFree(p);
    if (h->s) cudaStreamDestroy(h->s);
    delete h;
    return 0;
}

int sm2d_local_bins(sm2d_handle h) { return h ? h->L : SM2D_ERR_ARG; }
int sm2d_lanes(sm2d_handle h) { return h ? h->B : SM2D_ERR_ARG; }

// ---------------------------------------------------------------- single spot (lane 0)
int sm2d_inject_async(sm2d_handle h, const sm2d_beam* b) {
    if (!h || !b) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    if (host_gaussian(*b) && b->n_samples <= 0) return fail(SM2D_ERR_ARG, "n_samples must be positive");
    int max_n = 1;
    int rc = stage_beams(c, b, 1, &max_n);
    if (rc) return rc;
    set_lane_fe(c, 0, c.p.E0, c.p.sigma_x_initial);   // a single spot keeps the problem's tables
    if ((rc = upload_lane_fe(c))) return rc;
    if ((rc = DISPATCH(c, inject, max_n, true, false))) return rc;
    c.injected = true;
    return 0;
}

int sm2d_inject(sm2d_handle h, const sm2d_beam* b) {
    if (!h || !b) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    int rc = sync_state(c);
    if (rc) return rc;
    if (c.gs_host->occ_n[c.gs_host->parity] != 0)
        return fail(SM2D_ERR_STATE, "phase space not empty: call sm2d_reset before injecting");
    if ((rc = sm2d_inject_async(h, b))) return rc;
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

// inject_source_kernel with its spreads (k1k6_pipeline.cu:300-427).  Without
// spreads (sigma_theta <= 1e-4 and sigma_x <= 0.01) it is the pencil branch;
// otherwise the cells within +-4 sigma_x of x0 (clamped to the grid) take
// Gaussian weights of their centres, normalised over those cells, on the 7
// angle nodes when sigma_theta > 1e-4.  Source accounting as the wrapper
// books a non-Gaussian source: W_total and E0 W_total injected.
static int float_to_index(float v) {   // a float-to-int conversion that saturates
    if (!(v == v)) return 0;
    if (v >= 1e9f) return 1000000000;
    if (v <= -1e9f) return -1000000000;
    return (int)v;
}

int sm2d_inject_quadrature(sm2d_handle h, const sm2d_beam* b) {
    if (!h || !b) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    const bool ang = b->sigma_theta > 0.0001f, spat = b->sigma_x > 0.01f;
    if (!ang && !spat) {
        sm2d_beam p = *b;
        p.sigma_x = p.sigma_theta = p.sigma_E = 0.0f;
        p.n_samples = 1;
        return sm2d_inject(h, &p);
    }
    if (!(b->sigma_x > 0.0f) || !std::isfinite(b->sigma_x) || !std::isfinite(b->x0))
        return fail(SM2D_ERR_ARG, "the quadrature source needs a finite sigma_x > 0 (its cell weights divide by sigma_x^2)");
    int rc = sync_state(c);
    if (rc) return rc;
    if (c.gs_host->occ_n[c.gs_host->parity] != 0)
        return fail(SM2D_ERR_STATE, "phase space not empty: call sm2d_reset before injecting");
    // cells within +-4 sigma_x (k1k6_pipeline.cu:351-364)
    const float lo = b->x0 - 4.0f * b->sigma_x, hi = b->x0 + 4.0f * b->sigma_x;
    int ix0 = float_to_index((lo - c.p.x_min) / c.p.dx), ix1 = float_to_index((hi - c.p.x_min) / c.p.dx) + 1;
    ix0 = std::max(ix0, 0);
    ix1 = std::min(ix1, c.p.Nx);
    BeamArgs a = beam_args(*b);
    a.kind = 1;
    a.q_ix0 = ix0;
    a.q_nx = std::max(ix1 - ix0, 0);
    a.n = (ang ? 7 : 1) * a.q_nx;
    for (int ln = 0; ln < c.B; ++ln) c.beams_host[ln] = ln == 0 ? a : BeamArgs{};
    CK(cudaMemcpyAsync(c.beams_dev, c.beams_host, sizeof(BeamArgs) * c.B, cudaMemcpyHostToDevice, c.s));
    set_lane_fe(c, 0, c.p.E0, c.p.sigma_x_initial);
    if ((rc = upload_lane_fe(c))) return rc;
    if ((rc = DISPATCH(c, inject, std::max(a.n, 1), true, false))) return rc;
    c.injected = true;
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

// A caller's phase space in a single-lane engine: its values were copied in
// the dense layout, so the pages of cell gc are 32 gc .. 32 gc + 31, all of
// the lane's region held until the next classification consumes them.
static int pages_identity(Ctx& c, int par, int n_listed) {
    k_pages_identity<<<(unsigned)std::min((c.d.Nc + 255) / 256, 4096), 256, 0, c.s>>>(c.d, par, n_listed);
    CK(cudaGetLastError());
    c.ls_host[0].pool_top = n_listed > 0 ? c.d.pool_lane : 0;
    return 0;
}

int sm2d_set_psi_in(sm2d_handle h, const uint32_t* bid, const float* val) {
    if (!h || !bid || !val) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    if (c.B != 1) return fail(SM2D_ERR_STATE, "sm2d_set_psi_in needs a single-lane engine");
    int rc = sync_state(c);
    if (rc) return rc;
    if ((rc = DISPATCH(c, clear_all, 0))) return rc;   // drop what the lists hold
    CK(cudaStreamSynchronize(c.s));
    const int par = c.gs_host->parity;
    const size_t ns = (size_t)c.d.Nc * kKb;
    std::vector<int> occ(c.d.Nc, 0), list;
    for (int cell = 0; cell < c.d.Nc; ++cell)
        for (int k = 0; k < kKb; ++k)
            if (bid[(size_t)cell * kKb + k] != kEmpty) {
                occ[cell] = 1;
                list.push_back(cell);
                break;
            }
    CK(cudaMemcpyAsync(c.d.bid, bid, ns * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(c.d.val, val, ns * c.L * 4, cudaMemcpyHostToDevice, c.s));   // pages numbered like the slots
    if ((rc = DISPATCH(c, build_masks, ns))) return rc;
    CK(cudaMemcpyAsync(c.d.occ[par], occ.data(), sizeof(int) * occ.size(), cudaMemcpyHostToDevice, c.s));
    if (!list.empty())
        CK(cudaMemcpyAsync(c.d.occ_list[par], list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, c.s));
    if ((rc = pages_identity(c, par, (int)list.size()))) return rc;
    c.gs_host->occ_n[par] = (int)list.size();
    c.gs_host->occ_n[par ^ 1] = 0;
    c.ls_host[0].done = 0;
    if ((rc = push_state(c))) return rc;
    CK(cudaStreamSynchronize(c.s));
    c.injected = true;
    return 0;
}

int sm2d_get_psi_in(sm2d_handle h, uint32_t* bid, float* val) {
    if (!h || !bid) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    const size_t ns = (size_t)c.d.Nc * kKb;
    CK(cudaMemcpyAsync(bid, c.d.bid, ns * 4, cudaMemcpyDeviceToHost, c.s));
    if (val) {   // the values in the dense layout, through a device buffer of that size
        float* tmp = nullptr;
        CK(cudaMallocAsync(reinterpret_cast<void**>(&tmp), ns * c.L * 4, c.s));
        int rc = DISPATCH(c, gather_psi, tmp);
        if (!rc && cudaMemcpyAsync(val, tmp, ns * c.L * 4, cudaMemcpyDeviceToHost, c.s) != cudaSuccess)
            rc = fail(SM2D_ERR_CUDA, "psi copy");
        cudaFreeAsync(tmp, c.s);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

// psi_in from device arrays in the same layout: the ids come to the host
// once to list the occupied cells, the values are copied on the device
int sm2d_set_psi_in_device(sm2d_handle h, const uint32_t* d_bid, const float* d_val) {
    if (!h || !d_bid || !d_val) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    if (c.B != 1) return fail(SM2D_ERR_STATE, "sm2d_set_psi_in_device needs a single-lane engine");
    int rc = sync_state(c);
    if (rc) return rc;
    if ((rc = DISPATCH(c, clear_all, 0))) return rc;
    const int par = c.gs_host->parity;
    const size_t ns = (size_t)c.d.Nc * kKb;
    std::vector<uint32_t> bid(ns);
    CK(cudaMemcpyAsync(bid.data(), d_bid, ns * 4, cudaMemcpyDeviceToHost, c.s));
    CK(cudaMemcpyAsync(c.d.bid, d_bid, ns * 4, cudaMemcpyDeviceToDevice, c.s));
    CK(cudaMemcpyAsync(c.d.val, d_val, ns * c.L * 4, cudaMemcpyDeviceToDevice, c.s));   // pages numbered like the slots
    if ((rc = DISPATCH(c, build_masks, ns))) return rc;
    CK(cudaStreamSynchronize(c.s));
    std::vector<int> occ(c.d.Nc, 0), list;
    for (int cell = 0; cell < c.d.Nc; ++cell)
        for (int k = 0; k < kKb; ++k)
            if (bid[(size_t)cell * kKb + k] != kEmpty) {
                occ[cell] = 1;
                list.push_back(cell);
                break;
            }
    CK(cudaMemcpyAsync(c.d.occ[par], occ.data(), sizeof(int) * occ.size(), cudaMemcpyHostToDevice, c.s));
    if (!list.empty())
        CK(cudaMemcpyAsync(c.d.occ_list[par], list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, c.s));
    if ((rc = pages_identity(c, par, (int)list.size()))) return rc;
    c.gs_host->occ_n[par] = (int)list.size();
    c.gs_host->occ_n[par ^ 1] = 0;
    c.ls_host[0].done = 0;
    if ((rc = push_state(c))) return rc;
    CK(cudaStreamSynchronize(c.s));
    c.injected = true;
    return 0;
}

int sm2d_get_psi_in_device(sm2d_handle h, uint32_t* d_bid, float* d_val) {
    if (!h || !d_bid) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    const size_t ns = (size_t)c.d.Nc * kKb;
    CK(cudaMemcpyAsync(d_bid, c.d.bid, ns * 4, cudaMemcpyDeviceToDevice, c.s));
    if (d_val) {
        const int rc = DISPATCH(c, gather_psi, d_val);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

int sm2d_set_source_accounting(sm2d_handle h, const double* v7) {
    if (!h || !v7) return fail(SM2D_ERR_ARG, "null argument");
    Ctx& c = *h;
    int rc = sync_state(c);
    if (rc) return rc;
    LaneState& L = c.ls_host[0];
    L.src_inj_w = (float)v7[0];
    L.src_oog_w = (float)v7[1];
    L.src_slot_w = (float)v7[2];
    L.src_inj_e = v7[3];
    L.src_oog_e = v7[4];
    L.src_slot_e = v7[5];
    L.src_rep_loss = v7[6];
    L.include_source = 1;
    return push_state(c);
}

int sm2d_step(sm2d_handle h, int* n_active, int* n_coarse) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space: call sm2d_inject or sm2d_set_psi_in first");
    int rc = DISPATCH(c, launch_body, true, false, true);
    if (rc) return rc;
    if ((rc = sync_state(c))) return rc;
    if (c.gs_host->bin_ovf) return fail(SM2D_ERR_ALLOC, "cell list, bin list or value pages of a lane: capacity exceeded");
    // classify, lists, claim pass, selection, deposit pass, K4 bucket move, finalize
    for (int k = 0; k < 7; ++k) CK(cudaEventElapsedTime(&c.step_ms[k], c.ev[k], c.ev[k + 1]));
    if (n_active) *n_active = c.ls_host[0].done ? 0 : c.ls_host[0].n_active;
    if (n_coarse) *n_coarse = c.ls_host[0].done ? 0 : c.ls_host[0].n_coarse;
    return 0;
}

static int run_impl(Ctx& c, int max_it, int* done_iters, float* ms) {
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space: call sm2d_inject or sm2d_set_psi_in first");
    if (max_it <= 0) return fail(SM2D_ERR_ARG, "max_iterations must be positive");
    int rc = build_graph(c);
    if (rc) return rc;
    if ((rc = sync_state(c))) return rc;
    const int start = c.ls_host[0].iter;
    c.gs_host->max_pass = (int)std::min<long long>((long long)c.gs_host->pass + max_it, INT_MAX);
    if ((rc = push_state(c))) return rc;
    if (ms) CK(cudaEventRecord(c.ev[8], c.s));
    CK(cudaGraphLaunch(c.exec, c.s));
    if (ms) CK(cudaEventRecord(c.ev[9], c.s));
    CK(cudaStreamSynchronize(c.s));
    if (ms) CK(cudaEventElapsedTime(ms, c.ev[8], c.ev[9]));
    if ((rc = sync_state(c))) return rc;
    c.gs_host->max_pass = INT_MAX;
    if ((rc = push_state(c))) return rc;
    CK(cudaStreamSynchronize(c.s));
    if (done_iters) *done_iters = c.ls_host[0].iter - start;
    if (c.gs_host->bin_ovf) return fail(SM2D_ERR_ALLOC, "cell list, bin list or value pages of a lane: capacity exceeded");
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
    const unsigned long long cur = h->gs_host->gen;
    for (int i = 0; i < h->d.Nc; ++i) mask[i] = (cur != 0 && g[i] == cur) ? 1 : 0;
    return 0;
}

int sm2d_get_lists(sm2d_handle h, uint32_t* active, int* na, uint32_t* coarse, int* nc) {
    if (!h || !na || !nc) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    const LaneState& L = h->ls_host[0];
    *na = L.done ? 0 : L.n_active;
    *nc = L.done ? 0 : L.n_coarse;
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
    *out = h->ls_host[0].last;
    return 0;
}

int sm2d_get_audit_history(sm2d_handle h, sm2d_audit* out, int max_entries, int* n) {
    if (!h || !out || !n) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    *n = std::min(std::min(h->ls_host[0].iter, h->d.hist_cap), max_entries);
    if (*n > 0) CK(cudaMemcpyAsync(out, h->d.hist, sizeof(sm2d_audit) * *n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int sm2d_batch_audit_history(sm2d_handle h, int lane, sm2d_audit* out, int max_entries, int* n) {
    if (!h || !out || !n || lane < 0 || lane >= h->B) return fail(SM2D_ERR_ARG, "invalid argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    *n = std::min(std::min(h->ls_host[lane].iter, h->d.hist_cap), max_entries);
    if (*n > 0)
        CK(cudaMemcpyAsync(out, h->d.hist + (size_t)lane * h->d.hist_cap, sizeof(sm2d_audit) * *n,
                           cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int sm2d_get_scalars(sm2d_handle h, double* o) {
    if (!h || !o) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    const LaneState& L = h->ls_host[0];
    const IterGlobal& G = *h->gs_host;
    o[0] = L.transport_drop_w; o[1] = L.transport_drop_e; o[2] = L.audit_residual;
    o[3] = L.src_inj_w; o[4] = L.src_inj_e; o[5] = L.src_oog_w; o[6] = L.src_oog_e;
    o[7] = L.src_slot_w; o[8] = L.src_slot_e; o[9] = L.src_rep_loss;
    o[10] = L.iter; o[11] = L.cell_steps; o[12] = L.slots_in; o[13] = L.slots_out;
    o[14] = G.cand_ovf; o[15] = G.cand_miss; o[16] = G.bin_ovf;
    return 0;
}

int sm2d_get_debug_counters(sm2d_handle h, int stage, unsigned long long* counts, double* weights,
                            double* energies) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    if (stage < 2 || stage > 4) return fail(SM2D_ERR_ARG, "stage must be 2 (K2), 3 (K3) or 4 (K4)");
    int rc = sync_state(*h);
    if (rc) return rc;
    const DropCounters& D = h->gs_host->drops;
    for (int k = 0; k < 3; ++k) {
        if (counts) counts[k] = D.n[stage - 2][k];
        if (weights) weights[k] = D.w[stage - 2][k];
        if (energies) energies[k] = D.e[stage - 2][k];
    }
    return 0;
}

int sm2d_reset_debug_counters(sm2d_handle h, int stage) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    if (stage < 2 || stage > 4) return fail(SM2D_ERR_ARG, "stage must be 2 (K2), 3 (K3) or 4 (K4)");
    Ctx& c = *h;
    char* base = reinterpret_cast<char*>(c.d.gs) + offsetof(IterGlobal, drops);
    const int s = stage - 2;
    CK(cudaMemsetAsync(base + offsetof(DropCounters, n) + sizeof(unsigned long long) * 3 * s, 0,
                       sizeof(unsigned long long) * 3, c.s));
    CK(cudaMemsetAsync(base + offsetof(DropCounters, w) + sizeof(double) * 3 * s, 0, sizeof(double) * 3, c.s));
    CK(cudaMemsetAsync(base + offsetof(DropCounters, e) + sizeof(double) * 3 * s, 0, sizeof(double) * 3, c.s));
    CK(cudaStreamSynchronize(c.s));
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
    return reset_lanes(*h);
}

int sm2d_run_async(sm2d_handle h, int max_it) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space: call sm2d_inject or sm2d_set_psi_in first");
    if (max_it <= 0) return fail(SM2D_ERR_ARG, "max_iterations must be positive");
    int rc = build_graph(c);
    if (rc) return rc;
    k_set_pass_limit<<<1, 1, 0, c.s>>>(c.d.gs, max_it);
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

int sm2d_run_profiled(sm2d_handle h, int n, int* done_iters, float* ms7, int* launches, int* passes) {
    if (!h || !ms7 || n <= 0) return fail(SM2D_ERR_ARG, "invalid argument");
    Ctx& c = *h;
    if (!c.injected) return fail(SM2D_ERR_STATE, "no phase space");
    int rc = sync_state(c);
    if (rc) return rc;
    const int start = c.ls_host[0].iter;
    constexpr int E = 8;   // events per iteration
    const size_t need = (size_t)E * n;
    while (c.pev.size() < need) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        c.pev.push_back(e);
    }
    cudaEvent_t saved[E];
    memcpy(saved, c.ev, sizeof saved);
    // passes in chunks of 16, stopping once no lane has work
    int launched = 0;
    const int start_pass = c.gs_host->pass;
    while (launched < n) {
        const int m = std::min(16, n - launched);
        for (int i = launched; i < launched + m; ++i) {
            for (int k = 0; k < E; ++k) c.ev[k] = c.pev[(size_t)E * i + k];
            if ((rc = DISPATCH(c, launch_body, true, false, false))) break;
        }
        if (rc) break;
        launched += m;
        if ((rc = sync_state(c))) break;
        if (c.gs_host->halt) break;
    }
    memcpy(c.ev, saved, sizeof saved);
    if (rc) return rc;
    if ((rc = sync_state(c))) return rc;
    const int done = c.gs_host->pass - start_pass;   // passes that transported
    for (int k = 0; k < E - 1; ++k) ms7[k] = 0.0f;
    for (int i = 0; i < done; ++i)
        for (int k = 0; k < E - 1; ++k) {
            float t = 0.0f;
            CK(cudaEventElapsedTime(&t, c.pev[(size_t)E * i + k], c.pev[(size_t)E * i + k + 1]));
            ms7[k] += t;
        }
    if (done_iters) *done_iters = c.ls_host[0].iter - start;
    if (launches) *launches = launched * ((c.p.use_buckets ? 7 : 6) + (c.d.surr ? 2 : 0));
    if (passes) *passes = done;
    return 0;
}

int sm2d_get_step_timing(sm2d_handle h, float* ms7) {
    if (!h || !ms7) return fail(SM2D_ERR_ARG, "null argument");
    memcpy(ms7, h->step_ms, sizeof h->step_ms);
    return 0;
}

// ---------------------------------------------------------------- batched spots

static int check_beams(const sm2d_beam* beams, int n) {
    for (int i = 0; i < n; ++i)
        if (host_gaussian(beams[i]) && beams[i].n_samples <= 0)
            return fail(SM2D_ERR_ARG, "spot %d: n_samples must be positive", i);
    return 0;
}

int sm2d_batch_inject(sm2d_handle h, const sm2d_beam* beams, int n) {
    if (!h || (!beams && n > 0) || n < 0) return fail(SM2D_ERR_ARG, "invalid argument");
    Ctx& c = *h;
    if (n > c.B) return fail(SM2D_ERR_ARG, "%d beams for %d lanes", n, c.B);
    int rc = check_beams(beams, n);
    if (rc) return rc;
    if ((rc = reset_lanes(c))) return rc;
    int max_n = 1;
    if ((rc = stage_beams(c, beams, n, &max_n))) return rc;
    for (int ln = 0; ln < n; ++ln) set_lane_fe(c, ln, beams[ln].E0, beams[ln].sigma_x);
    if ((rc = upload_lane_fe(c))) return rc;
    if ((rc = DISPATCH(c, inject, max_n, false, false))) return rc;
    c.injected = true;
    return 0;
}

int sm2d_batch_results(sm2d_handle h, sm2d_spot_result* results, int n) {
    if (!h || !results || n < 0 || n > h->B) return fail(SM2D_ERR_ARG, "invalid argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) lane_result(h->ls_host[i], results[i]);
    return 0;
}

int sm2d_batch_dose(sm2d_handle h, double* dose, int n) {
    if (!h || !dose || n < 0 || n > h->B) return fail(SM2D_ERR_ARG, "invalid argument");
    int rc = enqueue_dose(*h);
    if (rc) return rc;
    CK(cudaMemcpyAsync(dose, h->dose_dev, sizeof(double) * h->d.Nc * n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

// ---------------------------------------------------------------- spot plan
int sm2d_plan_load(sm2d_handle h, const sm2d_beam* beams, int n_spots, int max_iterations, int with_dose) {
    if (!h || (!beams && n_spots > 0) || n_spots < 0 || max_iterations <= 0)
        return fail(SM2D_ERR_ARG, "invalid argument");
    Ctx& c = *h;
    int rc = check_beams(beams, n_spots);
    if (rc) return rc;
    if ((rc = build_graph(c))) return rc;
    const int Nz = c.d.Nz;
    const size_t per = 3 * (size_t)Nz + 1, n = (size_t)n_spots;
    // grow the device plan buffers (after the previous plan's work)
    if (n > c.plan_cap || (with_dose && n > c.plan_dose_cap)) {
        CK(cudaStreamSynchronize(c.s));
        auto grow = [&](void** p, size_t bytes) -> int {
            if (*p) cudaFree(*p);
            *p = nullptr;
            cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
            return e == cudaSuccess ? 0 : fail(SM2D_ERR_ALLOC, "plan buffers (%zu bytes): %s", bytes, cudaGetErrorString(e));
        };
        if (n > c.plan_cap) {
            c.plan_cap = 0;
            if ((rc = grow((void**)&c.plan_beams_dev, sizeof(BeamArgs) * n)) ||
                (rc = grow((void**)&c.plan_fe_dev, sizeof(float) * per * n)) ||
                (rc = grow((void**)&c.plan_res_dev, sizeof(sm2d_spot_result) * n)) ||
                (rc = grow((void**)&c.plan_order_dev, sizeof(int) * n)))
                return rc;
            c.plan_cap = n;
        }
        if (with_dose && n > c.plan_dose_cap) {
            c.plan_dose_cap = 0;
            if ((rc = grow((void**)&c.plan_dose_dev, sizeof(double) * (size_t)c.d.Nc * n))) return rc;
            c.plan_dose_cap = n;
        }
    }
    c.plan_beams_host.resize(n);
    for (size_t i = 0; i < n; ++i) c.plan_beams_host[i] = beam_args(beams[i]);
    // Fermi-Eyges tables per distinct (E0, sigma_x), on the host threads
    c.plan_fe_host.resize(per * n);
    std::unordered_map<unsigned long long, int> first;
    std::vector<int> src(n), uniq;
    for (size_t i = 0; i < n; ++i) {
        unsigned eb, sb;
        memcpy(&eb, &beams[i].E0, 4);
        memcpy(&sb, &beams[i].sigma_x, 4);
        auto ins = first.emplace(((unsigned long long)eb << 32) | sb, (int)i);
        src[i] = ins.first->second;
        if (ins.second) uniq.push_back((int)i);
    }
    auto fe_of = [&](int t, int T) {
        for (size_t k = t; k < uniq.size(); k += T) {
            const int i = uniq[k];
            float* f = c.plan_fe_host.data() + per * i;
            fermi_eyges_moments(beams[i].E0, Nz, c.d.dz, beams[i].sigma_x, f, f + Nz, f + 2 * Nz,
                                c.rho_host.empty() ? nullptr : c.rho_host.data());
            f[3 * Nz] = beams[i].sigma_x;
        }
    };
    const int T = (int)std::min<size_t>({(size_t)std::max(1u, std::thread::hardware_concurrency()), 16, uniq.size() / 16 + 1});
    if (T <= 1) fe_of(0, 1);
    else {
        std::vector<std::thread> pool;
        for (int t = 0; t < T; ++t) pool.emplace_back(fe_of, t, T);
        for (auto& th : pool) th.join();
    }
    for (size_t i = 0; i < n; ++i)
        if (src[i] != (int)i) std::copy_n(c.plan_fe_host.data() + per * src[i], per, c.plan_fe_host.data() + per * i);
    // the order the lanes take the spots: the longest first (the highest
    // energy, the deepest range), so that the plan does not end on a long
    // spot started late; results and dose maps stay in the plan's order
    c.plan_order_host.resize(n);
    for (size_t i = 0; i < n; ++i) c.plan_order_host[i] = (int)i;
    std::stable_sort(c.plan_order_host.begin(), c.plan_order_host.end(),
                     [&](int a, int b) { return beams[a].E0 > beams[b].E0; });
    // pageable sources: each copy has read its source when it returns
    if (n) {
        CK(cudaMemcpyAsync(c.plan_order_dev, c.plan_order_host.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.plan_beams_dev, c.plan_beams_host.data(), sizeof(BeamArgs) * n, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.plan_fe_dev, c.plan_fe_host.data(), sizeof(float) * per * n, cudaMemcpyHostToDevice, c.s));
    }
    c.plan_n = n_spots;
    c.plan_max_it = max_iterations;
    c.plan_dose_on = with_dose != 0;
    return 0;
}

int sm2d_plan_run_async(sm2d_handle h) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (c.plan_n == 0) return 0;
    int rc = build_graph(c);   // captured again after a change of the pass (surrogate, launch shape)
    if (rc) return rc;
    if ((rc = reset_lanes(c))) return rc;
    double* dose_out = c.plan_dose_on ? (c.plan_dose_ext ? c.plan_dose_ext : c.plan_dose_dev) : nullptr;
    k_plan_begin<<<1, 1, 0, c.s>>>(c.d, c.plan_beams_dev, c.plan_fe_dev, dose_out,
                                   c.plan_res_dev, c.plan_n, c.plan_max_it, c.lanes_in_flight, c.plan_order_dev);
    CK(cudaGetLastError());
    if ((rc = DISPATCH(c, refill, 0))) return rc;   // the first spots into every lane
    CK(cudaGraphLaunch(c.exec, c.s));
    k_plan_end<<<1, 1, 0, c.s>>>(c.d);
    CK(cudaGetLastError());
    c.injected = false;
    // the lanes now hold plan spots' tables: the next injection rebuilds its own
    std::fill(c.fe_E0.begin(), c.fe_E0.end(), NAN);
    return 0;
}

int sm2d_plan_results(sm2d_handle h, double* dose, sm2d_spot_result* results) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    const size_t n = (size_t)c.plan_n;
    if (dose && !c.plan_dose_on) return fail(SM2D_ERR_STATE, "the plan was loaded without dose maps");
    if (results && n)
        CK(cudaMemcpyAsync(results, c.plan_res_dev, sizeof(sm2d_spot_result) * n, cudaMemcpyDeviceToHost, c.s));
    if (dose && n)
        CK(cudaMemcpyAsync(dose, c.plan_dose_dev, sizeof(double) * (size_t)c.d.Nc * n, cudaMemcpyDeviceToHost, c.s));
    int rc = sync_state(c);
    if (rc) return rc;
    if (c.gs_host->bin_ovf) return fail(SM2D_ERR_ALLOC, "cell list, bin list or value pages of a lane: capacity exceeded");
    return 0;
}

int sm2d_page_stats(sm2d_handle h, int* pages_per_lane, int* peak_pages) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    int rc = sync_state(*h);
    if (rc) return rc;
    if (pages_per_lane) *pages_per_lane = h->d.pool_lane;
    if (peak_pages) *peak_pages = h->gs_host->pool_peak;
    return 0;
}

int sm2d_plan_stats(sm2d_handle h, int* passes, int* refills, double* bins) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    int rc = sync_state(*h);
    if (rc) return rc;
    if (passes) *passes = h->gs_host->pass;
    if (refills) *refills = h->gs_host->refills;
    if (bins) *bins = (double)h->gs_host->bins_total;
    return 0;
}

// ---------------------------------------------------------------- learned surrogate in the fine step
int sm2d_set_surrogate(sm2d_handle h, sm2d_mlp_handle m, float tol, int max_rows, int method_tables) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (m && !c.d.expect) return fail(SM2D_ERR_ARG, "the surrogate replaces the expectation form's tables (expectation = 1)");
    if (m && !method_tables && !mlp_calibrated(m))
        return fail(SM2D_ERR_STATE, "sm2d_set_surrogate before sm2d_mlp_calibrate");
    if (m && !(tol >= 0.0f)) return fail(SM2D_ERR_ARG, "tolerance %g", (double)tol);
    if (max_rows < 0) return fail(SM2D_ERR_ARG, "max_rows %d", max_rows);
    CK(cudaStreamSynchronize(c.s));
    if (m) {
        int rc = sm2d_mlp_sync(m);   // the network's weights are written on its own stream
        if (rc) return rc;
        const size_t rows = max_rows > 0 ? (size_t)max_rows : (size_t)std::min(c.d.bins_cap, 1 << 22);
        if (rows > (size_t)c.d.bins_cap)
            return fail(SM2D_ERR_ARG, "max_rows %d above the bin list's %d", max_rows, c.d.bins_cap);
        if (rows > c.k3_alloc) {
            float4* f = nullptr;
            int* b = nullptr;
            float* t = nullptr;
            int* fb = nullptr;
            if ((rc = dalloc(c, (void**)&f, sizeof(float4) * rows))) return rc;
            if ((rc = dalloc(c, (void**)&b, sizeof(int) * rows))) return rc;
            if ((rc = dalloc(c, (void**)&t, sizeof(float) * 32 * rows))) return rc;
            if ((rc = dalloc(c, (void**)&fb, sizeof(int) * rows))) return rc;
            c.d.kfeat = f;
            c.d.kbin = b;
            c.d.ktab = t;
            c.d.kfb = fb;
            c.k3_alloc = rows;
        }
        c.d.k3_cap = (int)rows;
        c.d.surr = 1;
        c.mlp = m;
        c.mlp_tol = tol;
        c.mlp_method = method_tables ? 1 : 0;
        int dev = 0, sms = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if ((rc = DISPATCH(c, rows_grid, sms))) return rc;
    } else {
        c.d.surr = 0;
        c.d.k3_cap = 0;
        c.mlp = nullptr;
    }
    // the device loop is captured again with the new pass
    if (c.exec) cudaGraphExecDestroy(c.exec);
    if (c.graph) cudaGraphDestroy(c.graph);
    c.exec = nullptr;
    c.graph = nullptr;
    return 0;
}

int sm2d_surrogate_stats(sm2d_handle h, double* out3) {
    if (!h || !out3) return fail(SM2D_ERR_ARG, "null argument");
    int rc = sync_state(*h);
    if (rc) return rc;
    out3[0] = (double)h->gs_host->k3_total + (double)std::min(std::max(h->gs_host->k3_rows, 0), h->d.k3_cap);
    out3[1] = (double)h->gs_host->k3_fb;
    out3[2] = (double)h->gs_host->k3_ovf;
    return 0;
}

// ---------------------------------------------------------------- launch shape and its autotuner
int sm2d_get_launch_shape(sm2d_handle h, int* shape4) {
    if (!h || !shape4) return fail(SM2D_ERR_ARG, "null argument");
    std::copy_n(h->shape, 4, shape4);
    return 0;
}

int sm2d_set_launch_shape(sm2d_handle h, const int* shape4) {
    if (!h || !shape4) return fail(SM2D_ERR_ARG, "null argument");
    for (int k = 0; k < 4; ++k)
        if (shape4[k] < (k < 2 ? 1 : 0) || shape4[k] > 32) return fail(SM2D_ERR_ARG, "launch shape entry %d: %d", k, shape4[k]);
    Ctx& c = *h;
    CK(cudaStreamSynchronize(c.s));
    std::copy_n(shape4, 4, c.shape);
    int rc = apply_shape(c);
    if (rc) return rc;
    if (c.exec) cudaGraphExecDestroy(c.exec);
    if (c.graph) cudaGraphDestroy(c.graph);
    c.exec = nullptr;
    c.graph = nullptr;
    return 0;
}

// Coordinate descent over the launch shape on the loaded plan: for each entry
// in turn (deposit pass, claim pass, warp-per-cell kernels, finalize) every
// candidate is timed on one run of the whole plan (CUDA events on the engine's
// stream, after one untimed run of the shape) and the fastest is kept.  The
// result does not depend on the shape (claims follow keys, not launch order).
int sm2d_set_lanes_in_flight(sm2d_handle h, int n) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    if (n < 0) return fail(SM2D_ERR_ARG, "lanes in flight %d", n);
    h->lanes_in_flight = n >= h->B ? 0 : n;
    return 0;
}

int sm2d_get_lanes_in_flight(sm2d_handle h, int* n) {
    if (!h || !n) return fail(SM2D_ERR_ARG, "null argument");
    *n = h->lanes_in_flight > 0 ? h->lanes_in_flight : h->B;
    return 0;
}

// One run of the loaded plan to warm the current settings, then one timed.
static int time_plan(sm2d_handle h, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
    Ctx& c = *h;
    int rc = sm2d_plan_run_async(h);
    if (!rc && cudaEventRecord(e0, c.s) != cudaSuccess) rc = fail(SM2D_ERR_CUDA, "event");
    if (!rc) rc = sm2d_plan_run_async(h);
    if (!rc && cudaEventRecord(e1, c.s) != cudaSuccess) rc = fail(SM2D_ERR_CUDA, "event");
    if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(SM2D_ERR_CUDA, "event sync");
    if (!rc && cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) rc = fail(SM2D_ERR_CUDA, "event time");
    return rc;
}

int sm2d_tune_lanes_in_flight(sm2d_handle h, int* lanes, float* best_ms) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (c.plan_n == 0) return fail(SM2D_ERR_STATE, "sm2d_tune_lanes_in_flight before sm2d_plan_load");
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // every lane, then 3/4, 1/2, 1/4, 1/8 and 1/16 of them (at most the
    // plan's spots, at least 8): each fewer lane in flight is a smaller working
    // set a pass, against a fixed cost per pass shared by fewer lanes
    const int top = std::min(c.B, c.plan_n);
    const int frac16[6] = {16, 12, 8, 4, 2, 1};
    int best = 0, rc = 0, prev = -1;
    float best_t = 0.0f;
    for (int q = 0; q < 6 && !rc; ++q) {
        const int n = std::max(std::min(top, 8), top * frac16[q] / 16);
        if (n == prev) continue;
        prev = n;
        c.lanes_in_flight = n >= c.B ? 0 : n;
        float t = 0.0f;
        rc = time_plan(h, e0, e1, &t);
        if (!rc && (best == 0 || t < best_t)) {
            best_t = t;
            best = n;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    c.lanes_in_flight = best >= c.B ? 0 : best;
    if (lanes) *lanes = best;
    if (best_ms) *best_ms = best_t;
    return 0;
}

int sm2d_autotune(sm2d_handle h, int* shape4, float* best_ms) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    Ctx& c = *h;
    if (c.plan_n == 0) return fail(SM2D_ERR_STATE, "sm2d_autotune before sm2d_plan_load");
    {   // the lanes in flight first, with the current shape
        const int rc = sm2d_tune_lanes_in_flight(h, nullptr, nullptr);
        if (rc) return rc;
    }
    int per_sm_keys = 0, per_sm_dep = 0;
    {
        int k = 0, t = 0;
        cudaError_t e = c.layout == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_transport<LayoutRef, PASS_KEYS>, kThreads, 0)
                                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_transport<LayoutB128, PASS_KEYS>, kThreads, 0);
        if (e == cudaSuccess)
            e = c.layout == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&t, k_transport<LayoutRef, PASS_DIRECT>, kThreads, 0)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&t, k_transport<LayoutB128, PASS_DIRECT>, kThreads, 0);
        if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
        per_sm_keys = std::max(k, 1);
        per_sm_dep = std::max(t, 1);
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto time_shape = [&](const int* sh, float* ms) -> int {   // the first run captures the loop again
        int rc = sm2d_set_launch_shape(h, sh);
        if (!rc) rc = time_plan(h, e0, e1, ms);
        return rc;
    };
    int best[4];
    std::copy_n(c.shape, 4, best);
    float best_t = 0.0f;
    int rc = time_shape(best, &best_t);
    const int order[4] = {3, 2, 0, 1};
    for (int oi = 0; oi < 4 && !rc; ++oi) {
        const int k = order[oi];
        std::vector<int> cand;
        if (k == 3) for (int v = 1; v <= per_sm_dep; ++v) cand.push_back(v);
        if (k == 2) for (int v = 1; v <= per_sm_keys; ++v) cand.push_back(v);
        if (k == 0) cand = {2, 4, 6, 8, 12, 16};
        if (k == 1) cand = {2, 4, 6, 8};
        for (int v : cand) {
            int trial[4];
            std::copy_n(best, 4, trial);
            if (trial[k] == v || (k >= 2 && trial[k] == 0 && v == (k == 3 ? per_sm_dep : per_sm_keys))) continue;
            trial[k] = v;
            float t = 0.0f;
            if ((rc = time_shape(trial, &t))) break;
            if (t < best_t) {
                best_t = t;
                std::copy_n(trial, 4, best);
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = sm2d_set_launch_shape(h, best))) return rc;
    if (shape4) std::copy_n(best, 4, shape4);
    if (best_ms) *best_ms = best_t;
    return 0;
}

int sm2d_batch_run(sm2d_handle h, const sm2d_beam* beams, int n_spots, int max_iterations, double* dose,
                   sm2d_spot_result* results) {
    if (!h) return fail(SM2D_ERR_ARG, "null handle");
    // dose maps into pinned host memory are written there by the device as
    // each spot completes, overlapped with the transport of the others;
    // other memory receives one copy at the end
    double* ext = nullptr;
    if (dose) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, dose) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer)
            ext = static_cast<double*>(a.devicePointer);
        (void)cudaGetLastError();
    }
    int rc = sm2d_plan_load(h, beams, n_spots, max_iterations, dose ? 1 : 0);
    if (rc) return rc;
    h->plan_dose_ext = ext;
    rc = sm2d_plan_run_async(h);
    if (!rc) rc = sm2d_plan_results(h, ext ? nullptr : dose, results);
    h->plan_dose_ext = nullptr;
    return rc;
}

}  // extern "C"
