// sm2d_stages.cu -- the reference's K-stages as stand-alone entries on
// caller-owned device arrays (K1 mask, list compaction, K4 bucket transfer,
// K5 audit, and the K5 audit on static scratch), the host-table entries, and
// diagnostics.  These mirror the reference's per-stage kernels one to one;
// the engine in sm2d_engine.cu runs its own fused forms of them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "sm2d.h"
#include "sm2d_common.cuh"
#include "sm2d_tables.h"

namespace sm2d {

static thread_local std::string g_err;
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

// ------------------------------------------------------------------ raw stage entries
template <int L>
__global__ void k_raw_k1(const uint32_t* __restrict__ bid, const float* __restrict__ val, uint8_t* mask,
                         const uint8_t* prev, int Nc, int b_on, int b_off, float wmin) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= Nc) return;
    float W = 0.0f;
    bool on = false, off = false;
    for (int s = 0; s < kKb; ++s) {
        const uint32_t b = bid[(size_t)cell * kKb + s];
        if (b == kEmpty) continue;
        const uint32_t be = (b >> 12) & 0xFFFu;
        if (be <= (uint32_t)b_on) on = true;
        if (be <= (uint32_t)b_off) off = true;
        const float* v = val + ((size_t)cell * kKb + s) * L;
        for (int l = 0; l < L; ++l) W += v[l];
    }
    const bool p = prev != nullptr && prev[cell] != 0;
    mask[cell] = ((on || (p && off)) && W > wmin) ? 1 : 0;
}

template <int L>
__global__ void k_raw_compact(const uint8_t* mask, const uint32_t* bid, const float* val, int Nc, uint32_t* active,
                              int* n_active, uint32_t* coarse, int* n_coarse) {
    __shared__ int s_w[2][32];
    __shared__ int s_base[2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    if (threadIdx.x == 0) { s_base[0] = 0; s_base[1] = 0; }
    __syncthreads();
    for (int c0 = 0; c0 < Nc; c0 += blockDim.x) {
        const int cell = c0 + threadIdx.x;
        int a = 0, c = 0;
        if (cell < Nc) {
            if (mask[cell] == 1) {
                a = 1;
            } else if (mask[cell] == 0) {
                for (int s = 0; s < kKb && !c; ++s) {
                    if (bid[(size_t)cell * kKb + s] == kEmpty) continue;
                    const float* v = val + ((size_t)cell * kKb + s) * L;
                    for (int l = 0; l < L; ++l)
                        if (v[l] > 0.0f) { c = 1; break; }
                }
            }
        }
        const unsigned ba = __ballot_sync(kFull, a), bc = __ballot_sync(kFull, c);
        if (lane == 0) { s_w[0][wid] = __popc(ba); s_w[1][wid] = __popc(bc); }
        __syncthreads();
        int oa = s_base[0], oc = s_base[1];
        for (int w = 0; w < wid; ++w) { oa += s_w[0][w]; oc += s_w[1][w]; }
        const unsigned lt = (1u << lane) - 1u;
        if (a) active[oa + __popc(ba & lt)] = (uint32_t)cell;
        if (c) coarse[oc + __popc(bc & lt)] = (uint32_t)cell;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 0; w < nwarp; ++w) { s_base[0] += s_w[0][w]; s_base[1] += s_w[1][w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { *n_active = s_base[0]; *n_coarse = s_base[1]; }
}

// K4_BucketTransfer (k4_transfer.cu:174-333) over caller arrays: per
// destination cell, pull the facing buckets of its four neighbours into
// psi_out (claim with fallback, lidx remap, drop accounting).  Warp per
// destination cell.
template <class Lay>
__device__ void bucket_gather_cell(const unsigned char* buckets, int bucket_bytes, const int* c2b, uint32_t* ids_out,
                                   float* vals_out, int cell, int Nx, int Nz, const float* Ee, int N_E, double* drop_w,
                                   double* drop_e, int lane) {
    const int ix = cell % Nx, iz = cell / Nx;
    for (int face = 0; face < 4; ++face) {
        int src = -1;
        if (face == 0 && iz > 0) src = cell - Nx;
        if (face == 1 && iz + 1 < Nz) src = cell + Nx;
        if (face == 2 && ix > 0) src = cell - 1;
        if (face == 3 && ix + 1 < Nx) src = cell + 1;
        if (src < 0) continue;
        const int base = c2b[src];
        if (base < 0) continue;
        const unsigned char* b = buckets + (size_t)(base + face) * bucket_bytes;
        const uint32_t sb = reinterpret_cast<const uint32_t*>(b)[lane];
        unsigned um = __ballot_sync(kFull, sb != kEmpty);
        const float* bv = reinterpret_cast<const float*>(b + 192);
        while (um) {
            const int s = __ffs(um) - 1;
            um &= um - 1;
            const uint32_t bid = __shfl_sync(kFull, sb, s);
            int os = 0;
            uint32_t sel = bid;
            if (lane == 0) os = claim_slot(ids_out + (size_t)cell * kKb, bid, sel);
            os = __shfl_sync(kFull, os, 0);
            sel = __shfl_sync(kFull, sel, 0);
            const float* v = bv + (size_t)s * Lay::L;
            if (os < 0) {
                double dw = 0.0, de = 0.0;
                for (int l = lane; l < Lay::L; l += 32) {
                    const float w = v[l];
                    if (w > 0.0f) {
                        int Eb = (int)((bid >> 12) & 0xFFFu) * Lay::NE + (l / Lay::NT) % Lay::NE;
                        Eb = max(0, min(Eb, N_E - 1));
                        const float E = Ee[Eb] + 1.0f * (0.5f * (Ee[Eb + 1] - Ee[Eb]));
                        dw += (double)w;
                        de += (double)E * (double)w;
                    }
                }
                dw = warp_sum(dw);
                de = warp_sum(de);
                if (lane == 0) { atomicAdd(drop_w, dw); atomicAdd(drop_e, de); }
                continue;
            }
            float* o = vals_out + ((size_t)cell * kKb + os) * Lay::L;
            for (int l = lane; l < Lay::L; l += 32) {
                const float w = v[l];
                if (w > 0.0f) atomicAdd(o + (sel != bid ? remap_lidx<Lay>(l, bid, sel) : l), w);
            }
        }
    }
}

template <class Lay>
__global__ void k_raw_gather(const unsigned char* buckets, int bucket_bytes, const int* c2b, uint32_t* ids_out,
                             float* vals_out, int Nx, int Nz, const float* Ee, int N_E, double* drop) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < Nx * Nz; cell += nw)
        bucket_gather_cell<Lay>(buckets, bucket_bytes, c2b, ids_out, vals_out, cell, Nx, Nz, Ee, N_E, drop,
                                drop + 1, lane);
}

struct RawK5 {
    const uint32_t *bid_in, *bid_out;
    const float *val_in, *val_out;
    const double *edep, *e_nuc, *e_bnd, *e_cut, *p_edep, *p_e_nuc, *p_e_bnd, *p_e_cut;
    const float *w_cut, *w_nuc, *w_bnd, *p_w_cut, *p_w_nuc, *p_w_bnd;
    const float* Ee;
    int N_E, NT, NE, L, Nc;
};

// K5_ConservationAudit over caller arrays (k5_audit.cu:22-167); the totals are
// reduced hierarchically in double and finalised by the last block.
__global__ void k_raw_k5(RawK5 a, double* acc /* [11] + counter */, float s_oog_w, float s_slot_w, double s_oog_e,
                         double s_slot_e, float drop_w, double drop_e, int inc_src, sm2d_audit* rep) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    double v[11] = {0};
    if (cell < a.Nc) {
        for (int pass = 0; pass < 2; ++pass) {
            const uint32_t* bid = pass ? a.bid_out : a.bid_in;
            const float* val = pass ? a.val_out : a.val_in;
            for (int s = 0; s < kKb; ++s) {
                const uint32_t b = bid[(size_t)cell * kKb + s];
                if (b == kEmpty) continue;
                for (int l = 0; l < a.L; ++l) {
                    const float w = val[((size_t)cell * kKb + s) * a.L + l];
                    if (w <= 0.0f) continue;
                    int Eb = (int)((b >> 12) & 0xFFFu) * a.NE + (l / a.NT) % a.NE;
                    Eb = max(0, min(Eb, a.N_E - 1));
                    const float E = a.Ee[Eb] + 1.0f * (0.5f * (a.Ee[Eb + 1] - a.Ee[Eb]));
                    v[pass] += (double)w;
                    v[2 + pass] += (double)w * (double)E;
                }
            }
        }
        v[4] = fmaxf(0.0f, a.w_cut[cell] - a.p_w_cut[cell]);
        v[5] = fmaxf(0.0f, a.w_nuc[cell] - a.p_w_nuc[cell]);
        v[6] = fmaxf(0.0f, a.w_bnd[cell] - a.p_w_bnd[cell]);
        v[7] = fmax(0.0, a.edep[cell] - a.p_edep[cell]);
        v[8] = fmax(0.0, a.e_cut[cell] - a.p_e_cut[cell]);
        v[9] = fmax(0.0, a.e_nuc[cell] - a.p_e_nuc[cell]);
        v[10] = fmax(0.0, a.e_bnd[cell] - a.p_e_bnd[cell]);
    }
    for (int k = 0; k < 11; ++k) {
        const double s = warp_sum(v[k]);
        if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(&acc[k], s);
    }
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned* cnt = reinterpret_cast<unsigned*>(&acc[11]);
        s_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!(s_last && threadIdx.x == 0)) return;
    __threadfence();
    volatile double* A = acc;
    sm2d_audit r;
    memset(&r, 0, sizeof r);
    r.W_in_total = (float)A[0];
    r.W_out_total = (float)A[1];
    r.E_in_total = A[2];
    r.E_out_total = A[3];
    r.W_cutoff_total = (float)A[4];
    r.W_nuclear_total = (float)A[5];
    r.W_boundary_total = (float)A[6];
    r.E_dep_total = A[7];
    r.E_cutoff_total = A[8];
    r.E_nuclear_total = A[9];
    r.E_boundary_total = A[10];
    r.W_transport_drop_total = fmaxf(0.0f, drop_w);
    r.E_transport_drop_total = fmax(0.0, drop_e);
    if (inc_src) {
        const float wso = fmaxf(0.0f, s_oog_w), wss = fmaxf(0.0f, s_slot_w);
        const double eso = fmax(0.0, s_oog_e), ess = fmax(0.0, s_slot_e);
        r.W_in_total += wso + wss;
        r.E_in_total += eso + ess;
        r.W_source_out_of_grid_total = wso;
        r.W_source_slot_drop_total = wss;
        r.E_source_out_of_grid_total = eso;
        r.E_source_slot_drop_total = ess;
    }
    r.processed_cells = a.Nc;
    const float Wr = r.W_out_total + r.W_cutoff_total + r.W_nuclear_total + r.W_boundary_total +
                     r.W_transport_drop_total + r.W_source_out_of_grid_total + r.W_source_slot_drop_total;
    r.W_error = fabsf(r.W_in_total - Wr) / fmaxf(r.W_in_total, 1e-20f);
    r.W_pass = (isfinite(r.W_error) && r.W_error < 1e-6f) ? 1 : 0;
    const double Er = r.E_out_total + r.E_dep_total + r.E_cutoff_total + r.E_nuclear_total + r.E_boundary_total +
                      r.E_transport_drop_total + r.E_source_out_of_grid_total + r.E_source_slot_drop_total;
    r.E_error = (float)(fabs(r.E_in_total - Er) / fmax(r.E_in_total, 1e-20));
    r.E_pass = (isfinite(r.E_error) && r.E_error < 1e-5f) ? 1 : 0;
    *rep = r;
}

// ---- K5 audit on static scratch (sm2d_k5_conservation_audit_static) ----
// File-scope scratch of the allocation-free K5 entry: one row of 11 partial
// sums per block (each written whole by its block, never accumulated) and,
// after the rows, the block-completion counter, which must be zero when a
// call starts (cleared by the entry before every launch and by the last
// block on exit).  All calls share it: calls whose kernels overlap on the
// GPU race.
constexpr int kK5StaticMaxBlocks = 2048;                 // 256 cells per block
constexpr int kK5StaticMaxCells = kK5StaticMaxBlocks * 256;
static __device__ __align__(256) double g_k5_scratch[kK5StaticMaxBlocks * 11 + 2];

__global__ void __launch_bounds__(256) k_raw_k5_static(RawK5 a, double* scratch, float s_oog_w, float s_slot_w,
                                                       double s_oog_e, double s_slot_e, float drop_w,
                                                       double drop_e, int inc_src, sm2d_audit* rep) {
    __shared__ double s_red[11][8];
    __shared__ double s_tree[256];
    __shared__ int s_last;
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double v[11] = {0};
    if (cell < a.Nc) {
        for (int pass = 0; pass < 2; ++pass) {
            const uint32_t* bid = pass ? a.bid_out : a.bid_in;
            const float* val = pass ? a.val_out : a.val_in;
            for (int s = 0; s < kKb; ++s) {
                const uint32_t b = bid[(size_t)cell * kKb + s];
                if (b == kEmpty) continue;
                for (int l = 0; l < a.L; ++l) {
                    const float w = val[((size_t)cell * kKb + s) * a.L + l];
                    if (w <= 0.0f) continue;
                    int Eb = (int)((b >> 12) & 0xFFFu) * a.NE + (l / a.NT) % a.NE;
                    Eb = max(0, min(Eb, a.N_E - 1));
                    const float E = a.Ee[Eb] + 1.0f * (0.5f * (a.Ee[Eb + 1] - a.Ee[Eb]));
                    v[pass] += (double)w;
                    v[2 + pass] += (double)w * (double)E;
                }
            }
        }
        v[4] = fmaxf(0.0f, a.w_cut[cell] - a.p_w_cut[cell]);
        v[5] = fmaxf(0.0f, a.w_nuc[cell] - a.p_w_nuc[cell]);
        v[6] = fmaxf(0.0f, a.w_bnd[cell] - a.p_w_bnd[cell]);
        v[7] = fmax(0.0, a.edep[cell] - a.p_edep[cell]);
        v[8] = fmax(0.0, a.e_cut[cell] - a.p_e_cut[cell]);
        v[9] = fmax(0.0, a.e_nuc[cell] - a.p_e_nuc[cell]);
        v[10] = fmax(0.0, a.e_bnd[cell] - a.p_e_bnd[cell]);
    }
    // block partials in a fixed order: warps, then the 8 warp sums
    for (int k = 0; k < 11; ++k) {
        const double w = warp_sum(v[k]);
        if (lane == 0) s_red[k][wid] = w;
    }
    __syncthreads();
    if (threadIdx.x < 11) {
        double b = 0.0;
        for (int w = 0; w < 8; ++w) b += s_red[threadIdx.x][w];
        scratch[(size_t)blockIdx.x * 11 + threadIdx.x] = b;
        __threadfence();
    }
    __syncthreads();
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(scratch + (size_t)kK5StaticMaxBlocks * 11);
    if (threadIdx.x == 0) s_last = atomicAdd(cnt, 1ull) == (unsigned long long)(gridDim.x - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // last block: totals over the block rows in a fixed order (strided
    // partial sums, then a binary tree), so repeated calls agree bit for bit
    double tot[11];
    for (int k = 0; k < 11; ++k) {
        double p = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            p += *(volatile double*)&scratch[(size_t)b * 11 + k];
        s_tree[threadIdx.x] = p;
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if (threadIdx.x < w) s_tree[threadIdx.x] += s_tree[threadIdx.x + w];
            __syncthreads();
        }
        tot[k] = s_tree[0];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    *cnt = 0ull;   // leave the counter at zero for the next call
    sm2d_audit r;
    memset(&r, 0, sizeof r);
    r.W_in_total = (float)tot[0];
    r.W_out_total = (float)tot[1];
    r.E_in_total = tot[2];
    r.E_out_total = tot[3];
    r.W_cutoff_total = (float)tot[4];
    r.W_nuclear_total = (float)tot[5];
    r.W_boundary_total = (float)tot[6];
    r.E_dep_total = tot[7];
    r.E_cutoff_total = tot[8];
    r.E_nuclear_total = tot[9];
    r.E_boundary_total = tot[10];
    r.W_transport_drop_total = fmaxf(0.0f, drop_w);
    r.E_transport_drop_total = fmax(0.0, drop_e);
    if (inc_src) {
        const float wso = fmaxf(0.0f, s_oog_w), wss = fmaxf(0.0f, s_slot_w);
        const double eso = fmax(0.0, s_oog_e), ess = fmax(0.0, s_slot_e);
        r.W_in_total += wso + wss;
        r.E_in_total += eso + ess;
        r.W_source_out_of_grid_total = wso;
        r.W_source_slot_drop_total = wss;
        r.E_source_out_of_grid_total = eso;
        r.E_source_slot_drop_total = ess;
    }
    r.processed_cells = a.Nc;
    const float Wr = r.W_out_total + r.W_cutoff_total + r.W_nuclear_total + r.W_boundary_total +
                     r.W_transport_drop_total + r.W_source_out_of_grid_total + r.W_source_slot_drop_total;
    r.W_error = fabsf(r.W_in_total - Wr) / fmaxf(r.W_in_total, 1e-20f);
    r.W_pass = (isfinite(r.W_error) && r.W_error < 1e-6f) ? 1 : 0;
    const double Er = r.E_out_total + r.E_dep_total + r.E_cutoff_total + r.E_nuclear_total + r.E_boundary_total +
                      r.E_transport_drop_total + r.E_source_out_of_grid_total + r.E_source_slot_drop_total;
    r.E_error = (float)(fabs(r.E_in_total - Er) / fmax(r.E_in_total, 1e-20));
    r.E_pass = (isfinite(r.E_error) && r.E_error < 1e-5f) ? 1 : 0;
    *rep = r;
}

// Device address of g_k5_scratch, looked up once per device at set-up
// (with that device current) and cached.
static int k5_static_scratch(double** out) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static void* addr[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SM2D_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(SM2D_ERR_ARG, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_k5_scratch);
        if (e != cudaSuccess || !p)
            return fail(SM2D_ERR_CUDA, "cudaGetSymbolAddress(g_k5_scratch): %s", cudaGetErrorString(e));
        addr[dev] = p;
    }
    *out = static_cast<double*>(addr[dev]);
    return 0;
}

// Both K5 entries index a slot's local bins as (l / nt_local) % N_E_local
// over `local_bins` values: refuse layouts that would divide by zero or read
// past a slot.
static int k5_check_layout(int L, int nt_local, int N_E_local, int N_E) {
    if (L != 128 && L != 256) return fail(SM2D_ERR_LAYOUT, "local_bins must be 256 or 128, got %d", L);
    if (nt_local <= 0 || N_E_local <= 0 || N_E <= 0 || L % (nt_local * N_E_local) != 0)
        return fail(SM2D_ERR_ARG, "invalid layout: nt_local %d, N_E_local %d, N_E %d", nt_local, N_E_local, N_E);
    return 0;
}

// ------------------------------------------------------------------ diagnostics
__global__ void k_math_eval(int fn, const float* __restrict__ x, float* __restrict__ y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = x[i];
    y[i] = fn == 0 ? sm2d_expf(v) : fn == 1 ? sm2d_logf(v) : fn == 2 ? sm2d_sinf(v) : fn == 3 ? sm2d_cosf(v) : sm2d_erff(v);
}



}  // namespace sm2d

using namespace sm2d;

extern "C" {

const char* sm2d_last_error(void) { return g_err.c_str(); }
int sm2d_version(void) { return 1; }
size_t sm2d_bucket_bytes(int L) { return (size_t)bucket_bytes_for(L); }

// ---------------------------------------------------------------- host tables
int sm2d_energy_grid_log(float E_min, float E_max, int N, float* edges, float* rep) {
    if (N <= 0 || !(E_min > 0.0f) || !(E_max > E_min) || !edges || !rep) return fail(SM2D_ERR_ARG, "invalid grid");
    energy_grid_log(E_min, E_max, N, edges, rep);
    return 0;
}
int sm2d_energy_grid_piecewise(int n, const float* g, float* edges, float* rep) {
    if (n <= 0 || !g) return fail(SM2D_ERR_ARG, "invalid groups");
    for (int k = 0; k < n; ++k)
        if (!(g[3 * k + 2] > 0.0f) || !(g[3 * k + 1] > g[3 * k])) return fail(SM2D_ERR_ARG, "invalid group %d", k);
    if (edges && !rep) return fail(SM2D_ERR_ARG, "rep is null");
    return energy_grid_piecewise(n, g, edges, rep);
}
int sm2d_angular_grid(float lo, float hi, int N, float* edges, float* rep) {
    if (N <= 0 || !(hi > lo) || !edges || !rep) return fail(SM2D_ERR_ARG, "invalid grid");
    angular_grid(lo, hi, N, edges, rep);
    return 0;
}
int sm2d_range_lut(int N, const float* rep, float* R, float* S, float* logE, float* logR, float* logS) {
    if (N <= 0 || !rep || !R || !S || !logE || !logR || !logS) return fail(SM2D_ERR_ARG, "null argument");
    range_lut(N, rep, R, S, logE, logR, logS);
    return 0;
}
int sm2d_fermi_eyges(float E0, int Nz, float dz, float sx0, float* A, float* B, float* S) {
    if (Nz <= 0 || !(dz > 0.0f) || !A || !B || !S) return fail(SM2D_ERR_ARG, "invalid argument");
    fermi_eyges_moments(E0, Nz, dz, sx0, A, B, S);
    return 0;
}

int sm2d_fermi_eyges_density(float E0, int Nz, float dz, float sx0, const float* rho, float* A, float* B, float* S) {
    if (Nz <= 0 || !A || !B || !S || !rho) return fail(SM2D_ERR_ARG, "invalid argument");
    fermi_eyges_moments(E0, Nz, dz, sx0, A, B, S, rho);
    return 0;
}

// ---------------------------------------------------------------- raw stage entries
int sm2d_k1_active_mask(const uint32_t* bid, const float* val, uint8_t* mask, const uint8_t* prev, int Nx, int Nz,
                        int L, int b_on, int b_off, float wmin, void* stream) {
    if (!bid || !val || !mask || Nx <= 0 || Nz <= 0) return fail(SM2D_ERR_ARG, "invalid argument");
    const int Nc = Nx * Nz, blocks = (Nc + 255) / 256;
    cudaStream_t s = (cudaStream_t)stream;
    if (L == 256) k_raw_k1<256><<<blocks, 256, 0, s>>>(bid, val, mask, prev, Nc, b_on, b_off, wmin);
    else if (L == 128) k_raw_k1<128><<<blocks, 256, 0, s>>>(bid, val, mask, prev, Nc, b_on, b_off, wmin);
    else return fail(SM2D_ERR_LAYOUT, "local_bins must be 256 or 128");
    CK(cudaGetLastError());
    return 0;
}

int sm2d_compact_lists(const uint8_t* mask, const uint32_t* bid, const float* val, int Nx, int Nz, int L,
                       uint32_t* active, int* n_active, uint32_t* coarse, int* n_coarse, void* stream) {
    if (!mask || !bid || !val || !active || !coarse || !n_active || !n_coarse) return fail(SM2D_ERR_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (L == 256) k_raw_compact<256><<<1, 1024, 0, s>>>(mask, bid, val, Nx * Nz, active, n_active, coarse, n_coarse);
    else if (L == 128) k_raw_compact<128><<<1, 1024, 0, s>>>(mask, bid, val, Nx * Nz, active, n_active, coarse, n_coarse);
    else return fail(SM2D_ERR_LAYOUT, "local_bins must be 256 or 128");
    CK(cudaGetLastError());
    return 0;
}

int sm2d_k4_bucket_transfer(const void* buckets, const int* c2b, float* val_out, uint32_t* bid_out, int Nx, int Nz,
                            int L, int nt_local, int ne_local, int nx_sub, const float* Ee, int N_E, int N_E_local,
                            double* drop, void* stream) {
    if (!buckets || !c2b || !val_out || !bid_out || !Ee || !drop) return fail(SM2D_ERR_ARG, "null argument");
    (void)N_E_local;
    cudaStream_t s = (cudaStream_t)stream;
    const int blocks = std::max(1, std::min((Nx * Nz + 7) / 8, 65535));
    if (L == 256 && nt_local == 4 && ne_local == 2 && nx_sub == 8)
        k_raw_gather<LayoutRef><<<blocks, 256, 0, s>>>((const unsigned char*)buckets, bucket_bytes_for(256), c2b,
                                                        bid_out, val_out, Nx, Nz, Ee, N_E, drop);
    else if (L == 128 && nt_local == 8 && ne_local == 4 && nx_sub == 4)
        k_raw_gather<LayoutB128><<<blocks, 256, 0, s>>>((const unsigned char*)buckets, bucket_bytes_for(128), c2b,
                                                         bid_out, val_out, Nx, Nz, Ee, N_E, drop);
    else return fail(SM2D_ERR_LAYOUT, "layout not compiled");
    CK(cudaGetLastError());
    return 0;
}

int sm2d_k5_conservation_audit(const uint32_t* bid_in, const float* val_in, const uint32_t* bid_out,
                               const float* val_out, const double* EdepC, const double* e_nuc, const double* e_bnd,
                               const double* e_cut, const double* p_edep, const double* p_e_nuc,
                               const double* p_e_bnd, const double* p_e_cut, const float* w_cut,
                               const float* w_nuc, const float* w_bnd, const float* p_w_cut,
                               const float* p_w_nuc, const float* p_w_bnd, float s_oog_w, float s_slot_w,
                               double s_oog_e, double s_slot_e, float drop_w, double drop_e, int inc_src,
                               const float* Ee, int N_E, int nt_local, int N_E_local, int L, sm2d_audit* d_report,
                               int N_cells, void* stream) {
    if (!bid_in || !val_in || !bid_out || !val_out || !EdepC || !Ee || !d_report || N_cells <= 0)
        return fail(SM2D_ERR_ARG, "invalid argument");
    int rc = k5_check_layout(L, nt_local, N_E_local, N_E);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // accumulator of the device current at the call, allocated on first use
    // of that device and kept until exit
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static double* acc_of[kMaxDevices] = {};
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(SM2D_ERR_ARG, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!acc_of[dev]) CK(cudaMalloc(&acc_of[dev], 12 * sizeof(double)));
    double* acc = acc_of[dev];
    CK(cudaMemsetAsync(acc, 0, 12 * sizeof(double), s));
    RawK5 a{bid_in, bid_out, val_in, val_out, EdepC, e_nuc, e_bnd, e_cut, p_edep, p_e_nuc, p_e_bnd, p_e_cut,
            w_cut, w_nuc, w_bnd, p_w_cut, p_w_nuc, p_w_bnd, Ee, N_E, nt_local, N_E_local, L, N_cells};
    k_raw_k5<<<(N_cells + 255) / 256, 256, 0, s>>>(a, acc, s_oog_w, s_slot_w, s_oog_e, s_slot_e, drop_w, drop_e, inc_src,
                                                   d_report);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return 0;
}

int sm2d_k5_conservation_audit_static(
    const uint32_t* bid_in, const float* val_in, const uint32_t* bid_out, const float* val_out, const double* EdepC,
    const double* e_nuc, const double* e_bnd, const double* e_cut, const double* p_edep, const double* p_e_nuc,
    const double* p_e_bnd, const double* p_e_cut, const float* w_cut, const float* w_nuc, const float* w_bnd,
    const float* p_w_cut, const float* p_w_nuc, const float* p_w_bnd, float s_oog_w, float s_slot_w, double s_oog_e,
    double s_slot_e, float drop_w, double drop_e, int inc_src, const float* Ee, int N_E, int nt_local, int N_E_local,
    int L, sm2d_audit* d_report, int N_cells, void* stream) {
    if (!bid_in || !val_in || !bid_out || !val_out || !EdepC || !Ee || !d_report || N_cells <= 0)
        return fail(SM2D_ERR_ARG, "invalid argument");
    int rc = k5_check_layout(L, nt_local, N_E_local, N_E);
    if (rc) return rc;
    if (N_cells > kK5StaticMaxCells)
        return fail(SM2D_ERR_ARG, "N_cells %d exceeds the static scratch limit of %d cells", N_cells,
                    kK5StaticMaxCells);
    double* scratch = nullptr;
    rc = k5_static_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // the completion counter must start at zero
    CK(cudaMemsetAsync(scratch + (size_t)kK5StaticMaxBlocks * 11, 0, sizeof(unsigned long long), s));
    RawK5 a{bid_in, bid_out, val_in, val_out, EdepC, e_nuc, e_bnd, e_cut, p_edep, p_e_nuc, p_e_bnd, p_e_cut,
            w_cut, w_nuc, w_bnd, p_w_cut, p_w_nuc, p_w_bnd, Ee, N_E, nt_local, N_E_local, L, N_cells};
    k_raw_k5_static<<<(N_cells + 255) / 256, 256, 0, s>>>(a, scratch, s_oog_w, s_slot_w, s_oog_e, s_slot_e, drop_w,
                                                          drop_e, inc_src, d_report);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return 0;
}

// ---------------------------------------------------------------- diagnostics
int sm2d_math_eval(int fn, const float* x, float* y, int n) {
    if (!x || !y || n < 0 || fn < 0 || fn > 4) return fail(SM2D_ERR_ARG, "invalid argument");
    if (n == 0) return 0;
    float* buf = nullptr;
    CK(cudaMalloc(&buf, sizeof(float) * 2 * (size_t)n));
    int rc = 0;
    if (cudaMemcpy(buf, x, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(SM2D_ERR_CUDA, "copy");
    if (!rc) {
        k_math_eval<<<(n + 255) / 256, 256>>>(fn, buf, buf + n, n);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(y, buf + n, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = fail(SM2D_ERR_CUDA, "math kernel");
    }
    cudaFree(buf);
    return rc;
}

}  // extern "C"
