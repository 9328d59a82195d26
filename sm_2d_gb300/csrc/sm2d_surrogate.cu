// sm2d_surrogate.cu -- the learned redistribution surrogate of the fine
// transport step: a 4 -> 128 -> 128 -> 32 MLP (ReLU, softmax) whose 32
// outputs are the 8 theta x 4 E redistribution weights of one phase-space
// component over one step, trained on tables that the transport's own K3
// per-bin physics generates.
//
// Tensor-core kernels (tcgen05, sm_103a):
//   * operands are bf16 in shared memory, K-major, no swizzle: 8-row x 16-byte
//     core matrices stored as 128 contiguous bytes, core matrices adjacent in
//     K 128 bytes apart, 8-row groups (K/8) * 128 bytes apart;
//   * accumulators are fp32 in tensor memory (one 128-lane x N-column tile
//     per product, lane = row), read back by tcgen05.ld in the epilogues;
//   * one elected thread issues the MMAs and commits them to an mbarrier;
//   * the weights reach shared memory as pre-packed bf16 images through
//     cp.async.bulk (the update kernel writes them in the core-matrix layout).
// Every mbarrier wait is bounded; a timeout sets the handle's error flag, the
// CTA releases its tensor memory and returns.
//
// The training kernel runs the forward pass, the softmax cross-entropy
// gradient and the backward pass of one 128-sample tile in one CTA and leaves
// the tile's weight and bias gradients as a partial; the update kernel sums
// the partials in CTA order (deterministic) and applies Adam to fp32 master
// weights.  The inference kernel is persistent over tiles with the weights
// resident in shared memory, renormalises the softmax so each row sums to 1
// (the weight of the component is conserved), and can replace a sample's row
// by the plain table where the calibrated error of its input region exceeds a
// tolerance.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sm2d.h"
#include "sm2d_common.cuh"
#include "sm2d_redist.h"

namespace sm2d {

int handle_dev(sm2d_handle h, Dev* d, cudaStream_t* s);

namespace mlp {

constexpr int kIn = 16;     // input width of the first GEMM: 4 features as bf16 hi/lo pairs, zero padded
constexpr int kPair = 4;    // input columns 0-3: bf16(u); 4-7: 128 (u - bf16(u)), weighted by W1[:, 0:4] / 128
constexpr int kHid = 128;
constexpr int kOut = 32;    // 8 theta x 4 E
constexpr int kTile = 128;  // samples per CTA tile (the MMA's M)
// fp32 parameter vector: W1 [128][16], W2 [128][128], W3 [32][128], b1, b2, b3
constexpr int oW1 = 0, oW2 = oW1 + kHid * kIn, oW3 = oW2 + kHid * kHid, ob1 = oW3 + kOut * kHid, ob2 = ob1 + kHid,
              ob3 = ob2 + kHid, kParams = ob3 + kOut;
// bf16 weight images in the core-matrix layout (bytes)
constexpr int iW1 = 0, iW2 = iW1 + kHid * kIn * 2, iW2T = iW2 + kHid * kHid * 2, iW3 = iW2T + kHid * kHid * 2,
              iW3T = iW3 + kOut * kHid * 2, iB2X = iW3T + kOut * kHid * 2, iB3X = iB2X + kHid * 16 * 2,
              kImgBytes = iB3X + kOut * 16 * 2;
// Inference adds the biases on the tensor cores: each bias is a bf16 pair
// (value, rounding remainder) in K columns 8-9 of the W1 image and 0-1 of the
// B2X [128][16] and B3X [32][16] images, multiplied by constant-one input
// columns.  The training kernel's inputs hold zeros there and it adds the
// fp32 biases itself.
constexpr int kBiasCol = 8;
// Input space: the expectation form's redistribution of one fine-step
// component depends on its physics only through four numbers (features
// f = (s, u, r, cap)): s = sigma_theta / dtheta, the MCS angle in angle bins;
// u in [0, 1), where the step's mean energy lies between the two energy-bin
// centres around it (spacing D); r = sigma_E / D, the straggling in bins;
// cap = 1 when the energy window's top is the incoming bin (the mean lies in
// the first interval below it), 0 when it is the second centre above the mean.
constexpr float kSMax = 8.0f, kRMax = 4.0f;
constexpr float kFloor = 1.0f / 4096.0f;   // network weights below this are zero (2^-12)
// calibration regions: sqrt(s / 8) x u x sqrt(r / 4) x cap
constexpr int kRegS = 16, kRegU = 16, kRegR = 8, kRegC = 2, kRegions = kRegS * kRegU * kRegR * kRegC;
constexpr long long kSpinCycles = 2000000000LL;   // about one second at the SM clock
constexpr int kMaxRows = 1 << 30;                  // rows per call (tile indices stay within int)

// element offset of (row r, column k) of a K-major bf16 operand with K columns
__host__ __device__ constexpr int core_off(int r, int k, int K) {
    return (((r >> 3) * (K >> 3) + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((128u >> 4) & 0x3FFFu) << 16;   // leading byte offset: next core matrix along K
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;    // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                          // descriptor version (sm_100 family); no swizzle
    return d;
}
// kind::f16 instruction descriptor: bf16 A and B, fp32 D, both K-major
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}
// bounded wait for the phase of `parity` to complete
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > kSpinCycles) return false;
    }
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 16 consecutive fp32 columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive fp32 columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
// relu of two values rounded to a bf16 pair (a in the low half) in one instruction
__device__ __forceinline__ uint32_t pack2_relu(float a, float b) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}
// relu of 32 values as bf16 into row r, columns c..c+31 of a K-major operand
__device__ __forceinline__ void st_row32_relu(unsigned char* base, int r, int c, int K, const float* v) {
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        const float* x = v + 8 * h;
        const uint4 q = make_uint4(pack2_relu(x[0], x[1]), pack2_relu(x[2], x[3]), pack2_relu(x[4], x[5]),
                                   pack2_relu(x[6], x[7]));
        *reinterpret_cast<uint4*>(base + 2 * core_off(r, c + 8 * h, K)) = q;
    }
}
// 16 values as bf16 into row r, columns c..c+15 (c a multiple of 8) of a K-major operand
__device__ __forceinline__ void st_row16(unsigned char* base, int r, int c, int K, const float* v) {
    uint4 a = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
    uint4 b = make_uint4(pack2(v[8], v[9]), pack2(v[10], v[11]), pack2(v[12], v[13]), pack2(v[14], v[15]));
    *reinterpret_cast<uint4*>(base + 2 * core_off(r, c, K)) = a;
    *reinterpret_cast<uint4*>(base + 2 * core_off(r, c + 8, K)) = b;
}
// 16 values as bf16 into column r, rows c..c+15 of a K-major operand (the transpose)
__device__ __forceinline__ void st_col16(unsigned char* base, int r, int c, int K, const float* v) {
    __nv_bfloat16* p = reinterpret_cast<__nv_bfloat16*>(base);
#pragma unroll
    for (int j = 0; j < 16; ++j) p[core_off(c + j, r, K)] = __float2bfloat16_rn(v[j]);
}
__device__ __forceinline__ float ld_bf(const unsigned char* base, int r, int k, int K) {
    return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(base)[core_off(r, k, K)]);
}
// sum of row r (K columns) of a K-major bf16 operand, in column order
__device__ __forceinline__ float row_sum(const unsigned char* base, int r, int K) {
    float s = 0.0f;
    for (int k = 0; k < K; k += 8) {
        const uint4 q = *reinterpret_cast<const uint4*>(base + 2 * core_off(r, k, K));
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[j]);
            s += __bfloat162float(h.x);
            s += __bfloat162float(h.y);
        }
    }
    return s;
}

// ------------------------------------------------------------------ features and the plain table
// Network inputs of one sample: each feature scaled to [-1, 1] and written as
// a bf16 pair (hi, 128 x the rounding remainder).  The W1 image multiplies
// the remainder column of input i by bf16(W1[o][i]) / 128 (exact: a power of
// two), so the first GEMM forms bf16(W1[o][i]) (hi + remainder) and sees the
// fp32 input to about 16 bits.
__host__ __device__ inline void feature_row(const float* f, float* x16) {
    const float u[4] = {2.0f * fminf(fmaxf(f[0], 0.0f), kSMax) / kSMax - 1.0f, 2.0f * f[1] - 1.0f,
                        2.0f * fminf(fmaxf(f[2], 0.0f), kRMax) / kRMax - 1.0f, 2.0f * f[3] - 1.0f};
    for (int i = 0; i < 4; ++i) {
#ifdef __CUDA_ARCH__
        const float hi = __bfloat162float(__float2bfloat16_rn(u[i]));
#else
        const float hi = u[i];
#endif
        x16[i] = hi;
        x16[4 + i] = (u[i] - hi) * 128.0f;
    }
    for (int i = 8; i < kIn; ++i) x16[i] = 0.0f;
}
__device__ __forceinline__ int region_of(const float* f) {
    const int ia = min(kRegS - 1, max(0, (int)(sqrtf(fmaxf(f[0], 0.0f) / kSMax) * kRegS)));
    const int ib = min(kRegU - 1, max(0, (int)(f[1] * kRegU)));
    const int ic = min(kRegR - 1, max(0, (int)(sqrtf(fmaxf(f[2], 0.0f) / kRMax) * kRegR)));
    const int id = f[3] > 0.5f ? 1 : 0;
    return ((ia * kRegU + ib) * kRegR + ic) * kRegC + id;
}

// The expectation form's redistribution of one component (sm2d_redist.h),
// out[t + 8 e] = Mt[t] Me[e], on centres of uniform spacing: in units of the
// spacing, the mean energy u lies between centres 0 and 1; the window is
// (1, 0, -1, -2) when its top is capped at the incoming bin, (2, 1, 0, -1)
// otherwise.  The transport evaluates the same masses on the grid's centres.
__host__ __device__ inline void plain_table(const float* f, float* out) {
    float Mt[SM2D_RD_NT], Me[SM2D_RD_NE];
    const float cap1[4] = {1.0f, 0.0f, -1.0f, -2.0f}, cap0[4] = {2.0f, 1.0f, 0.0f, -1.0f};
    sm2d_rd_theta(fmaxf(f[0], 0.0f), Mt);
    sm2d_rd_energy(f[1], fmaxf(f[2], 0.0f), f[3] > 0.5f ? cap1 : cap0, SM2D_RD_NE - 1, Me);
    for (int e = 0; e < SM2D_RD_NE; ++e)
        for (int t = 0; t < SM2D_RD_NT; ++t) out[t + 8 * e] = Mt[t] * Me[e];
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float unit(uint32_t seed, uint32_t i, uint32_t k) {
    return ((float)(hash32(seed * 0x9E3779B9u ^ hash32(4u * i + k)) >> 8) + 0.5f) * (1.0f / 16777216.0f);
}
// training-set inputs: s = 8 a^2, u uniform, r = 4 c^2 (more samples at
// the small spreads that dominate), cap 0 or 1
__global__ void k_features(int n, uint32_t seed, float4* f) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float a = unit(seed, i, 0), b = unit(seed, i, 1), c = unit(seed, i, 2), e = unit(seed, i, 3);
        f[i] = make_float4(kSMax * a * a, b, kRMax * c * c, e < 0.5f ? 0.0f : 1.0f);
    }
}
__global__ void k_plain(int n, const float4* f, float4* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 q = f[i];
        const float fi[4] = {q.x, q.y, q.z, q.w};
        float t[kOut];
        plain_table(fi, t);
        for (int j = 0; j < kOut / 4; ++j) out[(size_t)i * 8 + j] = make_float4(t[4 * j], t[4 * j + 1], t[4 * j + 2], t[4 * j + 3]);
    }
}
// per-region maximum absolute weight error of the surrogate against the plain table
__global__ void k_calibrate(int n, const float4* f, const float* plain, const float* surr, int* err_bits) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 q = f[i];
        const float fi[4] = {q.x, q.y, q.z, q.w};
        float m = 0.0f;
        for (int k = 0; k < kOut; ++k) m = fmaxf(m, fabsf(plain[(size_t)i * kOut + k] - surr[(size_t)i * kOut + k]));
        atomicMax(err_bits + region_of(fi), __float_as_int(m));   // non-negative floats order as ints
    }
}

// ------------------------------------------------------------------ shared-memory plans
namespace tr {   // training kernel
constexpr int X = 0, XT = 4096, W1 = 8192, W2 = 12288, W3 = 45056, H1 = 53248, H1T = 86016, H2 = 118784,
              H2T = 151552, D3 = 184320, D3T = 192512, BAR = 200704, BYTES = BAR + 64;
}
namespace inf {  // inference kernel: weights shared by the CTA, then X and H of each warpgroup's tile
constexpr int WG = 4;                                       // warpgroups (tiles in flight) per CTA
constexpr int W1 = 0, W2 = 4096, W3 = 36864, ONES = 45056, B2X = 49152, B3X = 53248, TILE0 = 54272;
constexpr int XB = 4096, TILE_BYTES = XB + 32768;           // X [128][16], H [128][128] (H2 over H1)
constexpr int BAR = TILE0 + WG * TILE_BYTES, BYTES = BAR + 96;
}
static_assert(inf::BYTES <= 227 * 1024, "inference CTA exceeds shared memory");
static_assert(tr::BYTES <= 227 * 1024, "training tile exceeds shared memory");

// TMEM columns of the training kernel (512 allocated, one CTA per SM)
constexpr uint32_t cZ1 = 0, cZ2 = 128, cZ3 = 256, cW3T = 320, cH2g = 384, cW2g = 0, cH1g = 128, cW1g = 256;
static_assert(cH2g + kHid <= 512 && cW3T + kOut <= cH2g && cZ3 + kOut <= cW3T && cW1g + kIn <= cW3T,
              "training kernel's TMEM plan overlaps or exceeds 512 columns");
static_assert(inf::WG * 128 <= 512, "inference warpgroups need 128 TMEM columns each");

struct TrainArgs {
    const float4* feats;
    const float4* target;   // [n][32] as 8 float4
    int n;
    float scale;            // 1 / (samples of the step)
    const unsigned char* img;
    const float* params;    // fp32 master (biases read here)
    float* partial;         // [gridDim.x][kParams]
    float* ploss;           // [gridDim.x]
    int* err;
};

// Forward, loss gradient and backward of one 128-sample tile.
__global__ void __launch_bounds__(128, 1) k_train(TrainArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    // one barrier per weight transfer (each completes once) and one for the MMAs
    uint64_t* bar_w = reinterpret_cast<uint64_t*>(sm + tr::BAR);
    uint64_t* bar_w2t = bar_w + 1;
    uint64_t* bar_w3t = bar_w + 2;
    uint64_t* bar_m = bar_w + 3;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + tr::BAR + 32);
    float* red = reinterpret_cast<float*>(sm + tr::BAR + 48);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid;
    const int i = blockIdx.x * kTile + row;
    const bool live = i < a.n;
    const float* b1 = a.params + ob1;
    const float* b2 = a.params + ob2;
    const float* b3 = a.params + ob3;
    uint32_t pm = 0;   // phase of the MMA barrier
    bool ok = true;

    if (tid == 0) {
        bar_init(bar_w, 1);
        bar_init(bar_w2t, 1);
        bar_init(bar_w3t, 1);
        bar_init(bar_m, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot, 512);
    __syncthreads();
    if (tid == 0) {
        bar_expect(bar_w, kHid * kIn * 2 + kHid * kHid * 2 + kOut * kHid * 2);
        bulk_g2s(sm + tr::W1, a.img + iW1, kHid * kIn * 2, bar_w);
        bulk_g2s(sm + tr::W2, a.img + iW2, kHid * kHid * 2, bar_w);
        bulk_g2s(sm + tr::W3, a.img + iW3, kOut * kHid * 2, bar_w);
    }
    fence_after();
    const uint32_t tm = *tslot;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;

    // inputs: X [sample][16] and X^T [16][sample]
    {
        float x[kIn];
        if (live) {
            const float4 q = a.feats[i];
            const float f[4] = {q.x, q.y, q.z, q.w};
            feature_row(f, x);
        } else {
            for (int k = 0; k < kIn; ++k) x[k] = 0.0f;
        }
        st_row16(sm + tr::X, row, 0, kIn, x);
        st_col16(sm + tr::XT, row, 0, kTile, x);
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        fence_after();
        ok = bar_wait(bar_w, 0);
        if (ok) {
            mma(tm + cZ1, sdesc(su32(sm + tr::X), 2 * 128), sdesc(su32(sm + tr::W1), 2 * 128), idesc(128, 128), 0);
            mma_commit(bar_m);
        }
    }
    if (__syncthreads_or(!ok)) goto fail;
    ok = bar_wait(bar_m, pm);
    pm ^= 1;
    if (__syncthreads_or(!ok)) goto fail;
    fence_after();
    // layer 1 epilogue: H1 = relu(Z1 + b1) -> H1 and H1^T
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tmem_ld16(tm + lane_base + cZ1 + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + b1[c + j], 0.0f);
        if (!live) for (int j = 0; j < 16; ++j) v[j] = 0.0f;
        st_row16(sm + tr::H1, row, c, kHid, v);
        st_col16(sm + tr::H1T, row, c, kTile, v);
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        fence_after();
        for (int k = 0; k < kHid / 16; ++k)
            mma(tm + cZ2, sdesc(su32(sm + tr::H1) + 256 * k, 2048), sdesc(su32(sm + tr::W2) + 256 * k, 2048),
                idesc(128, 128), k > 0);
        mma_commit(bar_m);
    }
    ok = bar_wait(bar_m, pm);
    pm ^= 1;
    if (__syncthreads_or(!ok)) goto fail;
    fence_after();
    if (tid == 0) {   // W2 has been read: bring W2^T into its place for the backward pass
        bar_expect(bar_w2t, kHid * kHid * 2);
        bulk_g2s(sm + tr::W2, a.img + iW2T, kHid * kHid * 2, bar_w2t);
    }
    for (int c = 0; c < kHid; c += 16) {
        float v[16];
        tmem_ld16(tm + lane_base + cZ2 + c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + b2[c + j], 0.0f);
        if (!live) for (int j = 0; j < 16; ++j) v[j] = 0.0f;
        st_row16(sm + tr::H2, row, c, kHid, v);
        st_col16(sm + tr::H2T, row, c, kTile, v);
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        fence_after();
        for (int k = 0; k < kHid / 16; ++k)
            mma(tm + cZ3, sdesc(su32(sm + tr::H2) + 256 * k, 2048), sdesc(su32(sm + tr::W3) + 256 * k, 2048),
                idesc(128, kOut), k > 0);
        mma_commit(bar_m);
    }
    ok = bar_wait(bar_m, pm);
    pm ^= 1;
    if (__syncthreads_or(!ok)) goto fail;
    fence_after();
    if (tid == 0) {   // W3 has been read: W3^T into its place
        bar_expect(bar_w3t, kOut * kHid * 2);
        bulk_g2s(sm + tr::W3, a.img + iW3T, kOut * kHid * 2, bar_w3t);
    }
    // layer 3 epilogue: softmax, cross-entropy against the target, dZ3 = (p - y) scale
    {
        float z[kOut];
        tmem_ld16(tm + lane_base + cZ3, z);
        tmem_ld16(tm + lane_base + cZ3 + 16, z + 16);
        float y[kOut];
        if (live) {
            for (int j = 0; j < 8; ++j) {
                const float4 q = a.target[(size_t)i * 8 + j];
                y[4 * j] = q.x; y[4 * j + 1] = q.y; y[4 * j + 2] = q.z; y[4 * j + 3] = q.w;
            }
        } else {
            for (int k = 0; k < kOut; ++k) y[k] = 0.0f;
        }
        float m = -3.0e38f;
        for (int k = 0; k < kOut; ++k) { z[k] += b3[k]; m = fmaxf(m, z[k]); }
        float s = 0.0f;
        float e[kOut];
        for (int k = 0; k < kOut; ++k) { e[k] = sm2d_expf(z[k] - m); s += e[k]; }
        const float ls = sm2d_logf(s), inv = 1.0f / s;
        float loss = 0.0f;
        for (int k = 0; k < kOut; ++k) {
            loss -= y[k] * (z[k] - m - ls);
            e[k] = live ? (e[k] * inv - y[k]) * a.scale : 0.0f;
        }
        loss = live ? loss * a.scale : 0.0f;
        st_row16(sm + tr::D3, row, 0, kOut, e);
        st_row16(sm + tr::D3, row, 16, kOut, e + 16);
        st_col16(sm + tr::D3T, row, 0, kTile, e);
        st_col16(sm + tr::D3T, row, 16, kTile, e + 16);
        loss = warp_sumf(loss);
        if ((tid & 31) == 0) red[warp] = loss;
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        a.ploss[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
        fence_after();
        ok = bar_wait(bar_w2t, 0);
        if (ok) ok = bar_wait(bar_w3t, 0);
        if (ok) {
            // dW3^T [hid][out] = H2^T dZ3
            for (int k = 0; k < kTile / 16; ++k)
                mma(tm + cW3T, sdesc(su32(sm + tr::H2T) + 256 * k, 2048), sdesc(su32(sm + tr::D3T) + 256 * k, 2048),
                    idesc(128, kOut), k > 0);
            // dH2 [sample][hid] = dZ3 W3
            for (int k = 0; k < kOut / 16; ++k)
                mma(tm + cH2g, sdesc(su32(sm + tr::D3) + 256 * k, 512), sdesc(su32(sm + tr::W3) + 256 * k, 512),
                    idesc(128, kHid), k > 0);
            mma_commit(bar_m);
        }
    }
    if (__syncthreads_or(!ok)) goto fail;
    ok = bar_wait(bar_m, pm);
    pm ^= 1;
    if (__syncthreads_or(!ok)) goto fail;
    fence_after();
    // dZ2 = dH2 * (H2 > 0) -> dZ2 (over H1) and dZ2^T (over H2)
    for (int c = 0; c < kHid; c += 16) {
        float g[16];
        tmem_ld16(tm + lane_base + cH2g + c, g);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (!(ld_bf(sm + tr::H2T, c + j, row, kTile) > 0.0f)) g[j] = 0.0f;
        st_row16(sm + tr::H1, row, c, kHid, g);
        st_col16(sm + tr::H2, row, c, kTile, g);
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        fence_after();
        // dW2 [out][in] = dZ2^T H1
        for (int k = 0; k < kTile / 16; ++k)
            mma(tm + cW2g, sdesc(su32(sm + tr::H2) + 256 * k, 2048), sdesc(su32(sm + tr::H1T) + 256 * k, 2048),
                idesc(128, kHid), k > 0);
        // dH1 [sample][in] = dZ2 W2
        for (int k = 0; k < kHid / 16; ++k)
            mma(tm + cH1g, sdesc(su32(sm + tr::H1) + 256 * k, 2048), sdesc(su32(sm + tr::W2) + 256 * k, 2048),
                idesc(128, kHid), k > 0);
        mma_commit(bar_m);
    }
    ok = bar_wait(bar_m, pm);
    pm ^= 1;
    if (__syncthreads_or(!ok)) goto fail;
    fence_after();
    // dZ1 = dH1 * (H1 > 0) -> dZ1^T (over H2^T)
    for (int c = 0; c < kHid; c += 16) {
        float g[16];
        tmem_ld16(tm + lane_base + cH1g + c, g);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (!(ld_bf(sm + tr::H1T, c + j, row, kTile) > 0.0f)) g[j] = 0.0f;
        st_col16(sm + tr::H2T, row, c, kTile, g);
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        fence_after();
        // dW1 [hid][16] = dZ1^T X
        for (int k = 0; k < kTile / 16; ++k)
            mma(tm + cW1g, sdesc(su32(sm + tr::H2T) + 256 * k, 2048), sdesc(su32(sm + tr::XT) + 256 * k, 2048),
                idesc(128, kIn), k > 0);
        mma_commit(bar_m);
    }
    ok = bar_wait(bar_m, pm);
    pm ^= 1;
    if (__syncthreads_or(!ok)) goto fail;
    fence_after();
    // the tile's gradients: lane `row` holds row `row` of dW2, dW1 and dW3^T
    {
        float* g = a.partial + (size_t)blockIdx.x * kParams;
        const int j = row;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + cW2g + c, v);
            float4* o = reinterpret_cast<float4*>(g + oW2 + j * kHid + c);
            for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
        {
            float v[16];
            tmem_ld16(tm + lane_base + cW1g, v);
            float4* o = reinterpret_cast<float4*>(g + oW1 + j * kIn);
            for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
        for (int c = 0; c < kOut; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + cW3T + c, v);
            for (int q = 0; q < 16; ++q) g[oW3 + (c + q) * kHid + j] = v[q];
        }
        g[ob2 + j] = row_sum(sm + tr::H2, j, kTile);    // dZ2^T row j
        g[ob1 + j] = row_sum(sm + tr::H2T, j, kTile);   // dZ1^T row j
        if (j < kOut) g[ob3 + j] = row_sum(sm + tr::D3T, j, kTile);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_free(tm, 512);
    }
    return;
fail:
    if (tid == 0) atomicExch(a.err, 1);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_free(tm, 512);
    }
}

// What the inference kernel writes for a row whose calibrated region error
// exceeds the tolerance, and where the rows come from.
enum {
    INFER_TABLES = 0,      // the plain table in place of the network's row (fallback flag 1)
    INFER_TRANSPORT = 1,   // the transport's rows: fallback flag 1, row left unwritten (the
                           // transport evaluates the closed forms on its own grid)
    INFER_METHOD = 2       // the transport's rows, every row the plain table (flag 0): the
                           // table path of the transport with the method's own numbers
};
struct InferArgs {
    const float4* feats;
    int n;                     // rows (with n_dev: the capacity)
    const int* n_dev;          // device row count (null: n rows)
    const unsigned char* img;
    const float* params;
    float* out;                // [n][32]
    const int* err_bits;       // calibrated region errors (null: no fallback)
    float tol;
    int* fallback;             // per sample: 1 where the plain table was used (may be null)
    int mode;                  // INFER_*
    int* err;
};

// Persistent inference, one CTA per SM with the weights resident in shared
// memory and four warpgroups, each running its own stream of 128-row tiles
// with its own X/H buffers, 128 TMEM columns (the three layers reuse them),
// MMA barrier and named barrier: one tile's GEMMs overlap the other tiles'
// epilogues.  Thread t of a warpgroup serves row t (TMEM lane t).
constexpr int kInferThreads = 128 * inf::WG;
__device__ __forceinline__ void wg_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(g + 1) : "memory"); }
// barrier of warpgroup g that returns, to all its threads, whether any passed v
__device__ __forceinline__ bool wg_any(int g, bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.or.pred p, %2, 128, q;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(g + 1)
        : "memory");
    return r != 0;
}

__global__ void __launch_bounds__(kInferThreads, 1) k_infer(InferArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, row = tid & (kTile - 1);
    uint64_t* bar_w = reinterpret_cast<uint64_t*>(sm + inf::BAR);
    uint64_t* bar_m = bar_w + 1 + g;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + inf::BAR + 48);
    int* wfail = reinterpret_cast<int*>(sm + inf::BAR + 64);
    unsigned char* X = sm + inf::TILE0 + g * inf::TILE_BYTES;
    unsigned char* H = X + inf::XB;
    if (tid == 0) {
        bar_init(bar_w, 1);
        for (int k = 0; k < inf::WG; ++k) bar_init(bar_w + 1 + k, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < inf::WG) wfail[tid] = 0;
    if (tid < kTile) {   // the constant-one operand of the bias products: columns 0-1 of [128][16]
        float o[kIn] = {1.0f, 1.0f};
        st_row16(sm + inf::ONES, tid, 0, kIn, o);
    }
    fence_async_smem();
    if (warp == 0) tmem_alloc(tslot, 512);
    __syncthreads();
    if (tid == 0) {
        bar_expect(bar_w, kHid * kIn * 2 + kHid * kHid * 2 + kOut * kHid * 2 + kHid * 16 * 2 + kOut * 16 * 2);
        bulk_g2s(sm + inf::W1, a.img + iW1, kHid * kIn * 2, bar_w);
        bulk_g2s(sm + inf::W2, a.img + iW2, kHid * kHid * 2, bar_w);
        bulk_g2s(sm + inf::W3, a.img + iW3, kOut * kHid * 2, bar_w);
        bulk_g2s(sm + inf::B2X, a.img + iB2X, kHid * 16 * 2, bar_w);
        bulk_g2s(sm + inf::B3X, a.img + iB3X, kOut * 16 * 2, bar_w);
    }
    fence_after();
    const uint32_t tm = *tslot + (uint32_t)(g * 128);
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    uint32_t pm = 0;
    // rows: a count the transport's claim pass left on the device, or n
    const int n = a.n_dev ? min(max(__ldcg(a.n_dev), 0), a.n) : a.n;
    // Per tile and warpgroup: X (features) -> L1 -> H1 -> L2 -> H2 -> L3 -> Z.
    // The softmax and stores of a tile run while the next tile's first GEMM
    // does, and the next tile's features are written to X while the second
    // GEMM runs (X is free once the first has completed).  A wait that runs
    // out of time marks the thread; the barrier before each tile's first
    // GEMM (and one after the loop) sends the warpgroup to the exit.
    const int stride = gridDim.x * inf::WG;
    bool bad = false;
    float4 qn = make_float4(1.0f, 0.0f, 1.0f, 1.0f);   // the next tile's row, loaded ahead
    float f[4];                                        // this tile's inputs
    // features of tile t into X (t's row read ahead in qn; loads t + stride's)
    auto stage_x = [&](int t) {
        const int i = t * kTile + row;
        const float4 q = qn;
        const long long inext = (long long)(t + stride) * kTile + row;
        if (inext < n) qn = __ldcg(a.feats + inext);
        float x[kIn];
        f[0] = 1.0f; f[1] = 0.0f; f[2] = 1.0f; f[3] = 1.0f;
        if (i < n) {
            f[0] = q.x; f[1] = q.y; f[2] = q.z; f[3] = q.w;
            feature_row(f, x);
        } else {
            for (int k = 0; k < kIn; ++k) x[k] = 0.0f;
        }
        x[kBiasCol] = 1.0f;       // picks up b1 (hi, lo) from the W1 image
        x[kBiasCol + 1] = 1.0f;
        st_row16(X, row, 0, kIn, x);
    };
    // softmax of a finished tile's logits z (row i, inputs fz) and its stores
    auto finish = [&](float* z, int i, const float* fz) {
        if (i >= n) return;
        float m = -3.0e38f;
        int am = 0;
#pragma unroll
        for (int k = 0; k < kOut; ++k) {
            if (z[k] > m) { m = z[k]; am = k; }
        }
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < kOut; ++k) { z[k] = __expf(z[k] - m); s += z[k]; }
        const float inv = 1.0f / s;
        float t = 0.0f;
        // weights below the floor are zero (a component's children
        // stay as few as the closed forms give), the rest sum to 1
#pragma unroll
        for (int k = 0; k < kOut; ++k) {
            z[k] *= inv;
            if (z[k] < kFloor) z[k] = 0.0f;
            if (k != am) t += z[k];
        }
#pragma unroll
        for (int k = 0; k < kOut; ++k)
            if (k == am) z[k] = 1.0f - t;   // the row sums to 1: the component's weight is conserved
        int fb = 0;
        if (a.mode == INFER_METHOD) {
            plain_table(fz, z);
        } else if (a.err_bits && __int_as_float(a.err_bits[region_of(fz)]) > a.tol) {
            if (a.mode == INFER_TABLES) plain_table(fz, z);
            fb = 1;
        }
        if (a.fallback) a.fallback[i] = fb;
        if (!(fb && a.mode == INFER_TRANSPORT)) {
            float4* o = reinterpret_cast<float4*>(a.out + (size_t)i * kOut);
#pragma unroll
            for (int q = 0; q < 8; ++q) o[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
        }
    };
    int tile = blockIdx.x * inf::WG + g;
    {
        const int i0 = tile * kTile + row;
        if (i0 < n) qn = __ldcg(a.feats + i0);
    }
    bool ok = bar_wait(bar_w, 0);
    if (wg_any(g, !ok)) goto fail;
    if (tile * kTile < n) stage_x(tile);
    {
        float zp[kOut];   // logits of the tile before, its softmax pending
        float fp[4] = {1.0f, 0.0f, 1.0f, 1.0f};
        int ip = n;       // its row (n: none)
        for (; tile * kTile < n; tile += stride) {
            const int i = tile * kTile + row;
            const float fc[4] = {f[0], f[1], f[2], f[3]};
            fence_async_smem();
            fence_before();
            if (wg_any(g, bad)) goto fail;   // X holds this tile's rows; TMEM is free
            if (row == 0) {
                fence_after();
                mma(tm, sdesc(su32(X), 256), sdesc(su32(sm + inf::W1), 256), idesc(128, 128), 0);
                mma_commit(bar_m);
            }
            finish(zp, ip, fp);
            bad |= !bar_wait(bar_m, pm);
            pm ^= 1;
            fence_after();
            for (int c = 0; c < kHid; c += 32) {
                float v[32];
                tmem_ld32(tm + lane_base + c, v);
                st_row32_relu(H, row, c, kHid, v);
            }
            fence_before();
            fence_async_smem();
            wg_sync(g);
            if (row == 0) {
                fence_after();
                for (int k = 0; k < kHid / 16; ++k)
                    mma(tm, sdesc(su32(H) + 256 * k, 2048), sdesc(su32(sm + inf::W2) + 256 * k, 2048), idesc(128, 128),
                        k > 0);
                mma(tm, sdesc(su32(sm + inf::ONES), 256), sdesc(su32(sm + inf::B2X), 256), idesc(128, 128), 1);   // + b2
                mma_commit(bar_m);
            }
            if ((tile + stride) * kTile < n) stage_x(tile + stride);
            bad |= !bar_wait(bar_m, pm);
            pm ^= 1;
            fence_after();
            for (int c = 0; c < kHid; c += 32) {
                float v[32];
                tmem_ld32(tm + lane_base + c, v);
                st_row32_relu(H, row, c, kHid, v);
            }
            fence_before();
            fence_async_smem();
            wg_sync(g);
            if (row == 0) {
                fence_after();
                for (int k = 0; k < kHid / 16; ++k)
                    mma(tm, sdesc(su32(H) + 256 * k, 2048), sdesc(su32(sm + inf::W3) + 256 * k, 2048), idesc(128, kOut),
                        k > 0);
                mma(tm, sdesc(su32(sm + inf::ONES), 256), sdesc(su32(sm + inf::B3X), 256), idesc(128, kOut), 1);   // + b3
                mma_commit(bar_m);
            }
            bad |= !bar_wait(bar_m, pm);
            pm ^= 1;
            fence_after();
            tmem_ld32(tm + lane_base, zp);
            ip = i;
            fp[0] = fc[0]; fp[1] = fc[1]; fp[2] = fc[2]; fp[3] = fc[3];
        }
        fence_before();
        if (wg_any(g, bad)) goto fail;
        finish(zp, ip, fp);
    }
    goto done;
fail:
    if (row == 0) wfail[g] = 1;
done:
    fence_before();
    __syncthreads();
    if (tid == 0) {
        for (int k = 0; k < inf::WG; ++k)
            if (wfail[k]) atomicExch(a.err, 1);
    }
    if (warp == 0) {
        fence_after();
        tmem_free(*tslot, 512);
    }
}

// Sum of the tiles' partials in tile order (mode 0: gradients out; 1: Adam
// step on the fp32 master and the bf16 images; 2: images only) and the loss.
__global__ void k_update(float* params, float* m1, float* m2, const float* partial, int n_part, float* grad_out,
                         const float* ploss, float* loss_out, int mode, float lr, float bc1, float bc2,
                         unsigned char* img) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && loss_out && mode != 2) {
        float l = 0.0f;
        for (int c = 0; c < n_part; ++c) l += ploss[c];
        *loss_out = l;
    }
    if (p >= kParams) return;
    // W1 columns kPair..2 kPair-1 multiply the inputs' rounding remainders
    // (scaled by 128): they are tied to columns 0..kPair-1 (the image holds
    // bf16(W1[o][i]) / 128 there) and their own parameters stay zero
    const bool tied = p < oW2 && (p % kIn) >= kPair && (p % kIn) < 2 * kPair;
    if (tied) {
        if (mode == 0) grad_out[p] = 0.0f;
        else params[p] = 0.0f;
        return;
    }
    float w = params[p];
    if (mode != 2) {
        float g = 0.0f;
        for (int c = 0; c < n_part; ++c) g += partial[(size_t)c * kParams + p];
        if (p < oW2 && (p % kIn) < kPair) {   // plus the tied column's gradient, d(w / 128) / dw = 1 / 128
            float gt = 0.0f;
            for (int c = 0; c < n_part; ++c) gt += partial[(size_t)c * kParams + p + kPair];
            g += gt * (1.0f / 128.0f);
        }
        if (mode == 0) {
            grad_out[p] = g;
            return;
        }
        const float a = 0.9f * m1[p] + 0.1f * g;
        const float b = 0.999f * m2[p] + 0.001f * g * g;
        m1[p] = a;
        m2[p] = b;
        w -= lr * (a / bc1) / (sqrtf(b / bc2) + 1e-8f);
        params[p] = w;
    }
    __nv_bfloat16* im = reinterpret_cast<__nv_bfloat16*>(img);
    const __nv_bfloat16 h = __float2bfloat16_rn(w);
    if (p < oW2) {
        const int o = p / kIn, k = p % kIn;
        if (k < kPair) {
            im[iW1 / 2 + core_off(o, k, kIn)] = h;
            im[iW1 / 2 + core_off(o, k + kPair, kIn)] = __float2bfloat16_rn(__bfloat162float(h) * (1.0f / 128.0f));
        }
    } else if (p < oW3) {
        const int q = p - oW2, o = q / kHid, k = q % kHid;
        im[iW2 / 2 + core_off(o, k, kHid)] = h;
        im[iW2T / 2 + core_off(k, o, kHid)] = h;
    } else if (p < ob1) {
        const int q = p - oW3, o = q / kHid, k = q % kHid;
        im[iW3 / 2 + core_off(o, k, kHid)] = h;
        im[iW3T / 2 + core_off(k, o, kOut)] = h;
    } else {   // a bias: its (value, remainder) bf16 pair for the inference kernel's bias products
        const __nv_bfloat16 lo = __float2bfloat16_rn(w - __bfloat162float(h));
        if (p < ob2) {
            const int o = p - ob1;
            im[iW1 / 2 + core_off(o, kBiasCol, kIn)] = h;
            im[iW1 / 2 + core_off(o, kBiasCol + 1, kIn)] = lo;
        } else if (p < ob3) {
            const int o = p - ob2;
            im[iB2X / 2 + core_off(o, 0, 16)] = h;
            im[iB2X / 2 + core_off(o, 1, 16)] = lo;
        } else {
            const int o = p - ob3;
            im[iB3X / 2 + core_off(o, 0, 16)] = h;
            im[iB3X / 2 + core_off(o, 1, 16)] = lo;
        }
    }
}

}  // namespace mlp
}  // namespace sm2d

using namespace sm2d;
using namespace sm2d::mlp;

struct sm2d_mlp {
    int max_batch = 0;
    cudaStream_t s = nullptr;
    float *params = nullptr, *m1 = nullptr, *m2 = nullptr, *partial = nullptr, *ploss = nullptr;
    unsigned char* img = nullptr;
    int* err = nullptr;
    int* err_bits = nullptr;   // calibration [kRegions]
    int calibrated = 0;
    cudaEvent_t order = nullptr;   // orders a transport handle's stream before this handle's work
    int t = 0;                 // Adam steps taken
    int sms = 0;
};

namespace {
int mlp_alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(SM2D_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return 0;
}
int check_err(sm2d_mlp* m) {
    int e = 0;
    CK(cudaMemcpyAsync(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->s));
    CK(cudaStreamSynchronize(m->s));
    if (e) {
        // reported once: clear the flag so that later calls start clean
        CK(cudaMemsetAsync(m->err, 0, sizeof(int), m->s));
        CK(cudaStreamSynchronize(m->s));
        return fail(SM2D_ERR_TIMEOUT, "surrogate kernel: a bounded mbarrier wait gave up");
    }
    return 0;
}
int launch_train(sm2d_mlp* m, const float* feats, const float* target, int n, float scale) {
    const int tiles = (n + kTile - 1) / kTile;
    TrainArgs a{reinterpret_cast<const float4*>(feats), reinterpret_cast<const float4*>(target), n, scale, m->img,
                m->params, m->partial, m->ploss, m->err};
    k_train<<<tiles, 128, tr::BYTES, m->s>>>(a);
    CK(cudaGetLastError());
    return 0;
}
int launch_update(sm2d_mlp* m, int n_part, float* grad_out, float* loss_out, int mode, float lr) {
    float bc1 = 1.0f, bc2 = 1.0f;
    if (mode == 1) {
        m->t += 1;
        bc1 = 1.0f - powf(0.9f, (float)m->t);
        bc2 = 1.0f - powf(0.999f, (float)m->t);
    }
    k_update<<<(kParams + 255) / 256, 256, 0, m->s>>>(m->params, m->m1, m->m2, m->partial, n_part, grad_out,
                                                      m->ploss, loss_out, mode, lr, bc1, bc2, m->img);
    CK(cudaGetLastError());
    return 0;
}
bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
}  // namespace

extern "C" {

int sm2d_mlp_param_count(void) { return kParams; }

int sm2d_mlp_create(int max_batch, void* stream, sm2d_mlp_handle* out) {
    if (!out || max_batch <= 0 || max_batch > kMaxRows) return fail(SM2D_ERR_ARG, "sm2d_mlp_create: bad argument");
    *out = nullptr;
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, tr::BYTES));
    CK(cudaFuncSetAttribute(k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, inf::BYTES));
    sm2d_mlp* m = new sm2d_mlp();
    m->max_batch = (max_batch + kTile - 1) / kTile * kTile;
    m->s = (cudaStream_t)stream;
    m->sms = sms;
    const int tiles = m->max_batch / kTile;
    int rc = 0;
    if (!rc) rc = mlp_alloc((void**)&m->params, sizeof(float) * kParams);
    if (!rc) rc = mlp_alloc((void**)&m->m1, sizeof(float) * kParams);
    if (!rc) rc = mlp_alloc((void**)&m->m2, sizeof(float) * kParams);
    if (!rc) rc = mlp_alloc((void**)&m->partial, sizeof(float) * kParams * (size_t)tiles);
    if (!rc) rc = mlp_alloc((void**)&m->ploss, sizeof(float) * tiles);
    if (!rc) rc = mlp_alloc((void**)&m->img, kImgBytes);
    if (!rc) rc = mlp_alloc((void**)&m->err, sizeof(int));
    if (!rc) rc = mlp_alloc((void**)&m->err_bits, sizeof(int) * kRegions);
    if (!rc && cudaEventCreateWithFlags(&m->order, cudaEventDisableTiming) != cudaSuccess)
        rc = fail(SM2D_ERR_CUDA, "cudaEventCreate");
    if (!rc && cudaMemsetAsync(m->err, 0, sizeof(int), m->s) != cudaSuccess) rc = fail(SM2D_ERR_CUDA, "cudaMemsetAsync");
    if (!rc && cudaMemsetAsync(m->err_bits, 0, sizeof(int) * kRegions, m->s) != cudaSuccess)
        rc = fail(SM2D_ERR_CUDA, "cudaMemsetAsync");
    if (rc) {
        sm2d_mlp_destroy(m);
        return rc;
    }
    // initial weights: uniform +-sqrt(6 / fan_in) (He), zero biases, fixed seed
    std::vector<float> p(kParams, 0.0f);
    uint32_t st = 12345u;
    auto u = [&st]() { st = 1664525u * st + 1013904223u; return ((st >> 8) + 0.5f) * (1.0f / 16777216.0f); };
    for (int k = oW1; k < oW2; ++k) p[k] = (2.0f * u() - 1.0f) * sqrtf(6.0f / 8.0f);
    for (int o = 0; o < kHid; ++o)   // the remainder columns are tied to columns 0-3
        for (int k = kPair; k < 2 * kPair; ++k) p[oW1 + o * kIn + k] = 0.0f;
    for (int k = oW2; k < oW3; ++k) p[k] = (2.0f * u() - 1.0f) * sqrtf(6.0f / kHid);
    for (int k = oW3; k < ob1; ++k) p[k] = (2.0f * u() - 1.0f) * sqrtf(1.0f / kHid);
    const int rc2 = sm2d_mlp_set_params(m, p.data());
    if (rc2) {
        sm2d_mlp_destroy(m);
        return rc2;
    }
    *out = m;
    return 0;
}

int sm2d_mlp_destroy(sm2d_mlp_handle m) {
    if (!m) return fail(SM2D_ERR_ARG, "null surrogate handle");
    cudaStreamSynchronize(m->s);
    void* ps[] = {m->params, m->m1, m->m2, m->partial, m->ploss, m->img, m->err, m->err_bits};
    for (void* q : ps)
        if (q) cudaFree(q);
    if (m->order) cudaEventDestroy(m->order);
    delete m;
    return 0;
}

int sm2d_mlp_set_params(sm2d_mlp_handle m, const float* host_params) {
    if (!m || !host_params) return fail(SM2D_ERR_ARG, "null argument");
    CK(cudaMemcpyAsync(m->params, host_params, sizeof(float) * kParams, cudaMemcpyHostToDevice, m->s));
    CK(cudaMemsetAsync(m->m1, 0, sizeof(float) * kParams, m->s));
    CK(cudaMemsetAsync(m->m2, 0, sizeof(float) * kParams, m->s));
    CK(cudaMemsetAsync(m->img, 0, kImgBytes, m->s));
    m->t = 0;
    m->calibrated = 0;
    int rc = launch_update(m, 0, nullptr, nullptr, 2, 0.0f);
    if (rc) return rc;
    CK(cudaStreamSynchronize(m->s));
    return 0;
}

int sm2d_mlp_get_params(sm2d_mlp_handle m, float* host_params) {
    if (!m || !host_params) return fail(SM2D_ERR_ARG, "null argument");
    CK(cudaMemcpyAsync(host_params, m->params, sizeof(float) * kParams, cudaMemcpyDeviceToHost, m->s));
    CK(cudaStreamSynchronize(m->s));
    return 0;
}

int sm2d_mlp_gradients(sm2d_mlp_handle m, const float* d_feats, const float* d_target, int n, float* d_grads,
                       float* d_loss) {
    if (!m || !d_feats || !d_target || !d_grads || !d_loss) return fail(SM2D_ERR_ARG, "null argument");
    if (n <= 0 || n > m->max_batch) return fail(SM2D_ERR_ARG, "batch %d outside 1..%d", n, m->max_batch);
    if (!aligned16(d_feats) || !aligned16(d_target)) return fail(SM2D_ERR_ARG, "inputs must be 16-byte aligned");
    int rc = launch_train(m, d_feats, d_target, n, 1.0f / (float)n);
    if (!rc) rc = launch_update(m, (n + kTile - 1) / kTile, d_grads, d_loss, 0, 0.0f);
    return rc;
}

int sm2d_mlp_train(sm2d_mlp_handle m, const float* d_feats, const float* d_target, int n_total, int batch, int steps,
                   float lr0, float lr_min, float* d_loss_hist) {
    if (!m || !d_feats || !d_target) return fail(SM2D_ERR_ARG, "null argument");
    if (batch <= 0 || batch > m->max_batch || batch % kTile) return fail(SM2D_ERR_ARG, "batch %d: a multiple of %d up to %d", batch, kTile, m->max_batch);
    if (n_total < batch || n_total > kMaxRows || steps < 0) return fail(SM2D_ERR_ARG, "training set of %d rows", n_total);
    if (!aligned16(d_feats) || !aligned16(d_target)) return fail(SM2D_ERR_ARG, "inputs must be 16-byte aligned");
    const int per_epoch = n_total / batch;
    for (int s = 0; s < steps; ++s) {
        const size_t off = (size_t)(s % per_epoch) * batch;
        const float lr = lr_min + 0.5f * (lr0 - lr_min) * (1.0f + cosf(3.14159265f * (float)s / (float)steps));
        int rc = launch_train(m, d_feats + off * 4, d_target + off * kOut, batch, 1.0f / (float)batch);
        if (!rc) rc = launch_update(m, batch / kTile, nullptr, d_loss_hist ? d_loss_hist + s : nullptr, 1, lr);
        if (rc) return rc;
    }
    m->calibrated = 0;
    return 0;
}

int sm2d_mlp_forward(sm2d_mlp_handle m, const float* d_feats, int n, float* d_table) {
    if (!m || !d_feats || !d_table) return fail(SM2D_ERR_ARG, "null argument");
    if (n <= 0 || n > kMaxRows) return fail(SM2D_ERR_ARG, "rows %d outside 1..%d", n, kMaxRows);
    if (!aligned16(d_feats) || !aligned16(d_table)) return fail(SM2D_ERR_ARG, "arrays must be 16-byte aligned");
    InferArgs a{};
    a.feats = reinterpret_cast<const float4*>(d_feats);
    a.n = n;
    a.img = m->img;
    a.params = m->params;
    a.out = d_table;
    a.err = m->err;
    const int tiles = (n + kTile - 1) / kTile;
    k_infer<<<std::min((tiles + inf::WG - 1) / inf::WG, m->sms), kInferThreads, inf::BYTES, m->s>>>(a);
    CK(cudaGetLastError());
    return 0;
}

int sm2d_redistribution_features(int n, uint32_t seed, float* d_feats, void* stream) {
    if (n <= 0 || n > kMaxRows || !d_feats || !aligned16(d_feats)) return fail(SM2D_ERR_ARG, "bad argument");
    k_features<<<std::min((n + 255) / 256, 4096), 256, 0, (cudaStream_t)stream>>>(n, seed, reinterpret_cast<float4*>(d_feats));
    CK(cudaGetLastError());
    return 0;
}

int sm2d_redistribution_table(sm2d_handle h, const float* d_feats, int n, float* d_table) {
    if (!d_feats || !d_table || n <= 0 || n > kMaxRows) return fail(SM2D_ERR_ARG, "bad argument");
    if (!aligned16(d_feats) || !aligned16(d_table)) return fail(SM2D_ERR_ARG, "arrays must be 16-byte aligned");
    Dev d;
    cudaStream_t s;
    int rc = handle_dev(h, &d, &s);
    if (rc) return rc;
    (void)d;
    k_plain<<<std::min((n + 255) / 256, 8192), 256, 0, s>>>(n, reinterpret_cast<const float4*>(d_feats),
                                                           reinterpret_cast<float4*>(d_table));
    CK(cudaGetLastError());
    return 0;
}

int sm2d_mlp_calibrate(sm2d_mlp_handle m, const float* d_feats, const float* d_plain, const float* d_surrogate, int n,
                       float* host_region_err) {
    if (!m || !d_feats || !d_plain || !d_surrogate || n <= 0 || n > kMaxRows) return fail(SM2D_ERR_ARG, "bad argument");
    CK(cudaMemsetAsync(m->err_bits, 0, sizeof(int) * kRegions, m->s));
    k_calibrate<<<std::min((n + 255) / 256, 8192), 256, 0, m->s>>>(n, reinterpret_cast<const float4*>(d_feats), d_plain,
                                                                  d_surrogate, m->err_bits);
    CK(cudaGetLastError());
    if (host_region_err)
        CK(cudaMemcpyAsync(host_region_err, m->err_bits, sizeof(int) * kRegions, cudaMemcpyDeviceToHost, m->s));
    CK(cudaStreamSynchronize(m->s));
    m->calibrated = 1;
    return 0;
}

int sm2d_mlp_redistribute(sm2d_mlp_handle m, sm2d_handle h, const float* d_feats, int n, float tol, float* d_table,
                          int* d_fallback) {
    if (!m || !d_feats || !d_table) return fail(SM2D_ERR_ARG, "null argument");
    if (n <= 0 || n > kMaxRows) return fail(SM2D_ERR_ARG, "rows %d outside 1..%d", n, kMaxRows);
    if (!m->calibrated) return fail(SM2D_ERR_STATE, "sm2d_mlp_redistribute before sm2d_mlp_calibrate");
    if (!aligned16(d_feats) || !aligned16(d_table)) return fail(SM2D_ERR_ARG, "arrays must be 16-byte aligned");
    InferArgs a{};
    Dev dev;
    cudaStream_t s;
    int rc = handle_dev(h, &dev, &s);
    if (rc) return rc;
    a.feats = reinterpret_cast<const float4*>(d_feats);
    a.n = n;
    a.img = m->img;
    a.params = m->params;
    a.out = d_table;
    a.err_bits = m->err_bits;
    a.tol = tol;
    a.fallback = d_fallback;
    a.err = m->err;
    // the fallback rows read h's device tables: order h's stream first
    if (s != m->s) {
        CK(cudaEventRecord(m->order, s));
        CK(cudaStreamWaitEvent(m->s, m->order, 0));
    }
    const int tiles = (n + kTile - 1) / kTile;
    k_infer<<<std::min((tiles + inf::WG - 1) / inf::WG, m->sms), kInferThreads, inf::BYTES, m->s>>>(a);
    CK(cudaGetLastError());
    return 0;
}

int sm2d_mlp_sync(sm2d_mlp_handle m) {
    if (!m) return fail(SM2D_ERR_ARG, "null surrogate handle");
    return check_err(m);
}

int sm2d_mlp_geometry(float* out8) {
    if (!out8) return fail(SM2D_ERR_ARG, "null argument");
    const float g[8] = {kSMax, 1.0f, kRMax, 1.0f, (float)kRegS, (float)kRegU, (float)kRegR, (float)kRegC};
    memcpy(out8, g, sizeof g);
    return 0;
}

}  // extern "C"

namespace sm2d {
// The network over the transport's surrogate rows, enqueued on the
// transport's stream (the engine captures it into its device loop): rows
// 0 .. min(*n_dev, cap) of feats, their tables into table [cap][32] and
// fallback flags into fb [cap].  method_tables: every row gets the plain
// table instead (the table path with the method's own numbers).  A bounded
// wait that gives up sets the surrogate handle's error flag (sm2d_mlp_sync).
int mlp_transport_rows(sm2d_mlp_handle m, cudaStream_t s, const float4* feats, const int* n_dev, int cap, float tol,
                       int method_tables, float* table, int* fb) {
    InferArgs a{};
    a.feats = feats;
    a.n = cap;
    a.n_dev = n_dev;
    a.img = m->img;
    a.params = m->params;
    a.out = table;
    a.err_bits = m->err_bits;
    a.tol = tol;
    a.fallback = fb;
    a.mode = method_tables ? INFER_METHOD : INFER_TRANSPORT;
    a.err = m->err;
    const int tiles = (cap + kTile - 1) / kTile;
    k_infer<<<std::max(1, std::min((tiles + inf::WG - 1) / inf::WG, m->sms)), kInferThreads, inf::BYTES, s>>>(a);
    CK(cudaGetLastError());
    return 0;
}
int mlp_calibrated(sm2d_mlp_handle m) { return m && m->calibrated; }
}  // namespace sm2d
