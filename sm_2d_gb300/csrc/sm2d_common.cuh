// sm2d_common.cuh -- error reporting, launch constants and warp reductions
// shared by the engine and the stage entries.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "sm2d.h"
#include "sm2d_device.cuh"

namespace sm2d {

// Records a formatted message for sm2d_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return ::sm2d::fail(SM2D_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                __FILE__, __LINE__);                                    \
    } while (0)

constexpr int kThreads = 256;

// The learned surrogate's network over a transport's surrogate rows
// (sm2d_surrogate.cu), enqueued on stream s.
int mlp_transport_rows(sm2d_mlp_handle m, cudaStream_t s, const float4* feats, const int* n_dev, int cap, float tol,
                       int method_tables, float* table, int* fb);
int mlp_calibrated(sm2d_mlp_handle m);

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

}  // namespace sm2d
