// The depth view of renderer.cpp:93 (`depth_buffer.normalize(0,255)` before it is saved): the
// smallest and largest depth over the buffer, then every value mapped linearly onto 0..255 and
// stored as a byte.
//
// CImg's normalize(a, b) computes (v - m) / (M - m) * (b - a) + a in float for each value, after
// taking m and M with `<` and `>` (NaN never replaces them), and fills with a when m == M; the byte
// is the C conversion of that float (truncation). Depth buffers of this library hold no NaN.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "rast_internal.h"

namespace rast {
namespace {

// Order-preserving key of a float (-0 and +0 alike).
__device__ __forceinline__ uint32_t order_key(float v) {
    uint32_t u = __float_as_uint(v);
    u = u == 0x80000000u ? 0u : u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_value(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__global__ void __launch_bounds__(256) k_depth_minmax(const float* __restrict__ depth, int64_t n,
                                                      uint32_t* __restrict__ mm) {
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = depth[i];
        if (v != v) continue;
        const uint32_t k = order_key(v);
        lo = min(lo, k);
        hi = max(hi, k);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm, lo);
        atomicMax(mm + 1, hi);
    }
}

__global__ void __launch_bounds__(256) k_depth_quantize(const float* __restrict__ depth, int64_t n,
                                                        const uint32_t* __restrict__ mm, uint8_t* __restrict__ out) {
    const uint32_t klo = mm[0], khi = mm[1];
    const float m = klo == 0xFFFFFFFFu ? 0.f : key_value(klo), M = khi == 0u ? 0.f : key_value(khi);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        if (m != M) v = __fadd_rn(__fmul_rn(__fdiv_rn(__fsub_rn(depth[i], m), __fsub_rn(M, m)), 255.f), 0.f);
        out[i] = (uint8_t)__float2uint_rz(v);
    }
}

}  // namespace

int launch_depth_view(const float* depth, int64_t n, uint32_t* mm, uint8_t* out, int n_sm, cudaStream_t stream) {
    if (cudaMemsetAsync(mm, 0xFF, sizeof(uint32_t), stream) != cudaSuccess ||
        cudaMemsetAsync(mm + 1, 0, sizeof(uint32_t), stream) != cudaSuccess)
        return -1;
    const int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)8 * n_sm);
    k_depth_minmax<<<grid > 0 ? grid : 1, 256, 0, stream>>>(depth, n, mm);
    k_depth_quantize<<<grid > 0 ? grid : 1, 256, 0, stream>>>(depth, n, mm, out);
    return cudaGetLastError() == cudaSuccess ? 2 : -1;
}

}  // namespace rast
