// Check of rast::div_by / rast::div_by_recip (rast_exact.cuh, the setup pass's shared-reciprocal
// division) against __fdiv_rn, calling the functions the kernels call:
//   y = div_by_recip(b); q = div_by(a, b, y)    must equal    __fdiv_rn(a, b)    bit for bit.
//
// Three parts, all in one run:
//  - significand pairs (a, b in [1, 2)): every b significand with every a_stride-th a
//    significand; a_stride 1 is all 2^46 pairs, about 40 s on a GB300. Scaling a and b by powers
//    of two scales every step exactly while all values stay normal, so one binade stands for every
//    exponent pair inside the guarded range;
//  - edges: every pair of 64 special values (+-2^-60 and +-2^60 and their neighbours on both sides,
//    +-0, +-inf, NaN, subnormals, the largest and smallest normals, +-1, +-3), so the range guard
//    and the __fdiv_rn fallback run too (NaN results compare equal when both are NaN);
//  - random pairs: 2^24 pairs with random significands, signs and exponents in [-70, 70], across
//    the guard's boundaries.
//
// Usage: div_by_check [a_stride]. Prints one JSON line; exits 1 on a CUDA error, 2 on a mismatch.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>

#include "rast_exact.cuh"

__device__ __forceinline__ bool same(float q, float ref) {
    return __float_as_uint(q) == __float_as_uint(ref) || (q != q && ref != ref);
}

__device__ void record(float a, float b, float q, float ref, unsigned long long* bad, uint32_t* ex) {
    if (atomicCAS(ex, 0u, 1u) == 0u) {
        ex[1] = __float_as_uint(a);
        ex[2] = __float_as_uint(b);
        ex[3] = __float_as_uint(q);
        ex[4] = __float_as_uint(ref);
    }
    atomicAdd(bad, 1ull);
}

__global__ void k_significands(uint32_t a0, uint32_t n_a, uint32_t a_stride, unsigned long long* bad, uint32_t* ex) {
    const uint32_t mb = blockIdx.x * blockDim.x + threadIdx.x;
    if (mb >= (1u << 23)) return;
    const float b = __uint_as_float(0x3F800000u | mb);
    const float y = rast::div_by_recip(b);
    for (uint32_t k = 0; k < n_a; ++k) {
        const float a = __uint_as_float(0x3F800000u | (a0 + k * a_stride));
        const float q = rast::div_by(a, b, y);
        const float ref = __fdiv_rn(a, b);
        if (!same(q, ref)) record(a, b, q, ref, bad, ex);
    }
}

constexpr int kEdges = 64;

__global__ void k_edges(const float* vals, unsigned long long* bad, uint32_t* ex) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kEdges * kEdges) return;
    const float a = vals[i / kEdges], b = vals[i % kEdges];
    const float q = rast::div_by(a, b, rast::div_by_recip(b));
    const float ref = __fdiv_rn(a, b);
    if (!same(q, ref)) record(a, b, q, ref, bad, ex);
}

__device__ __forceinline__ uint32_t mix(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float random_float(uint32_t h, uint32_t h2) {
    const uint32_t e = 127u - 70u + h2 % 141u;  // exponents -70 .. 70
    return __uint_as_float((h & 0x807FFFFFu) | (e << 23));
}

__global__ void k_random(uint32_t n, unsigned long long* bad, uint32_t* ex) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = random_float(mix(4 * i), mix(4 * i + 1)), b = random_float(mix(4 * i + 2), mix(4 * i + 3));
    const float q = rast::div_by(a, b, rast::div_by_recip(b));
    const float ref = __fdiv_rn(a, b);
    if (!same(q, ref)) record(a, b, q, ref, bad, ex);
}

static void edge_values(float* v) {
    int n = 0;
    auto bits = [](uint32_t u) { float f; memcpy(&f, &u, 4); return f; };
    const uint32_t u_lo = 0x21800000u, u_hi = 0x5D800000u;  // 2^-60, 2^60
    for (uint32_t u : {u_lo - 1, u_lo, u_lo + 1, u_hi - 1, u_hi, u_hi + 1, 0x00000000u, 0x00000001u, 0x00400000u,
                       0x007FFFFFu, 0x00800000u, 0x7F7FFFFFu, 0x7F800000u, 0x7FC00000u, 0x3F800000u, 0x40400000u,
                       0x3F7FFFFFu, 0x3FFFFFFFu, 0x2A000000u, 0x55000000u, 0x1F800000u, 0x5F800000u, 0x34000000u,
                       0x4B000000u, 0x3EAAAAABu, 0x40490FDBu, 0x219FFFFFu, 0x5D7FFFFFu, 0x21C00000u, 0x5DC00000u,
                       0x01000000u, 0x7E800000u}) {
        v[n++] = bits(u);
        v[n++] = bits(u | 0x80000000u);
    }
}

int main(int argc, char** argv) {
    const uint32_t a_stride = argc > 1 ? (uint32_t)atoi(argv[1]) : 1u;
    if (a_stride == 0 || ((1u << 23) % a_stride) != 0) return 1;
    unsigned long long* bad;
    uint32_t* ex;
    float* d_vals;
    float h_vals[kEdges];
    edge_values(h_vals);
    cudaMalloc(&bad, 3 * sizeof(unsigned long long));
    cudaMalloc(&ex, 8 * sizeof(uint32_t));
    cudaMalloc(&d_vals, sizeof h_vals);
    cudaMemcpy(d_vals, h_vals, sizeof h_vals, cudaMemcpyHostToDevice);
    cudaMemset(bad, 0, 3 * sizeof(unsigned long long));
    cudaMemset(ex, 0, 8 * sizeof(uint32_t));
    const uint32_t n_a = 8192 / a_stride > 0 ? 8192 / a_stride : 1;  // a values per launch
    const uint32_t n_random = 1u << 24;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    for (uint32_t a0 = 0; a0 < (1u << 23); a0 += n_a * a_stride)
        k_significands<<<(1u << 23) / 256, 256>>>(a0, n_a, a_stride, bad, ex);
    k_edges<<<(kEdges * kEdges + 255) / 256, 256>>>(d_vals, bad + 1, ex);
    k_random<<<n_random / 256, 256>>>(n_random, bad + 2, ex);
    cudaEventRecord(e1);
    cudaError_t err = cudaDeviceSynchronize();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    unsigned long long hb[3] = {0, 0, 0};
    uint32_t hex[8] = {0};
    cudaMemcpy(hb, bad, sizeof hb, cudaMemcpyDeviceToHost);
    cudaMemcpy(hex, ex, sizeof hex, cudaMemcpyDeviceToHost);
    printf("{\"status\": \"%s\", \"pairs\": %llu, \"mismatches\": %llu, \"edge_pairs\": %d, \"edge_mismatches\": %llu, "
           "\"random_pairs\": %u, \"random_mismatches\": %llu, \"seconds\": %.2f, \"example\": [%u, %u, %u, %u]}\n",
           cudaGetErrorString(err), ((unsigned long long)1 << 46) / a_stride, hb[0], kEdges * kEdges, hb[1], n_random,
           hb[2], ms / 1000.f, hex[1], hex[2], hex[3], hex[4]);
    return err != cudaSuccess ? 1 : (hb[0] + hb[1] + hb[2] ? 2 : 0);
}
