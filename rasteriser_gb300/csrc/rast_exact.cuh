// Exact single-rounding float helpers and the per-light Lambert shader, shared by the raster
// kernels (rast_kernels.cu) and the deferred shading kernels (rast_shade.cu).
//
// Every helper is one IEEE round-to-nearest operation written with an __f*_rn intrinsic, which the
// compiler never contracts into an FMA, so the results do not depend on -fmad.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rast {
namespace {

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dvd(float a, float b) { return __fdiv_rn(a, b); }
// glm::min / glm::max on scalars: x < y ? x : y and x > y ? x : y (NaN and -0 follow from this).
__device__ __forceinline__ float gmin(float x, float y) { return x < y ? x : y; }
__device__ __forceinline__ float gmax(float x, float y) { return x > y ? x : y; }

// RN(a / b) from y = RN(1/b), the correctly rounded reciprocal: q0 = RN(a*y), then one fused
// correction q = RN(q0 + RN(a - b*q0)*y) (Markstein's correction step). Checked bit for bit
// against __fdiv_rn on every pair of significands (2^46 pairs, a and b in [1, 2)); scaling a and
// b by powers of two scales every step exactly while all values stay normal, which holds for
// |a| and |b| in [2^-60, 2^60], and every step is symmetric in the signs. Outside that range, for
// zeros, and when y is 0 (b outside it), the quotient is __fdiv_rn's. Several divisions by one b
// share y = div_by_recip(b).
__device__ __forceinline__ float div_by_recip(float b) {
    const float ab = fabsf(b);
    return ab >= 0x1p-60f && ab <= 0x1p60f ? __frcp_rn(b) : 0.f;
}

__device__ __forceinline__ float div_by(float a, float b, float y) {
    const float aa = fabsf(a);
    if (y != 0.f && aa >= 0x1p-60f && aa <= 0x1p60f) {
        const float q0 = __fmul_rn(a, y);
        return __fmaf_rn(__fmaf_rn(-b, q0, a), y, q0);
    }
    return dvd(a, b);
}

// 1/pi as the reference's glm::one_over_pi<float>() rounds it.
constexpr float kOneOverPi = 0.318309886183790671537767526745028724f;

// The float radiance of shading.cpp:20-34 before clamping: for each light in order,
// c = intensity * colour, c *= albedo, c *= max(0, dot(normal, -trans_dir)) * (1/pi) summed
// left to right as (c * m) * (1/pi), accumulated in light order. Lights are 7 floats:
// trans_dir xyz, intensity, colour rgb.
__device__ __forceinline__ float3 light_sum(const float* lights, int nl, float3 n, float3 alb) {
    float accr = 0.f, accg = 0.f, accb = 0.f;
    for (int l = 0; l < nl; ++l) {
        const float* L = lights + 7 * l;
        const float I = __ldg(L + 3);
        float cr = mul(I, __ldg(L + 4)), cg = mul(I, __ldg(L + 5)), cb = mul(I, __ldg(L + 6));
        cr = mul(cr, alb.x); cg = mul(cg, alb.y); cb = mul(cb, alb.z);
        const float d = add(add(mul(n.x, -__ldg(L)), mul(n.y, -__ldg(L + 1))), mul(n.z, -__ldg(L + 2)));
        const float m = gmax(0.f, d);
        cr = mul(mul(cr, m), kOneOverPi);
        cg = mul(mul(cg, m), kOneOverPi);
        cb = mul(mul(cb, m), kOneOverPi);
        accr = add(accr, cr); accg = add(accg, cg); accb = add(accb, cb);
    }
    return make_float3(accr, accg, accb);
}

// The frame's byte per channel: min(value, 255) truncated (CImg's unsigned char store of the
// clamped float, shading.cpp:34).
__device__ __forceinline__ uint32_t pack_rgb(float3 acc) {
    const uint32_t r = __float2uint_rz(gmin(acc.x, 255.f)) & 0xFFu;
    const uint32_t g = __float2uint_rz(gmin(acc.y, 255.f)) & 0xFFu;
    const uint32_t b = __float2uint_rz(gmin(acc.z, 255.f)) & 0xFFu;
    return r | (g << 8) | (b << 16);
}

// The shaded colour r | g << 8 | b << 16.
__device__ __forceinline__ uint32_t shade_lights(const float* lights, int nl, float3 n, float3 alb) {
    return pack_rgb(light_sum(lights, nl, n, alb));
}

}  // namespace
}  // namespace rast
