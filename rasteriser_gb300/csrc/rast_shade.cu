// Deferred shading for sm_103a: the exact per-light shader and the learned many-light shader
// over the resolve pass's fragment records, and the kernels that train the learned shader.
//
//   k_shade_exact  shading.cpp:20-34 per fragment, lights staged in shared memory: the plain
//                  shader, bit for bit the reference's colour
//   k_shade_mlp    per tile of 128 records: Fourier features -> three tcgen05 BF16 MMAs with FP32
//                  accumulators in tensor memory -> radiance; a few records of every tile are also
//                  shaded exactly, and a tile whose checked error exceeds the bound is shaded
//                  exactly in full
//   k_shade_scan   the tile list for records staged by k_mlp_stage (draws list their tiles in the
//                  resolve pass)
//   k_mlp_samples / k_mlp_train / k_mlp_adam   training on (normal, albedo) samples labelled by
//                  the exact shader's float radiance
//
// The exact arithmetic lives in rast_exact.cuh (single-rounding intrinsics only), so the file's
// -fmad=false changes nothing there; the learned path uses explicit FMAs where it wants them.
#include <algorithm>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "rast_exact.cuh"
#include "rast_internal.h"
#include "rast_mlp.h"
#include "rast_tiles.cuh"

namespace rast {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

struct ShadeArgs {
    const float4* gbuf;
    const uint32_t* index;   // the tile list (rast_tiles.cuh)
    uint32_t n_blocks;       // 1024-pixel blocks the list covers
    int64_t npx;
    const float* lights;
    int32_t nl;
    uint8_t* rgb;
    uint32_t* counters;
    // learned shader
    const MlpImage* mlp;
    int32_t samples;
    float bound;
    unsigned long long* stats;
    float* eval_out;  // evaluation mode: radiance floats per record (pixel field = record index)
    uint32_t stall_test;  // test only: the first MMA wait polls an mbarrier nothing arrives on
};


__device__ __forceinline__ void write_rgb(uint8_t* rgb, int64_t npx, uint32_t p, uint32_t col) {
    rgb[p] = (uint8_t)(col & 0xFFu);
    rgb[npx + p] = (uint8_t)((col >> 8) & 0xFFu);
    rgb[2 * npx + p] = (uint8_t)((col >> 16) & 0xFFu);
}

__global__ void __launch_bounds__(1024) k_shade_scan(const uint32_t* __restrict__ bcount, uint32_t n_blocks,
                                                     uint32_t* __restrict__ index) {
    build_shade_tiles(bcount, n_blocks, index);
}

// ---------------------------------------------------------------------------------------------
// exact deferred shading
// ---------------------------------------------------------------------------------------------
constexpr int kLightChunk = 512;
constexpr int kExactThreads = 128;
constexpr int kExactCtasPerSm = 8;

// Stages lights [l0, l0 + n) as (-dir xyz, I*r), (I*g, I*b, 0, 0): the negation is exact and the
// products are the ones shading.cpp forms per light, so the per-fragment sum is unchanged.
__device__ __forceinline__ void stage_lights(const float* lights, int l0, int n, float4* sl) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float* L = lights + 7 * (int64_t)(l0 + i);
        const float I = __ldg(L + 3);
        sl[2 * i] = make_float4(-__ldg(L), -__ldg(L + 1), -__ldg(L + 2), mul(I, __ldg(L + 4)));
        sl[2 * i + 1] = make_float4(mul(I, __ldg(L + 5)), mul(I, __ldg(L + 6)), 0.f, 0.f);
    }
}

// One staged light's term of shading.cpp:24-31 for normal nv and albedo alb.
__device__ __forceinline__ float3 light_term(const float4* sl, int l, float3 nv, float3 alb) {
    const float4 A = sl[2 * l], B = sl[2 * l + 1];
    float cr = mul(A.w, alb.x), cg = mul(B.x, alb.y), cb = mul(B.y, alb.z);
    const float d = add(add(mul(nv.x, A.x), mul(nv.y, A.y)), mul(nv.z, A.z));
    const float m = gmax(0.f, d);
    cr = mul(mul(cr, m), kOneOverPi);
    cg = mul(mul(cg, m), kOneOverPi);
    cb = mul(mul(cb, m), kOneOverPi);
    return make_float3(cr, cg, cb);
}

__device__ __forceinline__ void accumulate_lights(const float4* sl, int n, float3 nv, float3 alb, float3& acc) {
#pragma unroll 4
    for (int l = 0; l < n; ++l) {
        const float3 c = light_term(sl, l, nv, alb);
        acc.x = add(acc.x, c.x);
        acc.y = add(acc.y, c.y);
        acc.z = add(acc.z, c.z);
    }
}

__global__ void __launch_bounds__(kExactThreads, kExactCtasPerSm) k_shade_exact(ShadeArgs a) {
    __shared__ float4 sl[2 * kLightChunk];
    const uint32_t r = threadIdx.x;
    const bool one_chunk = a.nl <= kLightChunk;
    if (one_chunk) stage_lights(a.lights, 0, a.nl, sl);
    // the records and the tile list are the previous kernel's output
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t n_tiles = a.index[1];
    __syncthreads();
    for (uint32_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const bool valid = r < shade_tile_count(a.index, t);
        const size_t slot =
            valid ? shade_record_slot(a.index, a.n_blocks, shade_tile_desc(a.index, a.n_blocks, t), t, r) : 0;
        float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f), g1 = g0;
        if (valid) {
            g0 = a.gbuf[2 * slot];
            g1 = a.gbuf[2 * slot + 1];
        }
        const float3 nv = make_float3(g0.x, g0.y, g0.z), alb = make_float3(g0.w, g1.x, g1.y);
        float3 acc = make_float3(0.f, 0.f, 0.f);
        for (int c0 = 0; c0 < a.nl; c0 += kLightChunk) {
            const int cn = min(kLightChunk, a.nl - c0);
            if (!one_chunk) {
                __syncthreads();
                stage_lights(a.lights, c0, cn, sl);
                __syncthreads();
            }
            if (valid) accumulate_lights(sl, cn, nv, alb, acc);
        }
        if (valid) {
            const uint32_t p = __float_as_uint(g1.z);
            if (a.eval_out) {
                a.eval_out[3 * (size_t)p] = acc.x;
                a.eval_out[3 * (size_t)p + 1] = acc.y;
                a.eval_out[3 * (size_t)p + 2] = acc.z;
            } else {
                write_rgb(a.rgb, a.npx, p, pack_rgb(acc));
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// learned shader: features
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// relu of both values, rounded to BF16 and packed (lo in the low half).
__device__ __forceinline__ uint32_t relu_bf16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

__device__ __forceinline__ float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

constexpr float kPi = 3.14159265358979323846f;

// sin and cos of f*pi*v for f = 1..kMlpFreq come from the base pair (the hardware sine and cosine of
// pi*v, |pi*v| <= pi) by the three-term recurrence x_{f+1} = 2 cos(pi v) x_f - x_{f-1}, which both
// sequences satisfy; one packed FMA advances the pair. Its error stays far below BF16's step.
// emit(f, pair) receives the BF16 pair (sin, cos) of frequency f + 1 (sin in the low half).
template <class Emit>
__device__ __forceinline__ void fourier_pairs(float v, Emit&& emit) {
    float s1, c1;
    __sincosf(kPi * v, &s1, &c1);
    const float2 k2 = make_float2(2.f * c1, 2.f * c1);
    float2 prev = make_float2(0.f, 1.f);
    float2 cur = make_float2(s1, c1);
#pragma unroll
    for (int f = 0; f < kMlpFreq; ++f) {
        emit(f, pack_bf16x2(cur.x, cur.y));
        const float2 next = __ffma2_rn(k2, cur, make_float2(-prev.x, -prev.y));
        prev = cur;
        cur = next;
    }
}

// The last 8 pairs of the features: n, albedo, the constant 1 that carries layer 1's bias
// (feature kMlpConst), zeros.
__device__ __forceinline__ void tail_pairs(float3 n, float3 alb, uint32_t (&t)[8]) {
    t[0] = pack_bf16x2(n.x, n.y);
    t[1] = pack_bf16x2(n.z, alb.x);
    t[2] = pack_bf16x2(alb.y, alb.z);
    t[3] = pack_bf16x2(1.f, 0.f);
    t[4] = t[5] = t[6] = t[7] = 0u;
}

// The kMlpIn input features, each rounded to BF16, as packed pairs (feature 2i in the low half).
static_assert(kMlpIn / 2 == 3 * kMlpFreq + 8 && kMlpConst == 6 * kMlpFreq + 6, "feature layout");
__device__ __forceinline__ void mlp_feature_pairs(float3 n, float3 alb, uint32_t (&pairs)[kMlpIn / 2]) {
    const float comp[3] = {n.x, n.y, n.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) fourier_pairs(comp[c], [&](int f, uint32_t p) { pairs[c * kMlpFreq + f] = p; });
    uint32_t t[8];
    tail_pairs(n, alb, t);
#pragma unroll
    for (int i = 0; i < 8; ++i) pairs[3 * kMlpFreq + i] = t[i];
}

// ---------------------------------------------------------------------------------------------
// learned shader: tcgen05 helpers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading (K-direction) and stride
// (row-direction) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t mma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// tcgen05.mma kind::f16 with the A operand in tensor memory (row m of A in lane m, K packed two
// BF16 per column) and B in shared memory.
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Waits for the phase with the given parity to complete; false after `tries` polls.
constexpr uint32_t kWaitTries = 1u << 22;
constexpr uint32_t kStallTestTries = 1024;  // RAST_OPT_TEST_SHADE_STALL: polls of the idle mbarrier
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t tries = kWaitTries) {
    for (uint32_t i = 0; i < tries; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// Bulk copy global -> shared (addresses 16-byte aligned, size a multiple of 16), completing on mbar.
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}

// 8 consecutive 32-bit columns of this thread's TMEM lane from registers.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(v[0]),
                 "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&v)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(taddr)
                 : "memory");
}

// tcgen05.wait::ld, with the loaded registers threaded through so no use moves above the wait.
__device__ __forceinline__ void tmem_wait16(uint32_t (&v)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15])::"memory");
}
__device__ __forceinline__ void tmem_wait4(uint32_t (&v)[4]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3])::"memory");
}
__device__ __forceinline__ void reg_fence16(uint32_t (&v)[16]) {
    asm volatile(""
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15])::"memory");
}

// ---------------------------------------------------------------------------------------------
// learned shader: the kernel
// ---------------------------------------------------------------------------------------------
// One CTA per SM with kSlots independent tile slots. A slot is four warps, one thread per row of a
// 128-record tile; it walks its tiles through the three layers on its own (named barriers), so
// while one slot waits for its MMAs the others compute features and epilogues. The slots share
// the weights (B operands, one copy in shared memory) and the light table of the checks. A slot's
// FP32 accumulators are 64 columns of tensor memory; its A operand (features, then h1, then h2) is
// either 32 further columns of tensor memory (kATmem) or a [128][K] BF16 matrix in shared memory.
//
// The layout can be changed at build time (RAST_MLP_SLOTS, RAST_MLP_LD, RAST_MLP_A_TMEM) to
// measure the alternatives; the defaults are the fastest measured.
#ifndef RAST_MLP_SLOTS
#define RAST_MLP_SLOTS 5
#endif
#ifndef RAST_MLP_LD
#define RAST_MLP_LD 4
#endif
#ifndef RAST_MLP_A_TMEM
#define RAST_MLP_A_TMEM 1
#endif
constexpr int kSlots = RAST_MLP_SLOTS;
constexpr int kLdBatch = RAST_MLP_LD;  // 16-column accumulator loads in flight per wait (1, 2 or 4)
constexpr bool kATmem = RAST_MLP_A_TMEM != 0;
constexpr int kSlotThreads = 128;  // warp w of a slot reads TMEM lanes 32w..32w+31 (w = warp id mod 4)
constexpr int kMlpThreads = kSlots * kSlotThreads;
constexpr uint32_t kSlotCols = 64;                       // a slot's accumulators
constexpr uint32_t kACols = kMlpIn / 2;                  // a slot's A operand in tensor memory
constexpr uint32_t kTmemCols = 512;
static_assert(kMlpIn == kMlpHid, "one A operand per slot serves every layer");
static_assert(kSlots * kSlotCols + (kATmem ? kSlots * kACols : 0u) <= kTmemCols, "tensor memory of one SM");
static_assert(kLdBatch == 1 || kLdBatch == 2 || kLdBatch == 4, "accumulator loads per wait");
constexpr uint32_t kABytes = kATmem ? 0u : kMlpRows * kMlpIn * 2;  // a slot's A operand in shared memory
constexpr uint32_t kALbo = kMlpRows * 16;                            // its K-direction core-matrix step
constexpr uint32_t kMaxSamples = 4;
constexpr int kMlpSmemLights = 512;  // lights staged in shared memory (24 bytes each) for the checks

// Shared memory (bytes): the weights and output scale, the slots' A operands, the light table,
// then the small block.
constexpr uint32_t kSmW1 = 0;
constexpr uint32_t kSmW2 = kSmW1 + kMlpHid * kMlpIn * 2;
constexpr uint32_t kSmW3 = kSmW2 + kMlpHid * kMlpHid * 2;
constexpr uint32_t kSmA = (sizeof(MlpImage) + 1023) / 1024 * 1024;
constexpr uint32_t kSmLights = kSmA + kSlots * kABytes;
constexpr uint32_t kSmMisc = kSmLights + 24u * kMlpSmemLights;

struct SlotMisc {
    unsigned long long mbar;          // MMA completion
    uint32_t fail[2];                 // by tile parity: a checked row exceeded the bound
    float rec[kMaxSamples][4];        // the checked rows' normals (xyz), written by their threads
    float part[4][4 * kMaxSamples];   // per warp: partial light sums of the checked rows (3s + c)
};
struct MlpMisc {
    unsigned long long mbar_w;        // the weights' bulk copy
    unsigned long long mbar_idle;     // nothing arrives on it (the stall test's first wait)
    uint32_t tmem;
    uint32_t pad[3];
    SlotMisc slot[kSlots];
};
constexpr uint32_t kMlpSmem = kSmMisc + sizeof(MlpMisc);
static_assert(kSmW2 % 16 == 0 && kSmW3 % 16 == 0 && kSmA % 1024 == 0 && kSmLights % 16 == 0 && kSmMisc % 16 == 0,
              "operand alignment");
static_assert(kMlpSmem <= 227 * 1024, "shared memory of one CTA");
static_assert(sizeof(MlpImage) % 16 == 0, "bulk copy alignment");

inline uint32_t mlp_smem_bytes() { return kMlpSmem; }

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// The checked records of tile t: ranks floor(hash(t, s) * count / 2^32), the same in every thread.
__device__ __forceinline__ uint32_t sample_rank(uint32_t t, int s, uint32_t count) {
    return __umulhi(hash32(t * 8u + (uint32_t)s + 0x9E3779B9u), count);
}

// Named barrier of slot s (ids 1..kSlots; 0 is __syncthreads), with an OR of `v` over its threads.
__device__ __forceinline__ bool slot_sync_or(int s, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(s + 1), "r"(kSlotThreads)
        : "memory");
    return r != 0u;
}
__device__ __forceinline__ void slot_sync(int s) {
    asm volatile("bar.sync %0, %1;" ::"r"(s + 1), "r"(kSlotThreads) : "memory");
}

// Makes this thread's shared-memory stores visible to the tensor cores' reads (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(x), "r"(y), "r"(z), "r"(w) : "memory");
}

// Row r's 16-byte chunk j (K elements 8j..8j+7) of a slot's A operand at `base`: the K-major,
// unswizzled core layout of core_offset().
__device__ __forceinline__ uint32_t a_chunk(uint32_t base, uint32_t r, uint32_t j) {
    return base + j * kALbo + (r >> 3) * 128u + (r & 7u) * 16u;
}

// tcgen05.mma kind::f16, A and B from shared memory (descriptors), D in tensor memory.
__device__ __forceinline__ void mma_bf16_ss(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// One layer's MMAs into the slot's accumulators, A (128 x K) from its operand (tensor memory
// columns or shared memory) and B (b_rows x K) from the weights; committed to mbar.
__device__ __forceinline__ void issue_layer(uint32_t d, uint32_t a, uint32_t b_smem, uint32_t b_rows, int k_steps,
                                            uint32_t idesc, uint32_t mbar) {
    tc_fence_after();
    const uint32_t lbo_b = b_rows * 16u;
    for (int s = 0; s < k_steps; ++s) {
        const uint64_t b = mma_desc(b_smem + 2u * s * lbo_b, lbo_b, 128);
        if constexpr (kATmem) mma_bf16_ta(d, a + 8u * s, b, idesc, s > 0);
        else mma_bf16_ss(d, mma_desc(a + 2u * s * kALbo, kALbo, 128), b, idesc, s > 0);
    }
    mma_commit(mbar);
}

// Eight packed pairs (16 K elements) of row r into the slot's A operand at chunk pair j2 (K
// elements 16 j2 .. 16 j2 + 15): 8 tensor-memory columns of this thread's lane, or two 16-byte
// shared-memory chunks.
__device__ __forceinline__ void put_a8(uint32_t a, uint32_t r, uint32_t j2, const uint32_t (&q)[8]) {
    if constexpr (kATmem) {
        tmem_st8(a + 8u * j2, q);
    } else {
        st_shared_v4(a_chunk(a, r, 2u * j2), q[0], q[1], q[2], q[3]);
        st_shared_v4(a_chunk(a, r, 2u * j2 + 1u), q[4], q[5], q[6], q[7]);
    }
}

// Makes the A operand written by this thread visible to the MMA the slot issues next (before the
// slot barrier).
__device__ __forceinline__ void a_written() {
    if constexpr (kATmem) tmem_wait_st();
    else fence_async_smem();
    tc_fence_before();
}

// The features of one row (mlp_feature_pairs' order) into its A operand, 8 pairs at a time.
__device__ __forceinline__ void store_features(float3 n, float3 alb, uint32_t a, uint32_t r) {
    static_assert(kMlpFreq == 8, "one 8-pair store per normal component");
    const float comp[3] = {n.x, n.y, n.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        uint32_t q[8];
        fourier_pairs(comp[c], [&](int f, uint32_t p) { q[f] = p; });
        put_a8(a, r, (uint32_t)c, q);
    }
    uint32_t t[8];
    tail_pairs(n, alb, t);
    put_a8(a, r, 3u, t);
}

// Epilogue of a hidden layer: row r's 64 accumulators (TMEM columns from d) through ReLU, rounded
// to BF16, into its A operand (over the consumed features or h1): the next layer's A.
// kLdBatch 16-column loads are in flight per wait.
__device__ __forceinline__ void hidden_epilogue(uint32_t d, uint32_t a, uint32_t r) {
#pragma unroll
    for (int g = 0; g < kMlpHid / 16; g += kLdBatch) {
        uint32_t v[kLdBatch][16];
#pragma unroll
        for (int i = 0; i < kLdBatch; ++i) tmem_ld16(d + 16u * (g + i), v[i]);
        tmem_wait16(v[0]);
#pragma unroll
        for (int i = 1; i < kLdBatch; ++i) reg_fence16(v[i]);
#pragma unroll
        for (int i = 0; i < kLdBatch; ++i) {
            uint32_t p[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) p[j] = relu_bf16x2(__uint_as_float(v[i][2 * j]), __uint_as_float(v[i][2 * j + 1]));
            put_a8(a, r, (uint32_t)(g + i), p);
        }
    }
}

// The light table of the checks: dirI[l] = (-dir xyz, I*r), gb[l] = (I*g, I*b).
struct SmemLights {
    const float4* dirI;
    const float2* gb;
};

__device__ __forceinline__ void stage_lights_soa(const float* lights, int n, float4* dirI, float2* gb) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float* p = lights + 7 * (int64_t)i;
        const float I = __ldg(p + 3);
        dirI[i] = make_float4(-__ldg(p), -__ldg(p + 1), -__ldg(p + 2), I * __ldg(p + 4));
        gb[i] = make_float2(I * __ldg(p + 5), I * __ldg(p + 6));
    }
}

// Sums V values over the 32 lanes by halving: at each level a lane keeps half of its values and
// adds its partner's copy of them. Returns, in lanes with (lane & (32/V - 1)) == 0, the total of
// value lane / (32/V).
template <int V>
__device__ __forceinline__ float halving_sum(float (&v)[V], int lane) {
#pragma unroll
    for (int h = V / 2, o = 16; h >= 1; h >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const float mine = up ? v[i + h] : v[i], other = up ? v[i] : v[i + h];
            v[i] = mine + __shfl_xor_sync(kFull, other, o);
        }
    }
#pragma unroll
    for (int o = 16 / V; o >= 1; o >>= 1) v[0] += __shfl_xor_sync(kFull, v[0], o);
    return v[0];
}

// This thread's share of the light sums of a tile's checked rows: the slot's 128 threads split
// the lights, each warp sums its lanes' shares (halving_sum) into S.part[warp]. The check only
// estimates the error (it never produces a colour), so it sums sum_l (I c)_l * max(0, n . -dir_l)
// with fused multiply-adds; albedo and 1/pi are applied by the checked row itself. Lights come
// from the shared table when it holds them, else from global memory.
template <int NS>
__device__ __forceinline__ void check_part(const ShadeArgs& a, const SmemLights* L, SlotMisc& S, int row) {
    constexpr int V = NS <= 2 ? 8 : 16;
    float v[V];
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = 0.f;
    float nx[NS], ny[NS], nz[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        nx[s] = S.rec[s][0];
        ny[s] = S.rec[s][1];
        nz[s] = S.rec[s][2];
    }
    for (int l = row; l < a.nl; l += kSlotThreads) {
        float4 A;
        float2 B;
        if (L) {
            A = L->dirI[l];
            B = L->gb[l];
        } else {
            const float* P = a.lights + 7 * (int64_t)l;
            const float I = __ldg(P + 3);
            A = make_float4(-__ldg(P), -__ldg(P + 1), -__ldg(P + 2), I * __ldg(P + 4));
            B = make_float2(I * __ldg(P + 5), I * __ldg(P + 6));
        }
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const float m = fmaxf(fmaf(nz[s], A.z, fmaf(ny[s], A.y, nx[s] * A.x)), 0.f);
            v[3 * s] = fmaf(A.w, m, v[3 * s]);
            v[3 * s + 1] = fmaf(B.x, m, v[3 * s + 1]);
            v[3 * s + 2] = fmaf(B.y, m, v[3 * s + 2]);
        }
    }
    const int lane = row & 31;
    const float total = halving_sum<V>(v, lane);
    const int j = lane / (32 / V);
    if ((lane & (32 / V - 1)) == 0 && j < 3 * NS) S.part[row >> 5][j] = total;
}

__global__ void __launch_bounds__(kMlpThreads, 1) k_shade_mlp(ShadeArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    MlpMisc& M = *reinterpret_cast<MlpMisc*>(sm + kSmMisc);
    const int slot = threadIdx.x / kSlotThreads, row = threadIdx.x % kSlotThreads;
    const int wq = row >> 5, lane = threadIdx.x & 31;  // warp within the slot = its TMEM lane quarter
    SlotMisc& S = M.slot[slot];
    const int n_samples = a.eval_out ? 0 : min(a.samples, (int)kMaxSamples);
    float4* lights_dirI = reinterpret_cast<float4*>(sm + kSmLights);
    float2* lights_gb = reinterpret_cast<float2*>(sm + kSmLights + 16u * kMlpSmemLights);
    SmemLights table{lights_dirI, lights_gb};
    const SmemLights* L = (n_samples > 0 && a.nl <= kMlpSmemLights) ? &table : nullptr;

    const uint32_t mbar_w = smem_addr(&M.mbar_w), mbar = smem_addr(&S.mbar);
    // The stall test's first MMA wait polls an mbarrier that nothing arrives on, briefly, and so
    // gives up as a wait for a lost MMA would; the MMA itself runs and completes.
    const uint32_t mbar_first = a.stall_test ? smem_addr(&M.mbar_idle) : mbar;
    const uint32_t tries_first = a.stall_test ? kStallTestTries : kWaitTries;
    if (threadIdx.x == 0) {
        mbar_init(mbar_w, 1);
        mbar_init(smem_addr(&M.mbar_idle), 1);
        for (int s = 0; s < kSlots; ++s) mbar_init(smem_addr(&M.slot[s].mbar), 1);
        // the weights and output scale arrive by one bulk copy (independent of the grid this
        // kernel may overlap with)
        mbar_expect_tx(mbar_w, sizeof(MlpImage));
        bulk_copy_g2s(smem_addr(sm), a.mlp, sizeof(MlpImage), mbar_w);
    }
    if (row == 0) S.fail[0] = S.fail[1] = 0u;
    if (L) stage_lights_soa(a.lights, a.nl, lights_dirI, lights_gb);
    if (threadIdx.x < 32) tmem_alloc(smem_addr(&M.tmem), kTmemCols);
    // the records and the tile list are the previous kernel's output
    asm volatile("griddepcontrol.wait;" ::: "memory");

    const uint32_t n_tiles = a.index[1];
    // Slot g = blockIdx.x * kSlots + slot takes tiles g, g + stride, ...
    const uint32_t stride = gridDim.x * kSlots;
    uint32_t t = blockIdx.x * kSlots + slot;
    uint32_t count = t < n_tiles ? shade_tile_count(a.index, t) : 0u;
    float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f), g1 = g0;
    if ((uint32_t)row < count) {
        const size_t rs = shade_record_slot(a.index, a.n_blocks, shade_tile_desc(a.index, a.n_blocks, t), t, row);
        g0 = a.gbuf[2 * rs];
        g1 = a.gbuf[2 * rs + 1];
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    bool failed = !__syncthreads_and(mbar_wait(mbar_w, 0));
    const bool weights_pending = failed;
    const uint32_t tmem = M.tmem;
    const uint32_t d_cols = tmem + (uint32_t)slot * kSlotCols;                // lane 0, this slot's accumulators
    const uint32_t lane_off = (uint32_t)(wq * 32) << 16;                      // this warp's lanes
    const uint32_t d_lane = d_cols + lane_off;
    const float out_scale = reinterpret_cast<const MlpImage*>(sm)->out_scale;
    const uint32_t sW1 = smem_addr(sm + kSmW1), sW2 = smem_addr(sm + kSmW2), sW3 = smem_addr(sm + kSmW3);
    // the slot's A operand: for the MMA (lane 0) and for this thread's writes
    const uint32_t a_mma = kATmem ? tmem + kSlots * kSlotCols + (uint32_t)slot * kACols
                                  : smem_addr(sm + kSmA + (size_t)slot * kABytes);
    const uint32_t a_mine = kATmem ? a_mma + lane_off : a_mma;

    // Every slot barrier of the loop also ORs the threads' timeout flags, so a slot's threads leave
    // the loop at the same barrier (the loop condition itself is the same in all of them).
    uint32_t phase = 0;
    uint32_t n_tile = 0, n_fallback = 0;
    float max_err = 0.f;
    uint32_t k = 0;  // tiles this slot shaded
    // The previous tile's record of this row, for its exact reshading when its check failed. The
    // verdict is read after the next slot barrier, which orders it after the checked rows' writes.
    const bool checking = n_samples > 0;
    float3 p_nv = make_float3(0.f, 0.f, 0.f), p_alb = p_nv;
    uint32_t p_pix = 0;
    bool p_valid = false;
    auto reshade_previous = [&]() {
        if (S.fail[(k - 1u) & 1u]) {  // the same in every thread of the slot
            if (row == 0) ++n_fallback;
            if (p_valid) write_rgb(a.rgb, a.npx, p_pix, shade_lights(a.lights, a.nl, p_nv, p_alb));
        }
    };

    while (!weights_pending && t < n_tiles) {
        const float3 nv = make_float3(g0.x, g0.y, g0.z), alb = make_float3(g0.w, g1.x, g1.y);
        // which checked sample this row is, if any
        int my_sample = -1;
        for (int s = 0; s < n_samples; ++s)
            if (sample_rank(t, s, count) == (uint32_t)row) my_sample = s;
        if (my_sample >= 0) {
            S.rec[my_sample][0] = nv.x;
            S.rec[my_sample][1] = nv.y;
            S.rec[my_sample][2] = nv.z;
        }
        // Rows past the tile's records hold zeros: finite features whose results are not stored.
        // The previous tile's MMAs completed (its last wait), so the operand is free, unless that
        // wait gave up. After a wait gave up (`failed`), a warp touches tensor memory and the A
        // operand no more: an MMA may still be using them. The test is warp-uniform, as the
        // .sync.aligned tcgen05 instructions need.
        if (!__any_sync(kFull, failed)) store_features(nv, alb, a_mine, (uint32_t)row);
        a_written();
        if (slot_sync_or(slot, failed)) break;

        // layer 1: D = X (128 x K) * W1^T
        if (row == 0) issue_layer(d_cols, a_mma, sW1, kMlpHid, kMlpIn / 16, idesc_bf16(kMlpRows, kMlpHid), mbar);
        // while the MMAs run: the previous tile's fallback, and the checked rows' light sums
        if (checking) {
            if (k > 0u) reshade_previous();
            if (n_samples <= 2) check_part<2>(a, L, S, row);
            else check_part<4>(a, L, S, row);
        }
        failed |= !mbar_wait(mbar_first, phase, tries_first);
        phase ^= 1u;
        tc_fence_after();
        if (!__any_sync(kFull, failed)) hidden_epilogue(d_lane, a_mine, (uint32_t)row);  // h1 over the features
        a_written();
        if (slot_sync_or(slot, failed)) break;
        // every thread read the previous tile's verdict before this barrier; the next tile's
        // checked rows write it after two more
        if (row == 0) S.fail[(k + 1u) & 1u] = 0u;

        // layer 2: D = H1 (128 x 64) * W2^T (layer 1's accumulators were read)
        if (row == 0) issue_layer(d_cols, a_mma, sW2, kMlpHid, kMlpHid / 16, idesc_bf16(kMlpRows, kMlpHid), mbar);
        // this thread's record of the slot's next tile, fetched during the last two MMAs
        const uint32_t t_next = t + stride;
        const uint32_t count_next = t_next < n_tiles ? shade_tile_count(a.index, t_next) : 0u;
        float4 g0n = make_float4(0.f, 0.f, 0.f, 0.f), g1n = g0n;
        if ((uint32_t)row < count_next) {
            const size_t rs =
                shade_record_slot(a.index, a.n_blocks, shade_tile_desc(a.index, a.n_blocks, t_next), t_next, row);
            g0n = a.gbuf[2 * rs];
            g1n = a.gbuf[2 * rs + 1];
        }
        failed |= !mbar_wait(mbar, phase);
        phase ^= 1u;
        tc_fence_after();
        if (!__any_sync(kFull, failed)) hidden_epilogue(d_lane, a_mine, (uint32_t)row);  // h2 over h1
        a_written();
        if (slot_sync_or(slot, failed)) break;

        // layer 3: D[0, 16) = H2 (128 x 64) * W3^T
        if (row == 0) issue_layer(d_cols, a_mma, sW3, kMlpOutPad, kMlpHid / 16, idesc_bf16(kMlpRows, kMlpOutPad), mbar);
        failed |= !mbar_wait(mbar, phase);
        phase ^= 1u;
        tc_fence_after();
        uint32_t o[4] = {0u, 0u, 0u, 0u};
        if (!__any_sync(kFull, failed)) {
            tmem_ld4(d_lane, o);
            tmem_wait4(o);
        }
        tc_fence_before();
        const bool valid = (uint32_t)row < count && !failed;
        const uint32_t pix = __float_as_uint(g1.z);
        const float3 rad = make_float3(alb.x * (__uint_as_float(o[0]) * out_scale),
                                       alb.y * (__uint_as_float(o[1]) * out_scale),
                                       alb.z * (__uint_as_float(o[2]) * out_scale));
        if (a.eval_out) {
            if (valid) {
                a.eval_out[3 * (size_t)pix] = rad.x;
                a.eval_out[3 * (size_t)pix + 1] = rad.y;
                a.eval_out[3 * (size_t)pix + 2] = rad.z;
            }
        } else {
            const float3 radc = make_float3(fminf(fmaxf(rad.x, 0.f), 255.f), fminf(fmaxf(rad.y, 0.f), 255.f),
                                            fminf(fmaxf(rad.z, 0.f), 255.f));
            if (valid)
                write_rgb(a.rgb, a.npx, pix,
                          __float2uint_rz(radc.x) | (__float2uint_rz(radc.y) << 8) | (__float2uint_rz(radc.z) << 16));
            if (checking) {
                // the checked rows against their light sums (the warps' parts, written before two
                // slot barriers); a failing tile is shaded again, exactly, by all its rows after
                // the next slot barrier
                if (my_sample >= 0 && valid) {
                    float sum[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        sum[c] = (S.part[0][3 * my_sample + c] + S.part[1][3 * my_sample + c]) +
                                 (S.part[2][3 * my_sample + c] + S.part[3][3 * my_sample + c]);
                    const float er = fabsf(radc.x - fminf(sum[0] * alb.x * kOneOverPi, 255.f));
                    const float eg = fabsf(radc.y - fminf(sum[1] * alb.y * kOneOverPi, 255.f));
                    const float eb = fabsf(radc.z - fminf(sum[2] * alb.z * kOneOverPi, 255.f));
                    const float err = fmaxf(er, fmaxf(eg, eb));
                    max_err = fmaxf(max_err, err);
                    if (err > a.bound) S.fail[k & 1u] = 1u;
                }
                p_nv = nv;
                p_alb = alb;
                p_pix = pix;
                p_valid = valid;
            }
            ++n_tile;
        }
        ++k;
        t = t_next;
        count = count_next;
        g0 = g0n;
        g1 = g1n;
    }

    // the last tile's verdict (every thread of the slot reaches this barrier: the loop ends at the
    // same point in all of them)
    if (checking && !weights_pending && !slot_sync_or(slot, failed) && k > 0u) reshade_previous();

    if (failed) {
        // the weights' copy or an MMA did not complete in time: record it, give the pending one
        // another bounded wait, then release the tensor memory
        if (row == 0) atomicOr(&a.counters[1], STATUS_SHADE_TIMEOUT);
        if (weights_pending) mbar_wait(mbar_w, 0);
        else mbar_wait(mbar, phase ^ 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
    if (a.stats && !a.eval_out) {
        if (row == 0 && n_tile) {
            atomicAdd(a.stats + 0, (unsigned long long)n_tile);
            if (n_fallback) atomicAdd(a.stats + 1, (unsigned long long)n_fallback);
            atomicAdd(a.stats + 2, (unsigned long long)n_tile * (unsigned long long)n_samples);
        }
        if (max_err > 0.f) atomicMax(a.stats + 3, (unsigned long long)__float_as_uint(max_err));
    }
}

// ---------------------------------------------------------------------------------------------
// training
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ float unit_float(uint64_t h) { return (float)(h >> 40) * 0x1p-24f; }

// Sample i: a normal uniform on the sphere, an albedo uniform in [0,1]^3, and the exact shader's
// float radiance for them under the lights (9 floats: normal, albedo, radiance).
__global__ void k_mlp_samples(float* __restrict__ out, int64_t n, uint64_t seed, const float* __restrict__ lights,
                              int nl) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)i));
    const float z = 2.f * unit_float(h) - 1.f;
    const float phi = unit_float(splitmix64(h + 1));
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp, cp;
    sincospif(2.f * phi, &sp, &cp);
    const float3 nv = make_float3(r * cp, r * sp, z);
    const float3 alb = make_float3(unit_float(splitmix64(h + 2)), unit_float(splitmix64(h + 3)),
                                   unit_float(splitmix64(h + 4)));
    const float3 rad = light_sum(lights, nl, nv, alb);
    float* o = out + 9 * i;
    o[0] = nv.x; o[1] = nv.y; o[2] = nv.z;
    o[3] = alb.x; o[4] = alb.y; o[5] = alb.z;
    o[6] = rad.x; o[7] = rad.y; o[8] = rad.z;
}

// Stores records (normal, albedo, index) for evaluation: record i in slot i, 1024 per block.
__global__ void k_mlp_stage(const float* __restrict__ src, int stride, int64_t n, float4* __restrict__ gbuf,
                            uint32_t* __restrict__ count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t blocks = (n + kShadeBlock - 1) / kShadeBlock;
    if (i < blocks) count[i] = (uint32_t)::min((int64_t)kShadeBlock, n - i * kShadeBlock);
    if (i >= n) return;
    const float* s = src + (int64_t)stride * i;
    gbuf[2 * i] = make_float4(s[0], s[1], s[2], s[3]);
    gbuf[2 * i + 1] = make_float4(s[4], s[5], __uint_as_float((uint32_t)i), 0.f);
}

constexpr int kTrainB = 64;          // samples per CTA and step
constexpr int kTrainThreads = 256;
constexpr int kSX = kMlpIn + 4;      // shared row stride (floats) of X and W1: rows stay 16-byte
constexpr int kSH = 68;              // aligned and eight rows cover all banks; of H, D and W2

struct TrainSmem {
    float w1[kMlpHid * kSX];
    float w2[kMlpHid * kSH];
    float w3[kMlpOut * kMlpHid];
    float pad[4];
    float x[kTrainB * kSX];
    float h1[kTrainB * kSH];
    float h2[kTrainB * kSH];
    float d1[kTrainB * kSH];
    float d2[kTrainB * kSH];
    float y[kTrainB * 4];     // label, then the output gradient
    float alb[kTrainB * 4];
    float red[kTrainThreads];
};

struct TrainArgs {
    const float* q;          // BF16-rounded parameters
    const float* samples;    // 9 floats each
    int64_t n;
    int64_t first;           // first sample of the step; CTA c takes [first + 64c, +64) mod n
    float out_scale;
    float grad_scale;        // d loss / d prediction = grad_scale * (prediction - label)
    float* grad;             // per CTA kMlpParams partial gradients
    float* loss;             // per CTA partial sum of squared errors
};

// One step's forward and backward pass for 64 samples per CTA, in FP32 with the rounding of the
// tensor-core kernel (BF16 features, weights and hidden activations); per-CTA partial gradients.
__global__ void __launch_bounds__(kTrainThreads) k_mlp_train(TrainArgs a) {
    extern __shared__ __align__(16) uint8_t smraw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smraw);
    const int tid = threadIdx.x;
    for (int i = tid; i < kMlpHid * kMlpIn; i += kTrainThreads) S.w1[(i / kMlpIn) * kSX + i % kMlpIn] = a.q[kPW1 + i];
    for (int i = tid; i < kMlpHid * kMlpHid; i += kTrainThreads) S.w2[(i / kMlpHid) * kSH + i % kMlpHid] = a.q[kPW2 + i];
    for (int i = tid; i < kMlpOut * kMlpHid; i += kTrainThreads) S.w3[i] = a.q[kPW3 + i];
    if (tid < kTrainB) {
        const int64_t i = (a.first + (int64_t)blockIdx.x * kTrainB + tid) % a.n;
        const float* s = a.samples + 9 * i;
        const float3 nv = make_float3(s[0], s[1], s[2]), alb = make_float3(s[3], s[4], s[5]);
        uint32_t pairs[kMlpIn / 2];
        mlp_feature_pairs(nv, alb, pairs);
        float* x = S.x + tid * kSX;
#pragma unroll
        for (int k = 0; k < kMlpIn / 2; ++k) {
            x[2 * k] = __uint_as_float(pairs[k] << 16);
            x[2 * k + 1] = __uint_as_float(pairs[k] & 0xFFFF0000u);
        }
        S.alb[4 * tid] = alb.x; S.alb[4 * tid + 1] = alb.y; S.alb[4 * tid + 2] = alb.z;
        S.y[4 * tid] = s[6]; S.y[4 * tid + 1] = s[7]; S.y[4 * tid + 2] = s[8];
    }
    __syncthreads();

    const int j = tid & 63, q4 = tid >> 6;  // unit j, quarter q4 of the samples / inputs
    // forward, layer 1: 16 samples of unit j
    {
        float acc[16];
#pragma unroll
        for (int bb = 0; bb < 16; ++bb) acc[bb] = 0.f;
        for (int k = 0; k < kMlpIn; k += 4) {
            const float4 w = *reinterpret_cast<const float4*>(S.w1 + j * kSX + k);
#pragma unroll
            for (int bb = 0; bb < 16; ++bb) {
                const float4 x = *reinterpret_cast<const float4*>(S.x + (16 * q4 + bb) * kSX + k);
                acc[bb] = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, fmaf(w.w, x.w, acc[bb]))));
            }
        }
#pragma unroll
        for (int bb = 0; bb < 16; ++bb) S.h1[(16 * q4 + bb) * kSH + j] = bf16_round(fmaxf(acc[bb], 0.f));
    }
    __syncthreads();
    // layer 2
    {
        float acc[16];
#pragma unroll
        for (int bb = 0; bb < 16; ++bb) acc[bb] = 0.f;
        for (int k = 0; k < kMlpHid; k += 4) {
            const float4 w = *reinterpret_cast<const float4*>(S.w2 + j * kSH + k);
#pragma unroll
            for (int bb = 0; bb < 16; ++bb) {
                const float4 x = *reinterpret_cast<const float4*>(S.h1 + (16 * q4 + bb) * kSH + k);
                acc[bb] = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, fmaf(w.w, x.w, acc[bb]))));
            }
        }
#pragma unroll
        for (int bb = 0; bb < 16; ++bb) S.h2[(16 * q4 + bb) * kSH + j] = bf16_round(fmaxf(acc[bb], 0.f));
    }
    __syncthreads();
    // layer 3, loss and output gradient
    float sq = 0.f;
    if (tid < kTrainB * kMlpOut) {
        const int b = tid / kMlpOut, c = tid % kMlpOut;
        float o = 0.f;
        for (int k = 0; k < kMlpHid; ++k) o = fmaf(S.w3[c * kMlpHid + k], S.h2[b * kSH + k], o);
        const float al = S.alb[4 * b + c];
        const float diff = al * (o * a.out_scale) - S.y[4 * b + c];
        sq = diff * diff;
        S.y[4 * b + c] = a.grad_scale * diff * al * a.out_scale;  // only this thread reads the label
    }
    __syncthreads();
    float* g = a.grad + (size_t)blockIdx.x * kMlpParams;
    // layer 3 gradients and dH2
    if (tid < kMlpOut * kMlpHid) {
        const int c = tid / kMlpHid, k = tid % kMlpHid;
        float s = 0.f;
        for (int b = 0; b < kTrainB; ++b) s = fmaf(S.y[4 * b + c], S.h2[b * kSH + k], s);
        g[kPW3 + c * kMlpHid + k] = s;
    }
#pragma unroll 4
    for (int bb = 0; bb < 16; ++bb) {
        const int b = 16 * q4 + bb;
        float v = 0.f;
#pragma unroll
        for (int c = 0; c < kMlpOut; ++c) v = fmaf(S.w3[c * kMlpHid + j], S.y[4 * b + c], v);
        S.d2[b * kSH + j] = S.h2[b * kSH + j] > 0.f ? v : 0.f;
    }
    __syncthreads();
    // layer 2 gradients (unit j, inputs 16*q4..) and dH1 (input unit j, samples 16*q4..)
    {
        float acc[16];
#pragma unroll
        for (int ii = 0; ii < 16; ++ii) acc[ii] = 0.f;
        for (int b = 0; b < kTrainB; ++b) {
            const float d = S.d2[b * kSH + j];
#pragma unroll
            for (int ii = 0; ii < 16; ii += 4) {
                const float4 h = *reinterpret_cast<const float4*>(S.h1 + b * kSH + 16 * q4 + ii);
                acc[ii] = fmaf(d, h.x, acc[ii]);
                acc[ii + 1] = fmaf(d, h.y, acc[ii + 1]);
                acc[ii + 2] = fmaf(d, h.z, acc[ii + 2]);
                acc[ii + 3] = fmaf(d, h.w, acc[ii + 3]);
            }
        }
#pragma unroll
        for (int ii = 0; ii < 16; ++ii) g[kPW2 + j * kMlpHid + 16 * q4 + ii] = acc[ii];
        float dh[16];
#pragma unroll
        for (int bb = 0; bb < 16; ++bb) dh[bb] = 0.f;
        for (int u = 0; u < kMlpHid; ++u) {
            const float w = S.w2[u * kSH + j];
#pragma unroll
            for (int bb = 0; bb < 16; ++bb) dh[bb] = fmaf(w, S.d2[(16 * q4 + bb) * kSH + u], dh[bb]);
        }
#pragma unroll
        for (int bb = 0; bb < 16; ++bb) {
            const int b = 16 * q4 + bb;
            S.d1[b * kSH + j] = S.h1[b * kSH + j] > 0.f ? dh[bb] : 0.f;
        }
    }
    __syncthreads();
    // layer 1 gradients: unit j, inputs kQ*q4 .. kQ*q4 + kQ - 1
    {
        constexpr int kQ = kMlpIn / 4;
        static_assert(kQ % 4 == 0, "a quarter of the inputs is whole float4s");
        float acc[kQ];
#pragma unroll
        for (int kk = 0; kk < kQ; ++kk) acc[kk] = 0.f;
        for (int b = 0; b < kTrainB; ++b) {
            const float d = S.d1[b * kSH + j];
#pragma unroll
            for (int kk = 0; kk < kQ; kk += 4) {
                const float4 x = *reinterpret_cast<const float4*>(S.x + b * kSX + kQ * q4 + kk);
                acc[kk] = fmaf(d, x.x, acc[kk]);
                acc[kk + 1] = fmaf(d, x.y, acc[kk + 1]);
                acc[kk + 2] = fmaf(d, x.z, acc[kk + 2]);
                acc[kk + 3] = fmaf(d, x.w, acc[kk + 3]);
            }
        }
#pragma unroll
        for (int kk = 0; kk < kQ; ++kk) g[kPW1 + j * kMlpIn + kQ * q4 + kk] = acc[kk];
    }
    // loss
    S.red[tid] = sq;
    __syncthreads();
    for (int o = kTrainThreads / 2; o > 0; o >>= 1) {
        if (tid < o) S.red[tid] += S.red[tid + o];
        __syncthreads();
    }
    if (tid == 0) a.loss[blockIdx.x] = S.red[0];
}

struct AdamArgs {
    float* w;              // parameters
    float* q;              // rounded copy for the next forward pass
    float* m;
    float* v;
    const float* grad;     // n_part x kMlpParams
    int n_part;
    float lr, beta1, beta2, eps, c1, c2;  // c1 = 1 - beta1^t, c2 = 1 - beta2^t
    const float* loss_part;
    float* loss_out;       // this step's summed squared error
};

__global__ void k_mlp_adam(AdamArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && a.loss_out) {
        float s = 0.f;
        for (int i = 0; i < a.n_part; ++i) s += a.loss_part[i];
        *a.loss_out = s;
    }
    if (p >= kMlpParams || mlp_param_fixed(p)) return;
    float gs = 0.f;
    for (int i = 0; i < a.n_part; ++i) gs += a.grad[(size_t)i * kMlpParams + p];
    const float m = a.beta1 * a.m[p] + (1.f - a.beta1) * gs;
    const float v = a.beta2 * a.v[p] + (1.f - a.beta2) * gs * gs;
    a.m[p] = m;
    a.v[p] = v;
    const float w = a.w[p] - a.lr * (m / a.c1) / (sqrtf(v / a.c2) + a.eps);
    a.w[p] = w;
    a.q[p] = bf16_round(w);
}

int grid_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
static ShadeArgs shade_args(const FrameScratch& s, const DrawParams& p) {
    ShadeArgs a;
    a.gbuf = s.gbuf;
    a.n_blocks = 0;
    a.index = s.shade_index;
    a.npx = (int64_t)p.width * p.height;
    a.lights = p.lights;
    a.nl = p.nl;
    a.rgb = p.rgb;
    a.counters = s.counters;
    a.mlp = static_cast<const MlpImage*>(p.mlp);
    a.samples = p.mlp_samples;
    a.bound = p.mlp_bound;
    a.stats = s.shade_stats;
    a.eval_out = nullptr;
    a.stall_test = p.mlp_stall_test ? 1u : 0u;
    return a;
}

static int mlp_grid(int n_sm, int64_t blocks) {
    static bool attr_set = false;  // per process: the attribute is per function, all devices alike
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_shade_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMlpSmem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_shade_mlp, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return -1;
        attr_set = true;
    }
    // one CTA per SM at most, and no more CTAs than the tiles need (a block of 1024 records makes
    // at most 8 tiles)
    const int64_t max_tiles = (int64_t)(kShadeBlock / kShadeTile) * blocks;
    return (int)std::min<int64_t>((int64_t)n_sm, std::max<int64_t>((max_tiles + kSlots - 1) / kSlots, 1));
}

static int exact_grid(int n_sm, int64_t blocks) {
    return (int)std::min<int64_t>((int64_t)kExactCtasPerSm * n_sm, std::max<int64_t>(8 * blocks, 1));
}

// Launches a shading kernel that may start while the resolve grid before it on the stream is
// still running (programmatic dependent launch); the kernel waits for that grid before it reads
// the records.
template <class Kernel>
static cudaError_t launch_dependent(Kernel kernel, int grid, int threads, uint32_t smem, cudaStream_t stream,
                                   const ShadeArgs& a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a);
}

int launch_shade(const FrameScratch& s, const DrawParams& p, int64_t blocks, cudaStream_t stream) {
    ShadeArgs a = shade_args(s, p);
    a.n_blocks = (uint32_t)blocks;
    cudaError_t err;
    if (p.shader == 1) {
        err = launch_dependent(k_shade_exact, exact_grid(p.n_sm, blocks), kExactThreads, 0, stream, a);
    } else {
        const int grid = mlp_grid(p.n_sm, blocks);
        if (grid < 0) return -1;
        err = launch_dependent(k_shade_mlp, grid, kMlpThreads, mlp_smem_bytes(), stream, a);
    }
    return err == cudaSuccess ? 1 : -1;
}

int launch_mlp_eval(const float* src, int stride, int64_t n, bool exact, float4* gbuf, uint32_t* count,
                    uint32_t* index, const float* lights, int nl, const void* mlp, uint32_t* counters, int n_sm,
                    float* out, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int64_t blocks = (n + kShadeBlock - 1) / kShadeBlock;
    k_mlp_stage<<<grid_for(n, 256), 256, 0, stream>>>(src, stride, n, gbuf, count);
    k_shade_scan<<<1, 1024, 0, stream>>>(count, (uint32_t)blocks, index);
    ShadeArgs a;
    a.gbuf = gbuf;
    a.index = index;
    a.n_blocks = (uint32_t)blocks;
    a.npx = 0;
    a.lights = lights;
    a.nl = nl;
    a.rgb = nullptr;
    a.counters = counters;
    a.mlp = static_cast<const MlpImage*>(mlp);
    a.samples = 0;
    a.bound = 0.f;
    a.stats = nullptr;
    a.eval_out = out;
    a.stall_test = 0u;
    if (exact) {
        k_shade_exact<<<exact_grid(n_sm, blocks), kExactThreads, 0, stream>>>(a);
    } else {
        const int grid = mlp_grid(n_sm, blocks);
        if (grid < 0) return -1;
        k_shade_mlp<<<grid, kMlpThreads, mlp_smem_bytes(), stream>>>(a);
    }
    return cudaGetLastError() == cudaSuccess ? 3 : -1;
}

int launch_mlp_samples(float* out, int64_t n, uint64_t seed, const float* lights, int nl, cudaStream_t stream) {
    if (n <= 0) return 0;
    k_mlp_samples<<<grid_for(n, 256), 256, 0, stream>>>(out, n, seed, lights, nl);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int launch_mlp_train_step(const float* q, const float* samples, int64_t n, int64_t first, int n_cta, float out_scale,
                          float grad_scale, float* grad, float* loss, cudaStream_t stream) {
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem)) !=
            cudaSuccess)
            return -1;
        attr_set = true;
    }
    TrainArgs a;
    a.q = q;
    a.samples = samples;
    a.n = n;
    a.first = first;
    a.out_scale = out_scale;
    a.grad_scale = grad_scale;
    a.grad = grad;
    a.loss = loss;
    k_mlp_train<<<n_cta, kTrainThreads, sizeof(TrainSmem), stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int launch_mlp_adam(float* w, float* q, float* m, float* v, const float* grad, int n_part, float lr, float beta1,
                    float beta2, float eps, float c1, float c2, const float* loss_part, float* loss_out,
                    cudaStream_t stream) {
    AdamArgs a;
    a.w = w; a.q = q; a.m = m; a.v = v; a.grad = grad; a.n_part = n_part;
    a.lr = lr; a.beta1 = beta1; a.beta2 = beta2; a.eps = eps; a.c1 = c1; a.c2 = c2;
    a.loss_part = loss_part;
    a.loss_out = loss_out;
    k_mlp_adam<<<grid_for(kMlpParams, 256), 256, 0, stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int train_batch_per_cta() { return kTrainB; }

}  // namespace rast
