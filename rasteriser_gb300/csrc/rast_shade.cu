// Deferred shading for sm_103a: the exact per-light shader and the learned many-light shader
// over the resolve pass's fragment records, and the kernels that train the learned shader.
//
//   k_shade_exact  shading.cpp:20-34 per fragment, lights staged in shared memory: the plain
//                  shader, bit for bit the reference's colour
//   k_shade_mlp    per tile of 128 records: Fourier features -> three tcgen05 BF16 MMAs with FP32
//                  accumulators in tensor memory -> radiance; a few records of every tile are
//                  checked against the per-light sum, and a tile whose checked error exceeds the
//                  bound is shaded exactly in full (compiled per number of checked records)
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
    const uint8_t* mlp;      // the weights' device image (MlpNet), then the check table
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

// sin and cos of f*pi*v for f = 1..F come from the base pair (the hardware sine and cosine of pi*v,
// |pi*v| <= pi) by the three-term recurrence x_{f+1} = 2 cos(pi v) x_f - x_{f-1}, which both
// sequences satisfy; one packed FMA advances the pair. Its error stays far below BF16's step.
// emit(f, pair) receives the BF16 pair (sin, cos) of frequency f + 1 (sin in the low half).
template <int F, class Emit>
__device__ __forceinline__ void fourier_pairs(float v, Emit&& emit) {
    float s1, c1;
    __sincosf(kPi * v, &s1, &c1);
    const float2 k2 = make_float2(2.f * c1, 2.f * c1);
    float2 prev = make_float2(0.f, 1.f);
    float2 cur = make_float2(s1, c1);
#pragma unroll
    for (int f = 0; f < F; ++f) {
        emit(f, pack_bf16x2(cur.x, cur.y));
        const float2 next = __ffma2_rn(k2, cur, make_float2(-prev.x, -prev.y));
        prev = cur;
        cur = next;
    }
}

// Network N's N::kIn input features, each rounded to BF16, as packed pairs (feature 2i in the low
// half): the Fourier pairs of n.x, n.y and n.z, then (n.x, n.y), (n.z, alb.x), (alb.y, alb.z),
// (1, 0) -- the constant that carries layer 1's bias -- and zero pairs.
constexpr int kTailPairs = 4;
template <class N>
__device__ __forceinline__ void mlp_feature_pairs(float3 n, float3 alb, uint32_t (&pairs)[N::kIn / 2]) {
    constexpr int F = N::kFreq;
    static_assert(N::kConst == 6 * F + 6 && 3 * F + kTailPairs <= N::kIn / 2, "feature layout");
    const float comp[3] = {n.x, n.y, n.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) fourier_pairs<F>(comp[c], [&](int f, uint32_t p) { pairs[c * F + f] = p; });
    pairs[3 * F] = pack_bf16x2(n.x, n.y);
    pairs[3 * F + 1] = pack_bf16x2(n.z, alb.x);
    pairs[3 * F + 2] = pack_bf16x2(alb.y, alb.z);
    pairs[3 * F + 3] = pack_bf16x2(1.f, 0.f);
#pragma unroll
    for (int i = 3 * F + kTailPairs; i < N::kIn / 2; ++i) pairs[i] = 0u;
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
// while one slot waits for its MMAs the others compute. The slots share the weights (B operands,
// one copy in shared memory) and the light table of the checks.
//
// A slot's tensor memory is its FP32 accumulators and two A operands, F for the features and H for
// the hidden layers, every region starting on a multiple of 32 columns: for the compact network
// 32 accumulator columns, F and H 32 each (16 in use: 32 BF16 values per row), 96 in all; for the
// wide one 64, 64 (56 in use) and 32, 160 in all. h2 overwrites h1 once layer 2 has read it, and
// the next tile's features overwrite this tile's while its last MMA runs:
//   features(k) -> F; h1 -> H; h2 -> H; features(k+1) -> F during layer 3.
//
// Checks: the sampled rows of each tile put their normal, albedo and learned colour into the slot's
// check buffer at the end of the tile; after every kCheckTiles tiles, and after the slot's last
// tile, the slot checks the buffered rows (each warp its own rows, its lanes splitting the lights)
// and shades the tiles that failed again, exactly. The kernel is compiled for each network and
// number of checked samples, and the light table comes with the weights (built with them for
// their rig).
//
// RAST_MLP_SLOTS (at most as many slots as fit the 512 columns of tensor memory: 5 compact, 3 wide) and
// RAST_MLP_CHECK_ROWS can be changed at build time to measure other shapes; the defaults are the
// fastest measured for the compact network: five slots, whose 640 threads leave 96 registers each.
#ifndef RAST_MLP_SLOTS
#define RAST_MLP_SLOTS 5
#endif
constexpr int kLdBatch = 4;        // 16-column accumulator loads in flight per wait
constexpr int kSlotThreads = 128;  // warp w of a slot reads TMEM lanes 32w..32w+31 (w = warp id mod 4)
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kMaxSamples = 4;
constexpr int kMlpSmemLights = 512;  // lights the checks read from shared memory
static_assert(kMlpSmemLights == kMlpCheckLights, "the shared table is the image's check table");

struct CheckRow {
    float n[3], alb[3], rad[3];  // the row's normal and albedo, and the learned radiance (clamped)
    uint32_t valid;
};
constexpr uint32_t kCheckTiles = 16;       // tiles a slot buffers before it checks them
struct SlotMisc {
    unsigned long long mbar;                // MMA completion
    uint32_t fail_mask;                     // after a check: bit j set when buffered tile j failed
    uint32_t pad;
    CheckRow q[kCheckTiles][kMaxSamples];   // the buffered tiles' sampled rows
};
template <int kSlots>
struct MlpMisc {
    unsigned long long mbar_w;     // the weights' bulk copy
    unsigned long long mbar_idle;  // nothing arrives on it (the stall test's first wait)
    unsigned long long sums[3];    // the CTA's tiles, fallback tiles and checked rows
    uint32_t max_err_bits;         // the CTA's largest checked error (a non-negative float's bits)
    uint32_t tmem;
    SlotMisc slot[kSlots];
};

constexpr uint32_t round32(uint32_t v) { return (v + 31u) / 32u * 32u; }

// The kernel's layout for network N: tensor-memory columns and slots, threads, and shared memory
// (bytes): the weights and output scale as in the device image, the checks' light table (dirI then
// gb, as in MlpCheckTable), then the small block.
template <class N>
struct MlpLayout {
    static constexpr uint32_t kSlotCols = round32((uint32_t)(N::kHid > kMlpOutPad ? N::kHid : kMlpOutPad));
    static constexpr uint32_t kFCols = round32((uint32_t)N::kIn / 2u);   // the features' A operand
    static constexpr uint32_t kHCols = round32((uint32_t)N::kHid / 2u);  // the hidden layers' A operand
    static constexpr uint32_t kSlotTmem = kSlotCols + kFCols + kHCols;
    static constexpr int kSlots = (int)(kTmemCols / kSlotTmem) < RAST_MLP_SLOTS ? (int)(kTmemCols / kSlotTmem)
                                                                                : RAST_MLP_SLOTS;
    static constexpr int kThreads = kSlots * kSlotThreads;
    static constexpr uint32_t kSmW1 = N::kW1Off, kSmW2 = N::kW2Off, kSmW3 = N::kW3Off, kSmScale = N::kScaleOff;
    static constexpr uint32_t kSmLights = N::kImageBytes;
    static constexpr uint32_t kSmMisc = kSmLights + 24u * kMlpSmemLights;
    static constexpr uint32_t kSmem = kSmMisc + (uint32_t)sizeof(MlpMisc<kSlots>);
    static_assert(kSlots >= 1 && kSlots * kSlotTmem <= kTmemCols, "tensor memory of one SM");
    static_assert(kSmW2 % 16 == 0 && kSmW3 % 16 == 0 && kSmLights % 16 == 0 && kSmMisc % 16 == 0,
                  "operand alignment");
    static_assert(kSmem <= 227 * 1024, "shared memory of one CTA");
};
static_assert(MlpLayout<MlpCompact>::kSlots == 5 || RAST_MLP_SLOTS != 5, "the compact network runs five slots");

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// The checked records of tile t: ranks floor(h_s * count / 2^32) for h_s = (hash(t) + s * c1) * c2
// (c2 odd: a bijection of the hash for each s), the same in every thread.
__device__ __forceinline__ uint32_t sample_hash(uint32_t t) { return hash32(t * 8u + 0x9E3779B9u); }
__device__ __forceinline__ uint32_t sample_rank(uint32_t h, int s, uint32_t count) {
    return __umulhi((h + (uint32_t)s * 0x9E3779B9u) * 0x85EBCA77u, count);
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

// One layer's MMAs into the slot's accumulators, A (128 x K) from tensor memory and B (b_rows x
// K) from the weights in shared memory; committed to mbar.
__device__ __forceinline__ void issue_layer(uint32_t d, uint32_t a, uint32_t b_smem, uint32_t b_rows, int k_steps,
                                            uint32_t idesc, uint32_t mbar) {
    tc_fence_after();
    const uint32_t lbo_b = b_rows * 16u;
    for (int s = 0; s < k_steps; ++s)
        mma_bf16_ta(d, a + 8u * s, mma_desc(b_smem + 2u * s * lbo_b, lbo_b, 128), idesc, s > 0);
    mma_commit(mbar);
}

// Makes the A operand this thread wrote (tcgen05.st) visible to the MMA the slot issues after its
// next barrier, and orders this thread's accumulator reads before that MMA.
__device__ __forceinline__ void a_written() {
    tmem_wait_st();
    tc_fence_before();
}

// The features of one row (mlp_feature_pairs' order) into an A operand (this thread's lane of it),
// 8 pairs (16 K elements) per store.
template <class N>
__device__ __forceinline__ void store_features(float3 n, float3 alb, uint32_t a) {
    static_assert(N::kIn % 16 == 0, "whole 8-pair stores");
    uint32_t q[N::kIn / 2];
    mlp_feature_pairs<N>(n, alb, q);
#pragma unroll
    for (int i = 0; i < N::kIn / 16; ++i) {
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) p[j] = q[8 * i + j];
        tmem_st8(a + 8u * i, p);
    }
}

// Epilogue of a hidden layer: this thread's row of N::kHid accumulators (TMEM columns from d)
// through ReLU, rounded to BF16, into an A operand: the next layer's A. Up to kLdBatch 16-column
// loads are in flight per wait.
template <class N>
__device__ __forceinline__ void hidden_epilogue(uint32_t d, uint32_t a) {
    constexpr int kEpiBatch = N::kHid / 16 < kLdBatch ? N::kHid / 16 : kLdBatch;
    static_assert(N::kHid % 16 == 0 && (N::kHid / 16) % kEpiBatch == 0, "whole batches of 16-column loads");
#pragma unroll
    for (int g = 0; g < N::kHid / 16; g += kEpiBatch) {
        uint32_t v[kEpiBatch][16];
#pragma unroll
        for (int i = 0; i < kEpiBatch; ++i) tmem_ld16(d + 16u * (g + i), v[i]);
        tmem_wait16(v[0]);
#pragma unroll
        for (int i = 1; i < kEpiBatch; ++i) reg_fence16(v[i]);
#pragma unroll
        for (int i = 0; i < kEpiBatch; ++i) {
            uint32_t p[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) p[j] = relu_bf16x2(__uint_as_float(v[i][2 * j]), __uint_as_float(v[i][2 * j + 1]));
            tmem_st8(a + 8u * (g + i), p);
        }
    }
}

// This thread's record of row `row` of tile t, whose descriptor is d (zeros past the tile's count).
__device__ __forceinline__ void load_record_desc(const ShadeArgs& a, uint32_t t, uint32_t count, uint4 d, int row,
                                                 float4& g0, float4& g1) {
    g0 = g1 = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((uint32_t)row < count) {
        const size_t rs = shade_record_slot(a.index, a.n_blocks, d, t, row);
        g0 = a.gbuf[2 * rs];
        g1 = a.gbuf[2 * rs + 1];
    }
}
__device__ __forceinline__ void load_record(const ShadeArgs& a, uint32_t t, uint32_t count, int row, float4& g0,
                                            float4& g1) {
    const uint4 d = (uint32_t)row < count ? shade_tile_desc(a.index, a.n_blocks, t) : make_uint4(0u, 0u, 0u, 0u);
    load_record_desc(a, t, count, d, row, g0, g1);
}
// Tile t's descriptor, read before the tile count is known: the list has room for 8 tiles per
// block, so every t below that reads inside it (what it reads past the last tile goes unused).
__device__ __forceinline__ uint4 tile_desc_early(const ShadeArgs& a, uint32_t t) {
    return t < a.n_blocks * (uint32_t)(kShadeBlock / kShadeTile) ? shade_tile_desc(a.index, a.n_blocks, t)
                                                                 : make_uint4(0u, 0u, 0u, 0u);
}

// Records in tile t of n_tiles, from the fragment total.
__device__ __forceinline__ uint32_t tile_count(uint32_t n_frag, uint32_t n_tiles, uint32_t t) {
    return t < n_tiles ? min((uint32_t)kShadeTile, n_frag - t * (uint32_t)kShadeTile) : 0u;
}

// The light table of the checks: dirI[l] = (-dir xyz, I*r), gb[l] = (I*g, I*b).
struct SmemLights {
    const float4* dirI;
    const float2* gb;
};

// The check of the slot's buffered tiles (n_rows = tiles * NS sampled rows, tile j's sample s at
// q[j][s]): warp w of the slot takes rows w, w + 4, ... (kCheckRows of them per pass), its lanes
// split the lights (lane `lane` takes lights lane, lane + 32, ...), and each lane sums, per row i
// and channel c, (I c)_l * max(0, n . -dir_l) with fused multiply-adds. The warp adds its lanes'
// sums by halving (each level a lane keeps half of its values and adds its partner's copy of them,
// leaving value j in the lanes j mod kCheckVals), then the lane groups, and lane 3 i + c compares
// |learned - min(sum * albedo / pi, 255)| with the bound, marking the row's tile in fail_mask. The
// sum only estimates the exact shade: it judges the learned colour and is never itself a colour.
// Lights come from the shared table when it holds them, else from global memory. The caller's next
// slot barrier orders the marks before they are read.
#ifndef RAST_MLP_CHECK_ROWS
#define RAST_MLP_CHECK_ROWS 2
#endif
constexpr int kCheckRows = RAST_MLP_CHECK_ROWS;  // rows of one warp per pass
constexpr int kCheckVals = 3 * kCheckRows <= 8 ? 8 : 16;  // sums per lane, a power of two
static_assert(3 * kCheckRows <= kCheckVals, "one sum per lane");
template <int NS>
__device__ void check_rows(const ShadeArgs& a, const SmemLights* L, SlotMisc& S, int n_rows, int wq, int lane,
                           float& max_err) {
    for (int r0 = wq; r0 < n_rows; r0 += 4 * kCheckRows) {
        float nx[kCheckRows], ny[kCheckRows], nz[kCheckRows];
#pragma unroll
        for (int i = 0; i < kCheckRows; ++i) {
            const int r = r0 + 4 * i;
            const bool in = r < n_rows;
            const CheckRow& q = S.q[in ? r / NS : 0][in ? r % NS : 0];
            nx[i] = in ? q.n[0] : 0.f;
            ny[i] = in ? q.n[1] : 0.f;
            nz[i] = in ? q.n[2] : 0.f;
        }
        float v[kCheckVals];
#pragma unroll
        for (int j = 0; j < kCheckVals; ++j) v[j] = 0.f;
        auto acc = [&](float4 A, float2 B) {
#pragma unroll
            for (int i = 0; i < kCheckRows; ++i) {
                const float m = fmaxf(fmaf(nz[i], A.z, fmaf(ny[i], A.y, nx[i] * A.x)), 0.f);
                v[3 * i] = fmaf(A.w, m, v[3 * i]);
                v[3 * i + 1] = fmaf(B.x, m, v[3 * i + 1]);
                v[3 * i + 2] = fmaf(B.y, m, v[3 * i + 2]);
            }
        };
        if (L) {
            for (int l = lane; l < a.nl; l += 32) acc(L->dirI[l], L->gb[l]);
        } else {
            for (int l = lane; l < a.nl; l += 32) {
                const float* P = a.lights + 7 * (int64_t)l;
                const float I = __ldg(P + 3);
                acc(make_float4(-__ldg(P), -__ldg(P + 1), -__ldg(P + 2), I * __ldg(P + 4)),
                    make_float2(I * __ldg(P + 5), I * __ldg(P + 6)));
            }
        }
#pragma unroll
        for (int h = kCheckVals / 2; h >= 1; h >>= 1) {
            const bool up = (lane & h) != 0;
#pragma unroll
            for (int i = 0; i < h; ++i) {
                const float mine = up ? v[i + h] : v[i], other = up ? v[i] : v[i + h];
                v[i] = mine + __shfl_xor_sync(kFull, other, h);
            }
        }
#pragma unroll
        for (int o = kCheckVals; o < 32; o <<= 1) v[0] += __shfl_xor_sync(kFull, v[0], o);
        const int i = lane / 3, c = lane - 3 * i, r = r0 + 4 * i;
        if (lane < 3 * kCheckRows && r < n_rows) {
            const CheckRow& q = S.q[r / NS][r % NS];
            if (q.valid) {
                const float err = fabsf(q.rad[c] - fminf(v[0] * q.alb[c] * kOneOverPi, 255.f));
                max_err = fmaxf(max_err, err);
                if (!(err <= a.bound)) atomicOr(&S.fail_mask, 1u << (r / NS));
            }
        }
    }
}

// Shades tile t again, exactly, in the reference's order: each row by the thread that shaded it
// before, so the exact colour is the last write.
__device__ void reshade_tile(const ShadeArgs& a, uint32_t t, int row) {
    const uint32_t count = shade_tile_count(a.index, t);
    float4 g0, g1;
    load_record(a, t, count, row, g0, g1);
    if ((uint32_t)row < count)
        write_rgb(a.rgb, a.npx, __float_as_uint(g1.z),
                  shade_lights(a.lights, a.nl, make_float3(g0.x, g0.y, g0.z), make_float3(g0.w, g1.x, g1.y)));
}

// N: the network; NS: checked records per tile (0: none, as in the evaluation mode)
template <class N, int NS>
__global__ void __launch_bounds__(MlpLayout<N>::kThreads, 1) k_shade_mlp(ShadeArgs a) {
    using Lay = MlpLayout<N>;
    constexpr int kSlots = Lay::kSlots;
    constexpr uint32_t kSlotTmem = Lay::kSlotTmem, kSlotCols = Lay::kSlotCols, kFCols = Lay::kFCols;
    constexpr uint32_t kSmLights = Lay::kSmLights, kSmMisc = Lay::kSmMisc;
    extern __shared__ __align__(1024) uint8_t sm[];
    MlpMisc<kSlots>& M = *reinterpret_cast<MlpMisc<kSlots>*>(sm + kSmMisc);
    const int slot = threadIdx.x / kSlotThreads, row = threadIdx.x % kSlotThreads;
    const int wq = row >> 5, lane = row & 31;  // warp within the slot = its TMEM lane quarter
    SlotMisc& S = M.slot[slot];
    static_assert(NS >= 0 && NS <= (int)kMaxSamples, "checked samples");
    constexpr int n_samples = NS;
    constexpr bool checking = NS > 0;
    float4* lights_dirI = reinterpret_cast<float4*>(sm + kSmLights);
    float2* lights_gb = reinterpret_cast<float2*>(sm + kSmLights + 16u * kMlpSmemLights);
    SmemLights table{lights_dirI, lights_gb};
    const bool staged = checking && a.nl <= kMlpSmemLights;
    const SmemLights* L = staged ? &table : nullptr;
    // the check table's bytes (dirI and gb of the rig's lights, each in whole 16-byte units)
    const uint32_t tab_dirI = staged ? 16u * (uint32_t)a.nl : 0u;
    const uint32_t tab_gb = staged ? 16u * (((uint32_t)a.nl + 1u) / 2u) : 0u;

    const uint32_t mbar_w = smem_addr(&M.mbar_w), mbar = smem_addr(&S.mbar);
    // The stall test's first MMA wait polls an mbarrier that nothing arrives on, briefly, and so
    // gives up as a wait for a lost MMA would; the MMA itself runs and completes.
    const uint32_t mbar_first = a.stall_test ? smem_addr(&M.mbar_idle) : mbar;
    const uint32_t tries_first = a.stall_test ? kStallTestTries : kWaitTries;
    if (threadIdx.x == 0) {
        M.sums[0] = M.sums[1] = M.sums[2] = 0ull;
        M.max_err_bits = 0u;
        mbar_init(mbar_w, 1);
        mbar_init(smem_addr(&M.mbar_idle), 1);
        for (int s = 0; s < kSlots; ++s) mbar_init(smem_addr(&M.slot[s].mbar), 1);
        // the weights and output scale, and the lights, arrive by bulk copy (independent of the
        // grid this kernel may overlap with)
        mbar_expect_tx(mbar_w, N::kImageBytes + tab_dirI + tab_gb);
        bulk_copy_g2s(smem_addr(sm), a.mlp, N::kImageBytes, mbar_w);
        if (staged) {
            const MlpCheckTable* tab = reinterpret_cast<const MlpCheckTable*>(a.mlp + N::kImageBytes);
            bulk_copy_g2s(smem_addr(lights_dirI), tab->dirI, tab_dirI, mbar_w);
            bulk_copy_g2s(smem_addr(lights_gb), tab->gb, tab_gb, mbar_w);
        }
    }
    if (row == 0) S.fail_mask = 0u;
    if (threadIdx.x < 32) tmem_alloc(smem_addr(&M.tmem), kTmemCols);
    // the records and the tile list are the previous kernel's output
    asm volatile("griddepcontrol.wait;" ::: "memory");

    // Slot g = blockIdx.x * kSlots + slot takes tiles g, g + stride, ...; this thread holds the
    // records of its row in the slot's current tile and the next one. The first two descriptors
    // are read with the list's header, not after it.
    const uint32_t stride = gridDim.x * kSlots;
    uint32_t t = blockIdx.x * kSlots + slot;
    uint32_t t_next = t + stride;
    const uint4 d_first = tile_desc_early(a, t), d_second = tile_desc_early(a, t_next);
    const uint32_t n_frag = a.index[0], n_tiles = a.index[1];
    uint32_t count = tile_count(n_frag, n_tiles, t);
    uint32_t count_next = tile_count(n_frag, n_tiles, t_next);
    float4 g0, g1, g0n, g1n;
    load_record_desc(a, t, count, d_first, row, g0, g1);
    load_record_desc(a, t_next, count_next, d_second, row, g0n, g1n);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = M.tmem;
    const uint32_t d_cols = tmem + (uint32_t)slot * kSlotTmem;  // lane 0, this slot's accumulators
    const uint32_t lane_off = (uint32_t)(wq * 32) << 16;         // this warp's lanes
    const uint32_t d_lane = d_cols + lane_off;
    const uint32_t a_f = d_cols + kSlotCols;  // lane 0 of the features' A operand
    const uint32_t a_h = a_f + kFCols;        // lane 0 of the hidden layers' A operand
    // the first tile's features, while the weights arrive
    if (t < n_tiles) store_features<N>(make_float3(g0.x, g0.y, g0.z), make_float3(g0.w, g1.x, g1.y), a_f + lane_off);
    a_written();
    bool failed = !__syncthreads_and(mbar_wait(mbar_w, 0));
    const bool weights_pending = failed;
    const float out_scale = *reinterpret_cast<const float*>(sm + Lay::kSmScale);
    const uint32_t sW1 = smem_addr(sm + Lay::kSmW1), sW2 = smem_addr(sm + Lay::kSmW2), sW3 = smem_addr(sm + Lay::kSmW3);

    // Every slot barrier of the loop also ORs the threads' timeout flags, so a slot's threads leave
    // the loop at the same barrier (the loop condition itself is the same in all of them).
    uint32_t phase = 0;
    uint32_t n_tile = 0, n_fallback = 0;
    float max_err = 0.f;
    uint32_t k = 0;  // tiles this slot shaded
    uint32_t kb = 0, t_batch = t;  // tiles in the check buffer, the first of them
    // Checks the buffered tiles and shades those that failed again, exactly (buffered tile j is
    // t0 + j * stride); every thread of the slot calls it after a slot barrier.
    auto check_buffer = [&](uint32_t n_buf, uint32_t t0) {
        if constexpr (checking) {
            check_rows<checking ? NS : 1>(a, L, S, (int)(n_buf * n_samples), wq, lane, max_err);
            slot_sync(slot);  // the marks are in
            const uint32_t f = S.fail_mask;
            slot_sync(slot);  // every thread read the verdicts before they are cleared
            if (row == 0) S.fail_mask = 0u;
            for (uint32_t m = f; m; m &= m - 1u) {
                if (row == 0) ++n_fallback;
                reshade_tile(a, t0 + (uint32_t)(__ffs(m) - 1) * stride, row);
            }
        }
    };
    // Layer L of the slot's tile k is issued by lane 0 of warp (k + L) mod 4: the issue holds its
    // warp for a few hundred cycles, and so falls on every warp (and scheduler) in turn.

    while (!weights_pending && t < n_tiles) {
        // the features are stored, the previous tile's accumulators read and its sampled rows
        // written, and tile k - 2's verdict is in
        if (slot_sync_or(slot, failed)) break;

        // layer 1: D = X (128 x K) * W1^T
        if (row == 32 * (int)((k + 1u) & 3u)) issue_layer(d_cols, a_f, sW1, N::kHid, N::kIn / 16, idesc_bf16(kMlpRows, N::kHid), mbar);
        // the slot's tile after next: its descriptor now, its records during layer 3
        const uint32_t t_nn = t_next + stride;
        const uint32_t count_nn = tile_count(n_frag, n_tiles, t_nn);
        const uint4 d_nn =
            (uint32_t)row < count_nn ? shade_tile_desc(a.index, a.n_blocks, t_nn) : make_uint4(0u, 0u, 0u, 0u);
        // the checked samples this row is (two samples may fall on one row)
        uint32_t my_samples = 0u;
        if constexpr (checking) {
            const uint32_t h_t = sample_hash(t);
#pragma unroll
            for (int s = 0; s < n_samples; ++s)
                if (sample_rank(h_t, s, count) == (uint32_t)row) my_samples |= 1u << s;
        }
        // After a wait gave up (`failed`), a warp touches tensor memory no more: an MMA may still
        // be using it. The test is warp-uniform, as the .sync.aligned tcgen05 instructions need.
        failed |= !mbar_wait(mbar_first, phase, tries_first);
        phase ^= 1u;
        tc_fence_after();
        if (!__any_sync(kFull, failed)) hidden_epilogue<N>(d_lane, a_h + lane_off);  // h1
        a_written();
        if (slot_sync_or(slot, failed)) break;

        // layer 2: D = H1 (128 x H) * W2^T
        if (row == 32 * (int)((k + 2u) & 3u)) issue_layer(d_cols, a_h, sW2, N::kHid, N::kHid / 16, idesc_bf16(kMlpRows, N::kHid), mbar);
        failed |= !mbar_wait(mbar, phase);
        phase ^= 1u;
        tc_fence_after();
        if (!__any_sync(kFull, failed)) hidden_epilogue<N>(d_lane, a_h + lane_off);  // h2 over h1 (layer 2 has read it)
        a_written();
        if (slot_sync_or(slot, failed)) break;

        // layer 3: D[0, 16) = H2 (128 x H) * W3^T; meanwhile the next tile's features go over this
        // tile's (layer 1 has read them)
        if (row == 32 * (int)((k + 3u) & 3u)) issue_layer(d_cols, a_h, sW3, kMlpOutPad, N::kHid / 16, idesc_bf16(kMlpRows, kMlpOutPad), mbar);
        if (t_next < n_tiles && !__any_sync(kFull, failed))
            store_features<N>(make_float3(g0n.x, g0n.y, g0n.z), make_float3(g0n.w, g1n.x, g1n.y), a_f + lane_off);
        float4 g0nn, g1nn;
        load_record_desc(a, t_nn, count_nn, d_nn, row, g0nn, g1nn);
        failed |= !mbar_wait(mbar, phase);
        phase ^= 1u;
        tc_fence_after();
        uint32_t o[4] = {0u, 0u, 0u, 0u};
        if (!__any_sync(kFull, failed)) {
            tmem_ld4(d_lane, o);
            tmem_wait4(o);
        }
        a_written();

        const float3 alb = make_float3(g0.w, g1.x, g1.y);
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
            for (uint32_t m = my_samples; m; m &= m - 1u) {  // every sampled row of the tile is written once
                CheckRow& q = S.q[kb][__ffs(m) - 1];
                q.n[0] = g0.x; q.n[1] = g0.y; q.n[2] = g0.z;
                q.alb[0] = alb.x; q.alb[1] = alb.y; q.alb[2] = alb.z;
                q.rad[0] = radc.x; q.rad[1] = radc.y; q.rad[2] = radc.z;
                q.valid = valid ? 1u : 0u;
            }
            ++n_tile;
            if constexpr (checking)
                if (++kb == kCheckTiles) {  // the same in every thread of the slot
                    if (slot_sync_or(slot, failed)) break;
                    check_buffer(kb, t_batch);
                    kb = 0u;
                    t_batch = t_next;
                }
        }
        ++k;
        t = t_next;
        count = count_next;
        g0 = g0n;
        g1 = g1n;
        t_next = t_nn;
        count_next = count_nn;
        g0n = g0nn;
        g1n = g1nn;
    }

    // the rest of the check buffer (every thread of the slot reaches this barrier: the loop ends
    // at the same point in all of them, and it orders the buffer's rows before the check)
    if (!slot_sync_or(slot, failed) && checking && !weights_pending && kb > 0u) check_buffer(kb, t_batch);

    if (failed) {
        // the weights' copy or an MMA did not complete in time: record it, give the pending one
        // another bounded wait, then release the tensor memory
        if (row == 0) atomicOr(&a.counters[1], STATUS_SHADE_TIMEOUT);
        if (weights_pending) mbar_wait(mbar_w, 0);
        else mbar_wait(mbar, phase ^ 1u);
    }
    // the statistics, summed in the CTA first: one global atomic per counter and CTA (thousands on
    // one address would hold the grid's completion, which the next pass waits for)
    const bool stats = a.stats && !a.eval_out;
    if (stats) {
        if (row == 0 && n_tile) {
            atomicAdd(&M.sums[0], (unsigned long long)n_tile);
            if (n_fallback) atomicAdd(&M.sums[1], (unsigned long long)n_fallback);
            atomicAdd(&M.sums[2], (unsigned long long)n_tile * (unsigned long long)n_samples);
        }
        const uint32_t e = __reduce_max_sync(kFull, __float_as_uint(max_err));  // max_err >= 0
        if (lane == 0 && e) atomicMax(&M.max_err_bits, e);
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
    if (stats && threadIdx.x == 0) {
        if (M.sums[0]) atomicAdd(a.stats + 0, M.sums[0]);
        if (M.sums[1]) atomicAdd(a.stats + 1, M.sums[1]);
        if (M.sums[2]) atomicAdd(a.stats + 2, M.sums[2]);
        if (M.max_err_bits) atomicMax(a.stats + 3, (unsigned long long)M.max_err_bits);
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
// The training step's layout for network N. Thread tid works on unit j = tid % H for group
// tid / H of the samples (forward, dH) or of the inputs (weight gradients).
template <class N>
struct TrainLayout {
    static constexpr int kSX = N::kIn + 4;   // shared row stride (floats) of X and W1: rows stay 16-byte
    static constexpr int kSH = N::kHid + 4;  // aligned and eight rows cover all banks; of H, D and W2
    static constexpr int kGroups = kTrainThreads / N::kHid;
    static constexpr int kSPG = kTrainB / kGroups;     // samples per group
    static constexpr int kHPG = N::kHid / kGroups;     // hidden inputs per group (layer 2 gradients)
    static constexpr int kXPG = N::kIn / kGroups;      // features per group (layer 1 gradients)
    static_assert(kTrainThreads % N::kHid == 0 && kTrainB % kGroups == 0 && kHPG % 4 == 0 && kXPG % 4 == 0 &&
                      N::kIn % 4 == 0 && kTrainB * kMlpOut <= kTrainThreads && kMlpOut * N::kHid <= kTrainThreads,
                  "training thread layout");
};

template <class N>
struct TrainSmem {
    static constexpr int kSX = TrainLayout<N>::kSX, kSH = TrainLayout<N>::kSH;
    float w1[N::kHid * kSX];
    float w2[N::kHid * kSH];
    float w3[kMlpOut * N::kHid];
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
    float* grad;             // per CTA, one partial gradient per parameter of the network
    float* loss;             // per CTA partial sum of squared errors
};

// One step's forward and backward pass for kTrainB samples per CTA, in FP32 with the rounding of the
// tensor-core kernel (BF16 features, weights and hidden activations); per-CTA partial gradients.
template <class N>
__global__ void __launch_bounds__(kTrainThreads) k_mlp_train(TrainArgs a) {
    using TL = TrainLayout<N>;
    constexpr int kSX = TL::kSX, kSH = TL::kSH, kSPG = TL::kSPG, kHPG = TL::kHPG, kXPG = TL::kXPG;
    // the network's sizes under the names the step's loops use
    constexpr int kMlpIn = N::kIn, kMlpHid = N::kHid, kPW1 = N::kPW1, kPW2 = N::kPW2, kPW3 = N::kPW3;
    constexpr int kMlpParams = N::kParams;
    extern __shared__ __align__(16) uint8_t smraw[];
    TrainSmem<N>& S = *reinterpret_cast<TrainSmem<N>*>(smraw);
    const int tid = threadIdx.x;
    for (int i = tid; i < kMlpHid * kMlpIn; i += kTrainThreads) S.w1[(i / kMlpIn) * kSX + i % kMlpIn] = a.q[kPW1 + i];
    for (int i = tid; i < kMlpHid * kMlpHid; i += kTrainThreads) S.w2[(i / kMlpHid) * kSH + i % kMlpHid] = a.q[kPW2 + i];
    for (int i = tid; i < kMlpOut * kMlpHid; i += kTrainThreads) S.w3[i] = a.q[kPW3 + i];
    if (tid < kTrainB) {
        const int64_t i = (a.first + (int64_t)blockIdx.x * kTrainB + tid) % a.n;
        const float* s = a.samples + 9 * i;
        const float3 nv = make_float3(s[0], s[1], s[2]), alb = make_float3(s[3], s[4], s[5]);
        uint32_t pairs[kMlpIn / 2];
        mlp_feature_pairs<N>(nv, alb, pairs);
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

    const int j = tid % kMlpHid, q4 = tid / kMlpHid;  // unit j, group q4 of the samples / inputs
    // forward, layer 1: kSPG samples of unit j
    {
        float acc[kSPG];
#pragma unroll
        for (int bb = 0; bb < kSPG; ++bb) acc[bb] = 0.f;
        for (int k = 0; k < kMlpIn; k += 4) {
            const float4 w = *reinterpret_cast<const float4*>(S.w1 + j * kSX + k);
#pragma unroll
            for (int bb = 0; bb < kSPG; ++bb) {
                const float4 x = *reinterpret_cast<const float4*>(S.x + (kSPG * q4 + bb) * kSX + k);
                acc[bb] = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, fmaf(w.w, x.w, acc[bb]))));
            }
        }
#pragma unroll
        for (int bb = 0; bb < kSPG; ++bb) S.h1[(kSPG * q4 + bb) * kSH + j] = bf16_round(fmaxf(acc[bb], 0.f));
    }
    __syncthreads();
    // layer 2
    {
        float acc[kSPG];
#pragma unroll
        for (int bb = 0; bb < kSPG; ++bb) acc[bb] = 0.f;
        for (int k = 0; k < kMlpHid; k += 4) {
            const float4 w = *reinterpret_cast<const float4*>(S.w2 + j * kSH + k);
#pragma unroll
            for (int bb = 0; bb < kSPG; ++bb) {
                const float4 x = *reinterpret_cast<const float4*>(S.h1 + (kSPG * q4 + bb) * kSH + k);
                acc[bb] = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, fmaf(w.w, x.w, acc[bb]))));
            }
        }
#pragma unroll
        for (int bb = 0; bb < kSPG; ++bb) S.h2[(kSPG * q4 + bb) * kSH + j] = bf16_round(fmaxf(acc[bb], 0.f));
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
    for (int bb = 0; bb < kSPG; ++bb) {
        const int b = kSPG * q4 + bb;
        float v = 0.f;
#pragma unroll
        for (int c = 0; c < kMlpOut; ++c) v = fmaf(S.w3[c * kMlpHid + j], S.y[4 * b + c], v);
        S.d2[b * kSH + j] = S.h2[b * kSH + j] > 0.f ? v : 0.f;
    }
    __syncthreads();
    // layer 2 gradients (unit j, inputs kHPG*q4..) and dH1 (input unit j, samples kSPG*q4..)
    {
        float acc[kHPG];
#pragma unroll
        for (int ii = 0; ii < kHPG; ++ii) acc[ii] = 0.f;
        for (int b = 0; b < kTrainB; ++b) {
            const float d = S.d2[b * kSH + j];
#pragma unroll
            for (int ii = 0; ii < kHPG; ii += 4) {
                const float4 h = *reinterpret_cast<const float4*>(S.h1 + b * kSH + kHPG * q4 + ii);
                acc[ii] = fmaf(d, h.x, acc[ii]);
                acc[ii + 1] = fmaf(d, h.y, acc[ii + 1]);
                acc[ii + 2] = fmaf(d, h.z, acc[ii + 2]);
                acc[ii + 3] = fmaf(d, h.w, acc[ii + 3]);
            }
        }
#pragma unroll
        for (int ii = 0; ii < kHPG; ++ii) g[kPW2 + j * kMlpHid + kHPG * q4 + ii] = acc[ii];
        float dh[kSPG];
#pragma unroll
        for (int bb = 0; bb < kSPG; ++bb) dh[bb] = 0.f;
        for (int u = 0; u < kMlpHid; ++u) {
            const float w = S.w2[u * kSH + j];
#pragma unroll
            for (int bb = 0; bb < kSPG; ++bb) dh[bb] = fmaf(w, S.d2[(kSPG * q4 + bb) * kSH + u], dh[bb]);
        }
#pragma unroll
        for (int bb = 0; bb < kSPG; ++bb) {
            const int b = kSPG * q4 + bb;
            S.d1[b * kSH + j] = S.h1[b * kSH + j] > 0.f ? dh[bb] : 0.f;
        }
    }
    __syncthreads();
    // layer 1 gradients: unit j, inputs kQ*q4 .. kQ*q4 + kQ - 1
    {
        constexpr int kQ = kXPG;
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

template <class N>
__global__ void k_mlp_adam(AdamArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && a.loss_out) {
        float s = 0.f;
        for (int i = 0; i < a.n_part; ++i) s += a.loss_part[i];
        *a.loss_out = s;
    }
    if (p >= N::kParams || N::fixed(p)) return;
    float gs = 0.f;
    for (int i = 0; i < a.n_part; ++i) gs += a.grad[(size_t)i * N::kParams + p];
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
    a.mlp = static_cast<const uint8_t*>(p.mlp);
    a.samples = p.mlp_samples;
    a.bound = p.mlp_bound;
    a.stats = s.shade_stats;
    a.eval_out = nullptr;
    a.stall_test = p.mlp_stall_test ? 1u : 0u;
    return a;
}

// Network N's learned-shader kernel for a number of checked samples per tile (0 .. kMaxSamples).
using MlpKernel = void (*)(ShadeArgs);
template <class N>
static MlpKernel mlp_kernel(int samples) {
    static const MlpKernel k[kMaxSamples + 1] = {k_shade_mlp<N, 0>, k_shade_mlp<N, 1>, k_shade_mlp<N, 2>,
                                                 k_shade_mlp<N, 3>, k_shade_mlp<N, 4>};
    return k[std::min(std::max(samples, 0), (int)kMaxSamples)];
}

template <class N>
static int mlp_grid(int n_sm, int64_t blocks) {
    static bool attr_set = false;  // per process: the attribute is per function, all devices alike
    if (!attr_set) {
        for (int ns = 0; ns <= (int)kMaxSamples; ++ns)
            if (cudaFuncSetAttribute(mlp_kernel<N>(ns), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)MlpLayout<N>::kSmem) != cudaSuccess ||
                cudaFuncSetAttribute(mlp_kernel<N>(ns), cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
                return -1;
        attr_set = true;
    }
    // one CTA per SM at most, and no more CTAs than the tiles need (a block of 1024 records makes
    // at most 8 tiles)
    constexpr int kSlots = MlpLayout<N>::kSlots;
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
        err = with_mlp_net(p.mlp_net, [&](auto n) {
            using N = decltype(n);
            const int grid = mlp_grid<N>(p.n_sm, blocks);
            if (grid < 0) return cudaErrorInvalidConfiguration;
            return launch_dependent(mlp_kernel<N>(a.samples), grid, MlpLayout<N>::kThreads, MlpLayout<N>::kSmem,
                                    stream, a);
        });
    }
    return err == cudaSuccess ? 1 : -1;
}

int launch_mlp_eval(int net, const float* src, int stride, int64_t n, bool exact, float4* gbuf, uint32_t* count,
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
    a.mlp = static_cast<const uint8_t*>(mlp);
    a.samples = 0;
    a.bound = 0.f;
    a.stats = nullptr;
    a.eval_out = out;
    a.stall_test = 0u;
    if (exact) {
        k_shade_exact<<<exact_grid(n_sm, blocks), kExactThreads, 0, stream>>>(a);
    } else {
        const int grid = with_mlp_net(net, [&](auto m) {
            using N = decltype(m);
            const int g = mlp_grid<N>(n_sm, blocks);
            if (g > 0) k_shade_mlp<N, 0><<<g, MlpLayout<N>::kThreads, MlpLayout<N>::kSmem, stream>>>(a);
            return g;
        });
        if (grid < 0) return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 3 : -1;
}

int launch_mlp_samples(float* out, int64_t n, uint64_t seed, const float* lights, int nl, cudaStream_t stream) {
    if (n <= 0) return 0;
    k_mlp_samples<<<grid_for(n, 256), 256, 0, stream>>>(out, n, seed, lights, nl);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

template <class N>
static bool train_attr() {
    static bool attr_set = false;  // per process: the attribute is per function
    if (!attr_set)
        attr_set = cudaFuncSetAttribute(k_mlp_train<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sizeof(TrainSmem<N>)) == cudaSuccess;
    return attr_set;
}

int launch_mlp_train_step(int net, const float* q, const float* samples, int64_t n, int64_t first, int n_cta,
                          float out_scale, float grad_scale, float* grad, float* loss, cudaStream_t stream) {
    TrainArgs a;
    a.q = q;
    a.samples = samples;
    a.n = n;
    a.first = first;
    a.out_scale = out_scale;
    a.grad_scale = grad_scale;
    a.grad = grad;
    a.loss = loss;
    const bool ok = with_mlp_net(net, [&](auto m) {
        using N = decltype(m);
        if (!train_attr<N>()) return false;
        k_mlp_train<N><<<n_cta, kTrainThreads, sizeof(TrainSmem<N>), stream>>>(a);
        return true;
    });
    return ok && cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int launch_mlp_adam(int net, float* w, float* q, float* m, float* v, const float* grad, int n_part, float lr,
                    float beta1, float beta2, float eps, float c1, float c2, const float* loss_part, float* loss_out,
                    cudaStream_t stream) {
    AdamArgs a;
    a.w = w; a.q = q; a.m = m; a.v = v; a.grad = grad; a.n_part = n_part;
    a.lr = lr; a.beta1 = beta1; a.beta2 = beta2; a.eps = eps; a.c1 = c1; a.c2 = c2;
    a.loss_part = loss_part;
    a.loss_out = loss_out;
    with_mlp_net(net, [&](auto n) {
        using N = decltype(n);
        k_mlp_adam<N><<<grid_for(N::kParams, 256), 256, 0, stream>>>(a);
        return 0;
    });
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int train_batch_per_cta() { return kTrainB; }

}  // namespace rast
