// Kernels of the per-frame rasteriser path for sm_103a (GB300).
//
// Parity contract: coverage, depth and the winning triangle of every pixel are bit for bit those
// of canmom/rasteriser's draw_frame (drawing.cpp:205-258). Every floating-point step that decides
// them is one IEEE round-to-nearest operation in the reference's order, written with __f*_rn
// intrinsics (never contracted into FMA), and the file is built with -fmad=false besides.
//
// Pipeline of one frame:
//   k_vertex        transform_vertices + z_divide_all + ndc_to_raster_all (geometry.cpp:85-142);
//                   also clears the frame's counters and statistics
//   k_setup_raster  per triangle: de-index, signed_area_2d cull, bounding_box (drawing.cpp:77-93,
//                   160-188); triangles with small boxes are rasterised here by their warp, the
//                   rest are appended to the binned list and counted into 16x16 (8/32) tiles
//   k_bin_scan      exclusive scans of the tile counts and of the tile work items
//   k_bin_scatter   binned triangles into per-tile lists
//   k_tile_raster   persistent CTAs take (tile, up to 64 binned triangles) work items; each thread
//                   owns pixels of the tile and keeps their minimum keys in registers; warp
//                   ballots give the coverage masks and skip triangles that miss a warp's block
//   k_resolve       per pixel: decode the winner (read-modify-write: test it against the incoming
//                   depth), recompute its barycentrics, perspective-correct normal, Lambert
//                   shading over the lights (shading.cpp:20-34), planar RGB8 + depth writes; re-arms
//                   the keys for the next frame
//
// Depth test: the reference keeps a fragment when `ndcdepth < depth(x,y)` while walking the
// triangles in order (drawing.cpp:119), so a pixel ends with the smallest depth and, among equal
// depths, the earliest triangle, provided that depth beats the incoming one. Here every fragment
// proposes the 64-bit key (order(depth) << 32 | triangle) and the pixel keeps the minimum, which
// is the same fragment whatever order the fragments arrive in. In clear mode the keys start at the
// key of the cleared depth 1.0, so only nearer fragments can land. In read-modify-write mode they
// start above every fragment, and the resolve pass keeps the nearest fragment when its depth is
// below the incoming one: it passes the reference's sequence of tests exactly when any fragment
// does.
#include <cstdint>
#include <cuda_runtime.h>
#include <utility>

#include "rast_exact.cuh"
#include "rast_internal.h"
#include "rast_tiles.cuh"

namespace rast {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned long long kNoWinner = 0xFFFFFFFFull;  // low word of a key with no fragment
constexpr unsigned long long kArmed = ~0ull;             // read-modify-write: a key before any fragment

// Row r of mat4 * vec4, summed (c0*x + c1*y) + (c2*z + c3*w).
__device__ __forceinline__ float mrow(const Mat4& M, int r, float x, float y, float z, float w) {
    const float lo = add(mul(M.m[r], x), mul(M.m[4 + r], y));
    const float hi = add(mul(M.m[8 + r], z), mul(M.m[12 + r], w));
    return add(lo, hi);
}

// Total order on non-NaN floats that matches `<`, with -0 and +0 equal.
__device__ __forceinline__ uint32_t depth_order(float z) {
    uint32_t u = __float_as_uint(z);
    u = (u == 0x80000000u) ? 0u : u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Clear mode: the key a fragment (z, t) beats exactly when z < 1.0 (the cleared depth).
__device__ __forceinline__ unsigned long long clear_key() {
    return (static_cast<unsigned long long>(depth_order(1.0f)) << 32) - 1ull;
}

__device__ __forceinline__ unsigned long long frag_key(float z, uint32_t tri) {
    return (static_cast<unsigned long long>(depth_order(z)) << 32) | tri;
}

// Edge-function data of one triangle (drawing.cpp:36-49): the vertex deltas are the same
// subtractions the reference repeats for every pixel, taken once.
struct EdgeTri {
    float x0, y0, x1, y1, x2, y2;
    float d12x, d12y, d20x, d20y, d01x, d01y;
    float z0, z1, z2, area, nthr, sgn;
};

__device__ __forceinline__ void make_edge_tri(float4 a, float4 b, float4 c, EdgeTri& T) {
    T.x0 = a.x; T.y0 = a.y; T.x1 = b.x; T.y1 = b.y; T.x2 = c.x; T.y2 = c.y;
    T.z0 = a.z; T.z1 = b.z; T.z2 = c.z;
    T.d12x = sub(c.x, b.x); T.d12y = sub(c.y, b.y);
    T.d20x = sub(a.x, c.x); T.d20y = sub(a.y, c.y);
    T.d01x = sub(b.x, a.x); T.d01y = sub(b.y, a.y);
    // area = edge(v2, v0, v1) = (v1.x-v0.x)*(v2.y-v0.y) - (v1.y-v0.y)*(v2.x-v0.x)
    T.area = sub(mul(T.d01x, sub(c.y, a.y)), mul(T.d01y, sub(c.x, a.x)));
    // Early reject: when |area| is a normal number >= 2^-26, an edge value e with
    // sgn(area)*e < -|area|*2^-100 gives e/area <= -2^-100 after rounding, so that barycentric is
    // negative and the pixel is outside; such pixels skip the three divisions. Every other pixel
    // takes the reference's divisions. The bound is exact (a power-of-two scale of a normal).
    const float aa = fabsf(T.area);
    if (aa >= 0x1p-26f && aa < __int_as_float(0x7f800000)) {
        T.nthr = -mul(aa, 0x1p-100f);
        T.sgn = T.area > 0.f ? 1.f : -1.f;
    } else {
        T.nthr = __int_as_float(0xff800000);  // -inf: never rejects early
        T.sgn = 1.f;
    }
}

// update_pixel's barycentric and inside test (drawing.cpp:108-111) at integer pixel (px, py).
__device__ __forceinline__ bool inside_test(const EdgeTri& T, float px, float py, float& b0, float& b1,
                                            float& b2) {
    const float e0 = sub(mul(T.d12x, sub(py, T.y1)), mul(T.d12y, sub(px, T.x1)));
    const float e1 = sub(mul(T.d20x, sub(py, T.y2)), mul(T.d20y, sub(px, T.x2)));
    const float e2 = sub(mul(T.d01x, sub(py, T.y0)), mul(T.d01y, sub(px, T.x0)));
    if (mul(T.sgn, e0) < T.nthr || mul(T.sgn, e1) < T.nthr || mul(T.sgn, e2) < T.nthr) return false;
    b0 = dvd(e0, T.area);
    b1 = dvd(e1, T.area);
    b2 = dvd(e2, T.area);
    return b0 >= 0.f && b1 >= 0.f && b2 >= 0.f;
}

// screen_interpolate of the NDC depths (drawing.cpp:51-56, 115-116).
__device__ __forceinline__ float interp_depth(const EdgeTri& T, float b0, float b1, float b2) {
    return add(add(mul(T.z0, b0), mul(T.z1, b1)), mul(T.z2, b2));
}

// bounding_box (drawing.cpp:77-93): truncated clamp of the min corner, clamp of the ceiled max
// corner, both to [0, W-1] x [0, H-1].
__device__ __forceinline__ void bounding_box(float4 a, float4 b, float4 c, float lim_x, float lim_y,
                                             uint32_t& tlx, uint32_t& tly, uint32_t& brx, uint32_t& bry) {
    const float mnx = gmin(gmin(a.x, b.x), c.x), mny = gmin(gmin(a.y, b.y), c.y);
    const float mxx = gmax(gmax(a.x, b.x), c.x), mxy = gmax(gmax(a.y, b.y), c.y);
    tlx = __float2uint_rz(gmin(gmax(mnx, 0.f), lim_x));
    tly = __float2uint_rz(gmin(gmax(mny, 0.f), lim_y));
    brx = __float2uint_rz(gmin(gmax(ceilf(mxx), 0.f), lim_x));
    bry = __float2uint_rz(gmin(gmax(ceilf(mxy), 0.f), lim_y));
}

// signed_area_2d (geometry.cpp:76-83), summed left to right, and the culling rule
// (drawing.cpp:176-178).
__device__ __forceinline__ bool front_facing(float4 a, float4 b, float4 c, bool cw) {
    float s = mul(a.x, b.y);
    s = sub(s, mul(b.x, a.y));
    s = add(s, mul(b.x, c.y));
    s = sub(s, mul(c.x, b.y));
    s = add(s, mul(c.x, a.y));
    s = sub(s, mul(a.x, c.y));
    const float sa = mul(-0.5f, s);
    return (sa > 0.f) != cw;
}

// transform_direction with the normal matrix (geometry.cpp:35-42, 97-108).
__device__ __forceinline__ float3 camera_normal(const Mat4& M, float x, float y, float z) {
    return make_float3(mrow(M, 0, x, y, z, 0.f), mrow(M, 1, x, y, z, 0.f), mrow(M, 2, x, y, z, 0.f));
}

// The face normal of flat shading (the reference's --flat, readme.md:46): cross(p1 - p0, p2 - p0)
// of the model-space positions, not normalised (the path normalises after interpolation), with
// cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y).
__device__ __forceinline__ float3 face_normal(const float* pos, int32_t i0, int32_t i1, int32_t i2) {
    const float* P0 = pos + 3 * (int64_t)i0;
    const float* P1 = pos + 3 * (int64_t)i1;
    const float* P2 = pos + 3 * (int64_t)i2;
    const float ax = sub(__ldg(P1), __ldg(P0)), ay = sub(__ldg(P1 + 1), __ldg(P0 + 1)), az = sub(__ldg(P1 + 2), __ldg(P0 + 2));
    const float bx = sub(__ldg(P2), __ldg(P0)), by = sub(__ldg(P2 + 1), __ldg(P0 + 1)), bz = sub(__ldg(P2 + 2), __ldg(P0 + 2));
    return make_float3(sub(mul(ay, bz), mul(by, az)), sub(mul(az, bx), mul(bz, ax)), sub(mul(ax, by), mul(bx, ay)));
}

// ---------------------------------------------------------------------------------------------
// warp and bookkeeping helpers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t n = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Programmatic dependent launch: the kernels of a frame after the first are launched while their
// predecessor runs; each lets its dependents launch as it starts, and waits for its predecessor
// (and so for every earlier kernel of the frame) before anything else.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Records a failed internal check: sets STATUS_CHECK_FAILED and keeps the first failure's code
// and detail in counters[2..3]. The caller skips the access that failed the check.
__device__ __noinline__ void report(uint32_t* counters, uint32_t code, uint32_t detail) {
    atomicOr(&counters[1], STATUS_CHECK_FAILED);
    if (atomicCAS(&counters[2], 0u, code) == 0u) atomicExch(&counters[3], detail);
}

// Adds the warp's sum of v to statistics counter `which`, in the slot of this warp. Must be
// called by all 32 lanes.
__device__ __forceinline__ void stat_add(unsigned long long* stats, int which, unsigned long long v) {
    v = warp_sum64(v);
    if ((threadIdx.x & 31) == 0 && v) {
        const uint32_t warp_id = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) + blockIdx.y * 977u;
        atomicAdd(stats + ((size_t)which * kStatSlots + (warp_id % kStatSlots)) * kSlotWords, v);
    }
}

// The same for a 32-bit count whose warp sum fits in 32 bits (one warp reduction instruction).
__device__ __forceinline__ void stat_add32(unsigned long long* stats, int which, uint32_t v) {
    v = __reduce_add_sync(kFull, v);
    if ((threadIdx.x & 31) == 0 && v) {
        const uint32_t warp_id = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) + blockIdx.y * 977u;
        atomicAdd(stats + ((size_t)which * kStatSlots + (warp_id % kStatSlots)) * kSlotWords, (unsigned long long)v);
    }
}

__device__ __forceinline__ unsigned long long* stat_slot0(unsigned long long* stats, int which) {
    return stats + (size_t)which * kStatSlots * kSlotWords;
}

// First lane j whose inclusive prefix exceeds k (the owner of work item k).
__device__ __forceinline__ int owner_of(const uint32_t* incl, uint32_t k) {
    int lo = 0, hi = 31;
#pragma unroll
    for (int it = 0; it < 5; ++it) {
        const int mid = (lo + hi) >> 1;
        if (incl[mid] > k) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// q = n / d for n <= 2^24, d >= 1: a float-reciprocal estimate (within 2 of the quotient at
// that range) corrected to the exact quotient.
__device__ __forceinline__ uint32_t div_small(uint32_t n, uint32_t d, float rd) {
    uint32_t q = __float2uint_rz(__fmul_rn(__uint2float_rn(n), rd));
    while (q > 0u && q * d > n) --q;
    while ((q + 1u) * d <= n) ++q;
    return q;
}

// ---------------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------------

// The frame's per-draw clears, done by its first kernel: counters (bins, status) and statistics.
struct FrameClear {
    uint32_t* words;
    uint32_t n_words;
    unsigned long long* stats;
    uint32_t n_stats;
    unsigned long long* shade_stats;
    uint32_t n_shade_stats;
};

__device__ __forceinline__ void frame_clear(const FrameClear& c) {
    const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x, step = gridDim.x * blockDim.x;
    for (uint32_t i = i0; i < c.n_words; i += step) c.words[i] = 0u;
    for (uint32_t i = i0; i < c.n_stats; i += step) c.stats[i] = 0ull;
    for (uint32_t i = i0; i < c.n_shade_stats; i += step) c.shade_stats[i] = 0ull;
}

// Vertex stage: clip = camera * (x, y, z, 1); (x/w, y/w, z/w, 1/w); x, y to raster pixels with
// the y flip (geometry.cpp:44-74).
__global__ void __launch_bounds__(256) k_vertex(const float* __restrict__ pos, int64_t nv, Mat4 cam, float wf,
                                                float hf, float4* __restrict__ rv, FrameClear clr) {
    pdl_launch_dependents();
    frame_clear(clr);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        const float cx = mrow(cam, 0, x, y, z, 1.f);
        const float cy = mrow(cam, 1, x, y, z, 1.f);
        const float cz = mrow(cam, 2, x, y, z, 1.f);
        const float cw = mrow(cam, 3, x, y, z, 1.f);
        const float nx = dvd(cx, cw), ny = dvd(cy, cw), nz = dvd(cz, cw), iw = dvd(1.f, cw);
        const float X = mul(mul(0.5f, add(nx, 1.0f)), wf);
        const float Y = mul(mul(0.5f, add(-ny, 1.0f)), hf);
        rv[i] = make_float4(X, Y, nz, iw);
    }
}

__device__ __forceinline__ float4 raster_vertex(const Mat4& cam, float x, float y, float z, float wf, float hf) {
    const float cx = mrow(cam, 0, x, y, z, 1.f);
    const float cy = mrow(cam, 1, x, y, z, 1.f);
    const float cz = mrow(cam, 2, x, y, z, 1.f);
    const float cw = mrow(cam, 3, x, y, z, 1.f);
    const float nx = dvd(cx, cw), ny = dvd(cy, cw), nz = dvd(cz, cw), iw = dvd(1.f, cw);
    return make_float4(mul(mul(0.5f, add(nx, 1.0f)), wf), mul(mul(0.5f, add(-ny, 1.0f)), hf), nz, iw);
}

// The same for four consecutive vertices per thread, read as three 16-byte loads (positions must
// be 16-byte aligned); the last nv % 4 vertices are done one by one.
__global__ void __launch_bounds__(256) k_vertex4(const float* __restrict__ pos, int64_t nv, Mat4 cam, float wf,
                                                 float hf, float4* __restrict__ rv, FrameClear clr) {
    pdl_launch_dependents();
    frame_clear(clr);
    const int64_t groups = nv / 4;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups + (nv % 4); g += (int64_t)gridDim.x * blockDim.x) {
        if (g < groups) {
            const float4* q = reinterpret_cast<const float4*>(pos) + 3 * g;
            const float4 a = q[0], b = q[1], c = q[2];
            float4* o = rv + 4 * g;
            o[0] = raster_vertex(cam, a.x, a.y, a.z, wf, hf);
            o[1] = raster_vertex(cam, a.w, b.x, b.y, wf, hf);
            o[2] = raster_vertex(cam, b.z, b.w, c.x, wf, hf);
            o[3] = raster_vertex(cam, c.y, c.z, c.w, wf, hf);
        } else {
            const int64_t i = 4 * groups + (g - groups);
            rv[i] = raster_vertex(cam, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], wf, hf);
        }
    }
}

__global__ void __launch_bounds__(256) k_arm_keys(unsigned long long* __restrict__ keys, int64_t n, bool clear) {
    const unsigned long long v = clear ? clear_key() : kArmed;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        keys[i] = v;
}

__global__ void __launch_bounds__(256) k_split_triangles(const int32_t* __restrict__ tris10, int64_t ntri,
                                                         int32_t* __restrict__ tri_v, int4* __restrict__ tri_nm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ntri; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t* t = tris10 + 10 * i;
        tri_v[3 * i] = t[0];
        tri_v[3 * i + 1] = t[1];
        tri_v[3 * i + 2] = t[2];
        tri_nm[i] = make_int4(t[3], t[4], t[5], t[9]);
    }
}

constexpr int kSetupThreads = 128;
constexpr int kSetupWarps = kSetupThreads / 32;
// Bounding boxes at most this many pixels wide take the per-triangle path; wider ones are binned.
// Whole-row items cost the same whatever their length and run along the box's longer side, so for
// them the limit is on the shorter side.
template <uint32_t kRowChunk>
__host__ __device__ constexpr uint32_t small_max_row() { return kRowChunk == 32u ? 64u : 32u; }

// Per-warp staging of 32 triangles. rec[j] holds lane j's triangle as five float4s so a lane
// working on another lane's triangle loads it with 16-byte shared loads:
//   rec[j][k] = U_k V_k W_k Z_k  (k = 0, 1, 2: edge k)   rec[j][3] = R_0 R_1 R_2 nthr
//   rec[j][4] = z0 z1 z2 |area|
// Edge k's value at the pixel with coordinate t along the item and `fixed` across it is
//   f_k = U_k * (fixed - V_k) - W_k * (t - Z_k),
// which is sgn(area) times the reference's edge function (drawing.cpp:36-39) bit for bit: for items
// along rows (t = px, fixed = py) U, V, W, Z = A, Y, B, X; along columns (t = py, fixed = px)
// U, V, W, Z = -B, X, -A, Y, where A = sgn * (b.x - a.x), B = sgn * (b.y - a.y) and (X, Y) is the
// edge's first vertex. Negating a product's factor negates the rounded product, and
// -p - (-q) = q - p exactly, so both give the same rounded f. R_k ~ 1/W_k (whole-row items only).
// The integer data (item range along, first item across and flags, items per row) is kept in
// integer arrays.
struct SetupStage {
    float4 rec[32][5];
    uint32_t tlx[32], tly[32], brx[32], cpr[32];
    float rcpr[32];
    uint32_t incl[32];
    int slot[32];
    // Ring of candidate runs (pixels of one item the early reject could not rule out): first pixel
    // (t | fixed << 16), owning lane with the column flag in bit 5, and the run's length.
    uint32_t q_tf[64], q_om[64], q_m[64];
};

struct SetupArgs {
    const int32_t* tri_v;
    const float4* rv;
    int64_t ntri;
    float lim_x, lim_y;
    uint32_t width, height;
    uint32_t small_max;
    uint32_t tile_shift;
    uint32_t tiles_x, n_tiles;
    bool cw;
    unsigned long long* keys;
    BinnedTri* large;
    int64_t cap_large;
    uint32_t* counters;
    unsigned long long* stats;
};

// One thread per triangle: load, cull and bound it. Front-facing triangles whose bounding box is
// at most small_max pixels, and at most small_max_row() pixels on its shorter side (whole items) or
// wide (row chunks), are rasterised by their warp; the others are appended to the binned list (one
// atomic per warp) and counted into the tiles their box overlaps.
//
// The warp's raster work is split into items: whole rows or columns of a box (kRowChunk 32, along
// the box's longer side), or chunks of kRowChunk pixels of one row. The items of its 32 triangles
// are laid end to end and taken 32 at a time. The owner of an item is the last triangle whose items
// start at or before it in the current window (an OR-reduction of start positions), else the owner
// of the window's first item, carried over from the previous window. Each edge function
//   e = (b.x - a.x)*(py - a.y) - (b.y - a.y)*(px - a.x)     (drawing.cpp:36-39)
// is evaluated in the reference's operation order, its first product taken once per item.
// At most 48 registers, so 10 CTAs of 4 warps (40 warps) fit an SM: the kernel is issue-bound on
// dependent chains, and the extra warps hide them (48 warps, at 40 registers, spill and measured
// slower). CTAs of 4 warps measured faster than of 2, 3, 8 or 16: the warps share no work across
// their CTA, and smaller CTAs leave fewer SMs idle at the end of the pass.
template <uint32_t kRowChunk>  // pixels of one bounding-box row per work item; 32: whole rows or columns
__global__ void __launch_bounds__(kSetupThreads, 10) k_setup_raster(SetupArgs a) {
    __shared__ SetupStage stage[kSetupWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SetupStage& S = stage[warp];
    const int64_t t = blockIdx.x * (int64_t)kSetupThreads + threadIdx.x;
    // The mesh's vertex indices were uploaded before the frame: they are fetched while the vertex
    // pass finishes. Everything after the wait depends on that pass or the frame's clears.
    int32_t i0 = 0, i1 = 0, i2 = 0;
    if (t < a.ntri) {
        i0 = a.tri_v[3 * t];
        i1 = a.tri_v[3 * t + 1];
        i2 = a.tri_v[3 * t + 2];
    }
    pdl_wait();
    pdl_launch_dependents();

    uint32_t n_items = 0, n_tiles = 0, cpr = 1;
    uint32_t tlx = 0, tly = 0, brx = 0, bry = 0;
    EdgeTri T;
    uint32_t c_front = 0;
    bool large = false, col = false;
    if (t < a.ntri) {
        const float4 v0 = a.rv[i0], v1 = a.rv[i1], v2 = a.rv[i2];
        if (front_facing(v0, v1, v2, a.cw)) {
            c_front = 1;
            bounding_box(v0, v1, v2, a.lim_x, a.lim_y, tlx, tly, brx, bry);
            const uint32_t bw = brx - tlx + 1u, bh = bry - tly + 1u;
            const unsigned long long npx = (unsigned long long)bw * bh;
            make_edge_tri(v0, v1, v2, T);
            if (npx <= a.small_max && (kRowChunk == 32u ? min(bw, bh) : bw) <= small_max_row<kRowChunk>()) {
                if (kRowChunk == 32u) {
                    col = bw < bh;  // whole items along the longer side: fewer of them
                    n_items = col ? bw : bh;
                } else {
                    cpr = (bw + kRowChunk - 1u) / kRowChunk;
                    n_items = bh * cpr;
                }
            } else {
                large = true;
            }
        }
    }

    // Binned path: append (one atomic per warp that has any, so no warp waits for the others of its
    // block), and count the tiles the box overlaps. The list's order does not matter: the depth
    // test is a minimum over keys.
    const unsigned lmask = __ballot_sync(kFull, large);
    uint32_t lbase = 0u;
    if (lmask) {
        if (lane == 0) lbase = atomicAdd(&a.counters[0], (uint32_t)__popc(lmask));
        lbase = __shfl_sync(kFull, lbase, 0);
    }
    if (large) {
        const uint32_t slot = lbase + __popc(lmask & ((1u << lane) - 1u));
        if (slot < a.cap_large) {
            BinnedTri r;
            r.x0 = T.x0; r.y0 = T.y0; r.x1 = T.x1; r.y1 = T.y1;
            r.x2 = T.x2; r.y2 = T.y2; r.z0 = T.z0; r.z1 = T.z1;
            r.z2 = T.z2; r.area = T.area; r.thr = T.nthr; r.sgn = T.sgn;
            r.tri = (uint32_t)t; r.tl = tlx | (tly << 16); r.br = brx | (bry << 16); r.pad = 0;
            a.large[slot] = r;
            const uint32_t tx0 = tlx >> a.tile_shift, tx1 = brx >> a.tile_shift;
            const uint32_t ty0 = tly >> a.tile_shift, ty1 = bry >> a.tile_shift;
            n_tiles = (tx1 - tx0 + 1u) * (ty1 - ty0 + 1u);
        } else {
            atomicOr(&a.counters[1], STATUS_LARGE_OVERFLOW);
        }
    }

    // Per-lane counts. A warp's small triangles have at most 32 * small_max (<= 2^21) tested pixels,
    // so the warp sums fit in 32 bits.
    uint32_t c_tested = 0, c_inside = 0;

    // Cooperative raster of the warp's small triangles. Each lane finds the run of pixels of its
    // item that the early reject cannot rule out: whole items (kRowChunk 32: a row or a column of
    // the box) from the two ends of their passing interval, verified exactly, shorter items (row
    // chunks) by evaluating the edges at each of their pixels. Non-empty runs go to a per-warp ring,
    // and whenever 32 pixels are pending the warp shares them out, one per lane, for the exact test
    // (the reference's three divisions), the depth and the atomic. So the divisions and atomics run
    // on full warps whatever the runs' lengths.
    {
        const uint32_t incl = warp_inclusive_scan(n_items, lane);
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        if (total) {
            const uint32_t start = incl - n_items;
            // The coefficients are staged multiplied by sgn (+-1, exact), so the staged edge values
            // are f = sgn*e bit for bit, and f / (sgn*area) is e / area exactly.
            const float sg = T.sgn;
            const float A[3] = {mul(sg, T.d12x), mul(sg, T.d20x), mul(sg, T.d01x)};
            const float B[3] = {mul(sg, T.d12y), mul(sg, T.d20y), mul(sg, T.d01y)};
            const float X[3] = {T.x1, T.x2, T.x0}, Y[3] = {T.y1, T.y2, T.y0};
            float R[3] = {0.f, 0.f, 0.f};
            // Whole items also flag (bit 31 of the `fixed` word) the triangles whose items may take
            // the crossing search: early reject on, every coefficient finite, and
            // |U| * (|V| + 2^16) < 2^126, so that each item's product U * (fixed - V) is finite too.
            bool searchable = T.nthr > -INFINITY;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float U = col ? -B[k] : A[k], V = col ? X[k] : Y[k];
                const float W = col ? -A[k] : B[k], Z = col ? Y[k] : X[k];
                S.rec[lane][k] = make_float4(U, V, W, Z);
                if (kRowChunk == 32u) {
                    R[k] = __fdividef(1.0f, W);  // an estimate: the search verifies what it gives
                    searchable = searchable && fabsf(U) * (fabsf(V) + 65536.f) < 0x1p126f && fabsf(W) < INFINITY &&
                                 fabsf(Z) < INFINITY;
                }
            }
            S.rec[lane][3] = make_float4(R[0], R[1], R[2], T.nthr);
            S.rec[lane][4] = make_float4(T.z0, T.z1, T.z2, mul(sg, T.area));
            S.tlx[lane] = col ? tly : tlx;  // the items' range along
            S.brx[lane] = col ? bry : brx;
            S.tly[lane] = (col ? tlx : tly) | (kRowChunk == 32u && searchable ? 0x80000000u : 0u) |
                          (col ? 0x40000000u : 0u);  // the first item across, flags
            if (kRowChunk != 32u) {
                S.cpr[lane] = cpr;
                S.rcpr[lane] = __frcp_rn((float)cpr);
            } else {
                // The correctly rounded reciprocal of the staged area (rec[4].w) for div_by, or 0
                // (use __fdiv_rn) when its magnitude is outside [2^-60, 2^60]. The correction step
                // is symmetric in the divisor's sign.
                S.rcpr[lane] = div_by_recip(mul(sg, T.area));
            }
            S.incl[lane] = incl;
            __syncwarp();
            const uint32_t tri_base = (uint32_t)(blockIdx.x * (int64_t)kSetupThreads + warp * 32);
            const unsigned lt_mask = (1u << lane) - 1u;
            // Ring state (warp-uniform): the oldest pending run, the runs pending, the pixels of the
            // oldest run already done, and the pixels pending.
            uint32_t q_head = 0, q_count = 0, q_skip = 0, q_pix = 0;

            // Exact test, depth and atomic (drawing.cpp:108-121) for the next min(q_pix, 32) pending
            // pixels, one per lane. The pending runs are laid end to end from the ring's head; a
            // lane's pixel belongs to the last run starting at or before it (an OR-reduction of the
            // runs' start positions). The runs it completes leave the ring, and a run it ends inside
            // stays at the head with its done pixels counted in q_skip.
            auto drain_round = [&]() {
                uint32_t cnt = 0u, tf = 0u, own = 0u;
                if ((uint32_t)lane < q_count) {
                    const uint32_t e = (q_head + lane) & 63u;
                    tf = S.q_tf[e];
                    own = S.q_om[e];
                    cnt = S.q_m[e];
                    if (lane == 0) {
                        tf += q_skip;  // t in the low half-word, below 2^15
                        cnt -= q_skip;
                    }
                }
                const uint32_t incl_p = warp_inclusive_scan(cnt, lane);
                const uint32_t excl_p = incl_p - cnt;
                // Every pending run has a pixel, so the first 32 pixels lie within the first 32 runs.
                const bool opens = cnt != 0u && excl_p < 32u;
                if (opens) S.slot[excl_p] = lane;
                const unsigned starts = __reduce_or_sync(kFull, opens ? (1u << excl_p) : 0u);
                __syncwarp();
                const int src = S.slot[31 - __clz(starts & (0xFFFFFFFFu >> (31 - lane)))];
                __syncwarp();
                // the lane's run, from the lane that loaded it
                const uint32_t r_tf = __shfl_sync(kFull, tf, src);
                const uint32_t r_om = __shfl_sync(kFull, own, src);
                const uint32_t r_excl = __shfl_sync(kFull, excl_p, src);
                const uint32_t avail = min(q_pix, 32u);
                if ((uint32_t)lane < avail) {
                    const uint32_t j = r_om & 31u;
                    const uint32_t tt = (r_tf & 0xFFFFu) + ((uint32_t)lane - r_excl), fx = r_tf >> 16;
                    const float4 q0 = S.rec[j][0], q1 = S.rec[j][1], q2 = S.rec[j][2], q4 = S.rec[j][4];
                    const float ff = (float)fx, tv = (float)tt;
                    const float e0 = sub(mul(q0.x, sub(ff, q0.y)), mul(q0.z, sub(tv, q0.w)));
                    const float e1 = sub(mul(q1.x, sub(ff, q1.y)), mul(q1.z, sub(tv, q1.w)));
                    const float e2 = sub(mul(q2.x, sub(ff, q2.y)), mul(q2.z, sub(tv, q2.w)));
                    const float ra = kRowChunk == 32u ? S.rcpr[j] : 0.f;
                    const float b0 = div_by(e0, q4.w, ra), b1 = div_by(e1, q4.w, ra), b2 = div_by(e2, q4.w, ra);
                    if (b0 >= 0.f && b1 >= 0.f && b2 >= 0.f) {
                        ++c_inside;
                        const float z = add(add(mul(q4.x, b0), mul(q4.y, b1)), mul(q4.z, b2));
                        const bool cl = (r_om & 32u) != 0u;
                        const uint32_t x = cl ? fx : tt, y = cl ? tt : fx;
                        if (z == z && x < a.width && y < a.height)
                            atomicMin(&a.keys[(size_t)y * a.width + x], frag_key(z, tri_base + j));
                    }
                }
                // runs completed by this round: a prefix of the ring
                const uint32_t nd = __popc(__ballot_sync(kFull, (uint32_t)lane < q_count && incl_p <= avail));
                const uint32_t sk = __shfl_sync(kFull, excl_p, nd & 31u);
                // A run left partly done is the one at lane nd (when there is one within the first 32).
                q_skip = nd == 0u ? q_skip + avail : (nd < q_count && nd < 32u ? avail - sk : 0u);
                q_head = (q_head + nd) & 63u;
                q_count -= nd;
                q_pix -= avail;
            };

            int carry = 0;
            for (uint32_t base = 0; base < total; base += 32) {
                // Bit b of `starts` is set when a triangle's items begin at item base + b; that
                // triangle's lane is in slot[b].
                const bool opens = n_items != 0u && start >= base && start < base + 32u;
                if (opens) S.slot[start - base] = lane;
                const unsigned starts = __reduce_or_sync(kFull, opens ? (1u << (start - base)) : 0u);
                __syncwarp();
                const unsigned upto = starts & (0xFFFFFFFFu >> (31 - lane));
                const int owner = upto ? S.slot[31 - __clz(upto)] : carry;
                carry = __shfl_sync(kFull, owner, 31);
                __syncwarp();
                const uint32_t k = base + lane;
                // The item's candidate run: pixels run_t .. run_t + run_n - 1 along the item at
                // `fixed` across it. It holds every pixel of the item that the early reject cannot
                // rule out (and possibly more).
                uint32_t run_t = 0u, run_n = 0u, fixed = 0u, cflag = 0u;
                if (k < total) {
                    const uint32_t ostart = owner ? S.incl[owner - 1] : 0u;
                    const uint32_t local = k - ostart;
                    uint32_t lo, hi;
                    bool searchable = false;
                    if constexpr (kRowChunk == 32u) {
                        const uint32_t fw = S.tly[owner];
                        searchable = (fw >> 31) != 0u;
                        cflag = (fw >> 25) & 32u;  // the column flag, as ring bit 5
                        lo = S.tlx[owner];
                        hi = S.brx[owner];
                        fixed = (fw & 0x3FFFFFFFu) + local;
                    } else {
                        const uint32_t ocpr = S.cpr[owner];
                        const uint32_t row = ocpr == 1u ? local : div_small(local, ocpr, S.rcpr[owner]);
                        lo = S.tlx[owner] + (local - row * ocpr) * kRowChunk;
                        hi = min(S.brx[owner], lo + (kRowChunk - 1u));
                        fixed = S.tly[owner] + row;
                    }
                    bool live = true;
#ifdef RAST_CHECKED
                    if (owner < 0 || owner > 31 || local >= S.incl[owner] - ostart || lo > hi ||
                        hi >= (cflag ? a.height : a.width) || fixed >= (cflag ? a.width : a.height)) {
                        report(a.counters, 1u, (uint32_t)owner);
                        live = false;
                    }
#endif
                    if (live) {
                        const float4 q0 = S.rec[owner][0], q1 = S.rec[owner][1], q2 = S.rec[owner][2],
                                     q3 = S.rec[owner][3];
                        const float ff = (float)fixed;
                        const float K0 = mul(q0.x, sub(ff, q0.y));  // U * (fixed - V), edge 0
                        const float K1 = mul(q1.x, sub(ff, q1.y));
                        const float K2 = mul(q2.x, sub(ff, q2.y));
                        const float thr = q3.w;
                        c_tested += hi - lo + 1u;  // the reference tests every pixel of the box
                        bool scan_row = true;  // evaluate every pixel of the item
                        if constexpr (kRowChunk == 32u) {
                            // Along the item each staged edge value is f(t) = K - W*(t - Z), every
                            // step rounded. Rounding is monotone, so for finite K, W, Z the computed
                            // f is monotone in t: non-increasing for W > 0, non-decreasing for W < 0,
                            // and K itself for W = 0. The pixels passing the early reject (f >= thr
                            // on all three edges) are then one interval of the item. Its ends are
                            // found from an estimate of each edge's crossing, Z + K/W, and each end
                            // is verified exactly at the two pixels either side of it. An item whose
                            // ends do not verify evaluates every pixel instead.
                            if (searchable) {
                                const float P[3] = {K0, K1, K2}, Wc[3] = {q0.z, q1.z, q2.z};
                                const float Zc[3] = {q0.w, q1.w, q2.w}, Rc[3] = {q3.x, q3.y, q3.z};
                                const float lof = (float)lo, hif = (float)hi;
                                float Lf = lof, Uf = hif;
                                bool ok = true;
#pragma unroll
                                for (int ed = 0; ed < 3; ++ed) {
                                    // Branch-free. W >= 0 edges (W = 0 included) pass a prefix of
                                    // the item, W < 0 edges a suffix. For W = 0, f = K along the item,
                                    // so the prefix is the whole item or nothing.
                                    const bool pos = Wc[ed] >= 0.f;
                                    const float est = Zc[ed] + P[ed] * Rc[ed];
                                    const float fl = floorf(est);
                                    // W > 0: the last passing pixel is floor(est); W < 0: the first is
                                    // ceil(est), and m is the pixel before it.
                                    float mf = (!pos && fl == est) ? fl - 1.f : fl;
                                    if (Wc[ed] == 0.f) mf = P[ed] >= thr ? hif : lof - 1.f;
                                    mf = fminf(fmaxf(mf, lof - 1.f), hif);  // a NaN estimate gives lo - 1
                                    const float mf1 = mf + 1.f;  // exact: integers below 2^16
                                    const float f0 = sub(P[ed], mul(Wc[ed], sub(mf, Zc[ed])));
                                    const float f1 = sub(P[ed], mul(Wc[ed], sub(mf1, Zc[ed])));
                                    const bool in0 = mf >= lof, in1 = mf1 <= hif;
                                    const bool pass0 = f0 >= thr, pass1 = f1 >= thr;
                                    // the prefix ends at m (pixel m passes, m + 1 does not), or the
                                    // suffix starts at m + 1 (m does not pass, m + 1 does)
                                    ok = ok && (!in0 || pass0 == pos) && (!in1 || pass1 != pos);
                                    Uf = pos ? fminf(Uf, mf) : Uf;
                                    Lf = pos ? Lf : fmaxf(Lf, mf1);
                                }
                                if (ok) {
                                    scan_row = false;
                                    if (Lf <= Uf) {
                                        run_t = (uint32_t)Lf;
                                        run_n = (uint32_t)(Uf - Lf) + 1u;
                                    }
                                }
                            } else if (!(thr > -INFINITY)) {
                                scan_row = false;  // no early reject: every pixel is a candidate
                                run_t = lo;
                                run_n = hi - lo + 1u;
                            }
                            if (scan_row && hi - lo >= 32u) {
                                scan_row = false;  // too long for the mask below: the whole item
                                run_t = lo;
                                run_n = hi - lo + 1u;
                            }
                            if (scan_row) {
                                const uint32_t n_px = hi - lo + 1u;
                                uint32_t mask = 0u;
                                for (uint32_t sx = 0; sx < n_px; ++sx) {
                                    const float tv = (float)(lo + sx);
                                    const float e0 = sub(K0, mul(q0.z, sub(tv, q0.w)));
                                    const float e1 = sub(K1, mul(q1.z, sub(tv, q1.w)));
                                    const float e2 = sub(K2, mul(q2.z, sub(tv, q2.w)));
                                    if (fminf(fminf(e0, e1), e2) >= thr) mask |= 1u << sx;
                                }
                                if (mask) {
                                    const uint32_t f0 = __ffs(mask) - 1u;
                                    run_t = lo + f0;
                                    run_n = (32u - __clz(mask)) - f0;
                                }
                            }
                        } else {
                            // Early reject on the smallest edge value of each pixel; the run spans the
                            // first to the last candidate. Two pixels per instruction: __fadd2_rn /
                            // __fmul2_rn round each component exactly as __fadd_rn / __fmul_rn, and
                            // a - b is a + (-b) bit for bit, so
                            //   f = K - W * (t - Z)  ==  K + -(W * (t + -Z)).
                            const float2 P0 = make_float2(K0, K0), P1 = make_float2(K1, K1), P2 = make_float2(K2, K2);
                            const float2 NZ0 = make_float2(-q0.w, -q0.w), NZ1 = make_float2(-q1.w, -q1.w),
                                         NZ2 = make_float2(-q2.w, -q2.w);
                            const float2 W0 = make_float2(q0.z, q0.z), W1 = make_float2(q1.z, q1.z),
                                         W2 = make_float2(q2.z, q2.z);
                            const float t_lo = (float)lo;
                            const uint32_t n_px = hi - lo + 1u;
                            uint32_t mask = 0u;
#pragma unroll
                            for (uint32_t sx = 0; sx < kRowChunk; sx += 2) {
                                // pixel centres t_lo + sx, + sx + 1: exact, integers below 2^24
                                const float2 tv = make_float2(add(t_lo, (float)sx), add(t_lo, (float)(sx + 1)));
                                const float2 t0 = __fmul2_rn(W0, __fadd2_rn(tv, NZ0));
                                const float2 t1 = __fmul2_rn(W1, __fadd2_rn(tv, NZ1));
                                const float2 t2 = __fmul2_rn(W2, __fadd2_rn(tv, NZ2));
                                const float2 e0 = __fadd2_rn(P0, make_float2(-t0.x, -t0.y));
                                const float2 e1 = __fadd2_rn(P1, make_float2(-t1.x, -t1.y));
                                const float2 e2 = __fadd2_rn(P2, make_float2(-t2.x, -t2.y));
                                const bool ca = sx < n_px && fminf(fminf(e0.x, e1.x), e2.x) >= thr;
                                const bool cb = sx + 1 < n_px && fminf(fminf(e0.y, e1.y), e2.y) >= thr;
                                mask |= ((uint32_t)ca | ((uint32_t)cb << 1)) << sx;
                            }
                            if (mask) {
                                const uint32_t f0 = __ffs(mask) - 1u;
                                run_t = lo + f0;
                                run_n = (32u - __clz(mask)) - f0;
                            }
                        }
#ifdef RAST_CHECKED
                        if (run_n && (run_t < lo || run_t + run_n - 1u > hi)) {
                            report(a.counters, 4u, run_t);
                            run_n = 0u;
                        }
#endif
                    }
                }
                const bool has = run_n != 0u;
                const unsigned m = __ballot_sync(kFull, has);
                if (has) {
                    const uint32_t e = (q_head + q_count + __popc(m & lt_mask)) & 63u;
                    S.q_tf[e] = run_t | (fixed << 16);
                    S.q_om[e] = (uint32_t)owner | cflag;
                    S.q_m[e] = run_n;
                }
                q_count += __popc(m);
                q_pix += __reduce_add_sync(kFull, run_n);
                __syncwarp();
                while (q_pix >= 32u) drain_round();  // leaves fewer than 32 runs pending
            }
            if (q_pix) drain_round();
            __syncwarp();
        }
    }

    // Cooperative tile counting over the warp's binned triangles.
    {
        const uint32_t incl = warp_inclusive_scan(n_tiles, lane);
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        if (total) {
            const uint32_t tx0 = tlx >> a.tile_shift, tx1 = brx >> a.tile_shift;
            const uint32_t tw = tx1 - tx0 + 1u;
            S.tlx[lane] = tx0;
            S.tly[lane] = tly >> a.tile_shift;
            S.cpr[lane] = tw;
            S.rcpr[lane] = __frcp_rn((float)tw);
            S.incl[lane] = incl;
            __syncwarp();
            for (uint32_t base = 0; base < total; base += 32) {
                const uint32_t k = base + lane;
                if (k < total) {
                    const int j = owner_of(S.incl, k);
                    const uint32_t local = k - (j ? S.incl[j - 1] : 0u);
                    const uint32_t w = S.cpr[j];
                    const uint32_t dy = div_small(local, w, S.rcpr[j]);
                    const uint32_t tile = (S.tly[j] + dy) * a.tiles_x + S.tlx[j] + (local - dy * w);
                    if (tile < a.n_tiles) atomicAdd(&a.counters[kCounterHeader + tile], 1u);
                }
            }
        }
    }

    stat_add32(a.stats, STAT_FRONT, c_front);
    stat_add32(a.stats, STAT_TESTED, c_tested);
    stat_add32(a.stats, STAT_INSIDE, c_inside);
}

// Exclusive scans over the tiles: entry offsets (the tile counts) into offset[0..n_tiles] and
// work-item offsets (ceil(count / kTileChunk)) into offset[n_tiles+1 .. 2*n_tiles+1]. One CTA of
// 1024 threads walks the tiles 8192 at a time, eight consecutive tiles a thread (two 16-byte loads
// and stores). Flags an overflow of the bin pool.
__global__ void __launch_bounds__(1024) k_bin_scan(const uint32_t* __restrict__ counters, uint32_t n_tiles,
                                                   uint32_t* __restrict__ offset, int64_t cap_entries,
                                                   uint32_t* __restrict__ status, unsigned long long* stats) {
    pdl_wait();
    pdl_launch_dependents();
    __shared__ uint32_t warp_tot[2][32];
    __shared__ uint32_t carry_s[2];
    const uint32_t* cnt = counters + kCounterHeader;  // 16-byte aligned: the header is 8 words
    uint32_t* chunk_offset = offset + n_tiles + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (counters[0] == 0u) {
        // Nothing binned: every tile count is zero (the counters are cleared before each frame), and
        // the consumers read only the totals.
        if (tid == 0) {
            offset[n_tiles] = 0u;
            chunk_offset[n_tiles] = 0u;
            *stat_slot0(stats, STAT_BIN_ENTRIES) = 0ull;
        }
        return;
    }
    if (tid < 2) carry_s[tid] = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n_tiles; base += 8192) {
        const uint32_t i0 = base + tid * 8;
        uint32_t v[8], c[8];
        if (i0 + 8 <= n_tiles) {
            const uint4 a = reinterpret_cast<const uint4*>(cnt + i0)[0], b = reinterpret_cast<const uint4*>(cnt + i0)[1];
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = i0 + k < n_tiles ? cnt[i0 + k] : 0u;
        }
        uint32_t s = 0, sc = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            c[k] = (v[k] + kTileChunk - 1) / kTileChunk;
            s += v[k];
            sc += c[k];
        }
        const uint32_t incl = warp_inclusive_scan(s, lane);
        const uint32_t incl_c = warp_inclusive_scan(sc, lane);
        if (lane == 31) {
            warp_tot[0][warp] = incl;
            warp_tot[1][warp] = incl_c;
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = warp_tot[0][lane], wc = warp_tot[1][lane];
            warp_tot[0][lane] = warp_inclusive_scan(w, lane) - w;
            warp_tot[1][lane] = warp_inclusive_scan(wc, lane) - wc;
        }
        __syncthreads();
        uint32_t run = carry_s[0] + warp_tot[0][warp] + incl - s;
        uint32_t run_c = carry_s[1] + warp_tot[1][warp] + incl_c - sc;
        uint32_t o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            o[k] = run;
            if (i0 + k < n_tiles) chunk_offset[i0 + k] = run_c;
            run += v[k];
            run_c += c[k];
        }
        if (i0 + 8 <= n_tiles) {
            reinterpret_cast<uint4*>(offset + i0)[0] = make_uint4(o[0], o[1], o[2], o[3]);
            reinterpret_cast<uint4*>(offset + i0)[1] = make_uint4(o[4], o[5], o[6], o[7]);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (i0 + k < n_tiles) offset[i0 + k] = o[k];
        }
        __syncthreads();
        if (tid == 1023) {
            carry_s[0] = run;
            carry_s[1] = run_c;
        }
        __syncthreads();
    }
    if (tid == 0) {
        offset[n_tiles] = carry_s[0];
        chunk_offset[n_tiles] = carry_s[1];
        *stat_slot0(stats, STAT_BIN_ENTRIES) = carry_s[0];
        if ((int64_t)carry_s[0] > cap_entries) atomicOr(status, STATUS_BIN_OVERFLOW);
    }
}

struct ScatterArgs {
    const BinnedTri* large;
    uint32_t n_tiles;
    const uint32_t* counters;  // [0] n_large
    uint32_t* cursors;         // n_tiles, zeroed
    const uint32_t* offset;
    uint32_t* entries;
    int64_t cap_large, cap_entries;
    uint32_t tile_shift, tiles_x;
    unsigned long long* stats;
};

// Writes every binned triangle's index into the lists of the tiles its box overlaps. Lanes of a
// warp share the work of their 32 triangles' tiles, as in k_setup_raster.
__global__ void __launch_bounds__(256) k_bin_scatter(ScatterArgs a) {
    pdl_wait();
    pdl_launch_dependents();
    __shared__ uint32_t s_tx0[8][32], s_ty0[8][32], s_tw[8][32], s_incl[8][32];
    __shared__ float s_rtw[8][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t n_large = (uint32_t)min((int64_t)a.counters[0], a.cap_large);
    if (blockIdx.x == 0 && threadIdx.x == 0) *stat_slot0(a.stats, STAT_BINNED_TRIS) = n_large;
    for (uint32_t wb = (blockIdx.x * 256u + warp * 32u); wb < n_large; wb += gridDim.x * 256u) {
        const uint32_t i = wb + lane;
        uint32_t n = 0, tx0 = 0, ty0 = 0, tw = 1;
        if (i < n_large) {
            const uint32_t tl = a.large[i].tl, br = a.large[i].br;
            tx0 = (tl & 0xFFFFu) >> a.tile_shift;
            ty0 = (tl >> 16) >> a.tile_shift;
            const uint32_t tx1 = (br & 0xFFFFu) >> a.tile_shift, ty1 = (br >> 16) >> a.tile_shift;
            tw = tx1 - tx0 + 1u;
            n = tw * (ty1 - ty0 + 1u);
        }
        const uint32_t incl = warp_inclusive_scan(n, lane);
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        s_tx0[warp][lane] = tx0; s_ty0[warp][lane] = ty0; s_tw[warp][lane] = tw;
        s_rtw[warp][lane] = __frcp_rn((float)tw); s_incl[warp][lane] = incl;
        __syncwarp();
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t k = base + lane;
            if (k < total) {
                const int j = owner_of(s_incl[warp], k);
                const uint32_t local = k - (j ? s_incl[warp][j - 1] : 0u);
                const uint32_t w = s_tw[warp][j];
                const uint32_t dy = div_small(local, w, s_rtw[warp][j]);
                const uint32_t tile = (s_ty0[warp][j] + dy) * a.tiles_x + s_tx0[warp][j] + (local - dy * w);
                if (tile < a.n_tiles) {
                    const uint32_t pos = a.offset[tile] + atomicAdd(&a.cursors[tile], 1u);
                    if ((int64_t)pos < a.cap_entries) a.entries[pos] = wb + (uint32_t)j;
                }
            }
        }
        __syncwarp();
    }
}

struct TileStage {
    float x0[kTileChunk], y0[kTileChunk], x1[kTileChunk], y1[kTileChunk], x2[kTileChunk], y2[kTileChunk];
    float d12x[kTileChunk], d12y[kTileChunk], d20x[kTileChunk], d20y[kTileChunk], d01x[kTileChunk],
        d01y[kTileChunk];
    float z0[kTileChunk], z1[kTileChunk], z2[kTileChunk], area[kTileChunk], nthr[kTileChunk], sgn[kTileChunk];
    uint32_t tri[kTileChunk], tl[kTileChunk], br[kTileChunk];
};

struct TileArgs {
    const BinnedTri* large;
    uint32_t* counters;        // [0] binned triangles, [1..3] status, [4] work counter, then tile counts
    const uint32_t* offset;    // entry offsets (n_tiles + 1), then work-item offsets (n_tiles + 1)
    const uint32_t* entries;
    int64_t cap_entries, cap_large;
    unsigned long long* keys;
    uint32_t width, height, tiles_x, n_tiles;
    unsigned long long* stats;
};

// Persistent CTAs take work items (a tile and up to kTileChunk of its binned triangles) from a
// counter until none are left, so a tile crowded with triangles is shared out among CTAs. Each of
// the TPT threads of a CTA (threads per tile) owns kPPT pixels of the tile (a warp covers an 8x4
// block per pixel slot) and keeps their minimum keys in registers; the item ends with one 64-bit
// atomicMin per pixel it improved (items of one tile may run at once, and the per-triangle pass
// wrote its keys earlier on the stream).
template <int TS, int TPT>
__global__ void __launch_bounds__(TPT) k_tile_raster(TileArgs a) {
    pdl_wait();
    pdl_launch_dependents();
    constexpr int kThreads = TPT;
    static_assert(TPT % 32 == 0 && (TS * TS) % TPT == 0, "whole warps, whole pixels per thread");
    constexpr int kPPT = (TS * TS) / kThreads;  // pixels per thread
    constexpr int kBlocksX = TS / 8;             // 8x4 blocks across a tile
    __shared__ TileStage S;
    __shared__ uint32_t s_item, s_tile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t* chunk_offset = a.offset + a.n_tiles + 1;
    const uint32_t total_items = chunk_offset[a.n_tiles];
    if (total_items == 0u) return;  // nothing binned
    const uint32_t n_large = a.counters[0];
    unsigned long long c_tested = 0, c_inside = 0;

    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t item = atomicAdd(&a.counters[4], 1u);
            uint32_t tile = 0;
            if (item < total_items) {
                // last tile whose first work item is <= item
                uint32_t lo = 0, hi = a.n_tiles - 1u;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1u) >> 1;
                    if (chunk_offset[mid] <= item) lo = mid; else hi = mid - 1u;
                }
                tile = lo;
            }
            s_item = item;
            s_tile = tile;
        }
        __syncthreads();
        const uint32_t item = s_item, tile = s_tile;
        if (item >= total_items) break;
        const uint32_t count = a.counters[kCounterHeader + tile];
        const uint32_t c0 = (item - chunk_offset[tile]) * kTileChunk;
        const uint32_t n = min((uint32_t)kTileChunk, count - c0);
        const uint32_t first = a.offset[tile] + c0;
        for (uint32_t i = threadIdx.x; i < n; i += kThreads) {
            const uint32_t e = first + i;
            uint32_t idx = (int64_t)e < a.cap_entries ? a.entries[e] : 0u;
            if (idx >= n_large || (int64_t)idx >= a.cap_large) {
                // Only a pool overflow (already flagged) can leave an entry unwritten.
                report(a.counters, 2u, idx);
                idx = 0;
            }
            const BinnedTri r = a.large[idx];
            S.x0[i] = r.x0; S.y0[i] = r.y0; S.x1[i] = r.x1; S.y1[i] = r.y1; S.x2[i] = r.x2; S.y2[i] = r.y2;
            S.d12x[i] = sub(r.x2, r.x1); S.d12y[i] = sub(r.y2, r.y1);
            S.d20x[i] = sub(r.x0, r.x2); S.d20y[i] = sub(r.y0, r.y2);
            S.d01x[i] = sub(r.x1, r.x0); S.d01y[i] = sub(r.y1, r.y0);
            S.z0[i] = r.z0; S.z1[i] = r.z1; S.z2[i] = r.z2;
            S.area[i] = r.area; S.nthr[i] = r.thr; S.sgn[i] = r.sgn;
            S.tri[i] = r.tri; S.tl[i] = r.tl; S.br[i] = r.br;
        }
        __syncthreads();

        const uint32_t tx = tile % a.tiles_x, ty = tile / a.tiles_x;
        uint32_t px[kPPT], py[kPPT];
        bool valid[kPPT];
        unsigned long long best[kPPT];
#pragma unroll
        for (int s = 0; s < kPPT; ++s) {
            const int blk = warp + s * (kThreads / 32);
            px[s] = tx * TS + (blk % kBlocksX) * 8 + (lane & 7);
            py[s] = ty * TS + (blk / kBlocksX) * 4 + (lane >> 3);
            valid[s] = px[s] < a.width && py[s] < a.height;
            best[s] = ~0ull;
        }
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t tl = S.tl[j], br = S.br[j];
            const uint32_t tlx = tl & 0xFFFFu, tly = tl >> 16, brx = br & 0xFFFFu, bry = br >> 16;
#pragma unroll
            for (int s = 0; s < kPPT; ++s) {
                const bool in_box = valid[s] && px[s] >= tlx && px[s] <= brx && py[s] >= tly && py[s] <= bry;
                if (!__any_sync(kFull, in_box)) continue;
                bool covered = false;
                if (in_box) {
                    EdgeTri U;
                    U.x0 = S.x0[j]; U.y0 = S.y0[j]; U.x1 = S.x1[j]; U.y1 = S.y1[j]; U.x2 = S.x2[j]; U.y2 = S.y2[j];
                    U.d12x = S.d12x[j]; U.d12y = S.d12y[j]; U.d20x = S.d20x[j]; U.d20y = S.d20y[j];
                    U.d01x = S.d01x[j]; U.d01y = S.d01y[j];
                    U.area = S.area[j]; U.nthr = S.nthr[j]; U.sgn = S.sgn[j];
                    float b0, b1, b2;
                    ++c_tested;
                    if (inside_test(U, (float)px[s], (float)py[s], b0, b1, b2)) {
                        covered = true;
                        U.z0 = S.z0[j]; U.z1 = S.z1[j]; U.z2 = S.z2[j];
                        const float z = interp_depth(U, b0, b1, b2);
                        if (z == z) {
                            const unsigned long long k = frag_key(z, S.tri[j]);
                            best[s] = k < best[s] ? k : best[s];
                        }
                    }
                }
                // Coverage mask of the warp's 8x4 block for this triangle.
                const unsigned mask = __ballot_sync(kFull, covered);
                if (lane == 0) c_inside += (unsigned)__popc(mask);
            }
        }
#pragma unroll
        for (int s = 0; s < kPPT; ++s)
            if (valid[s] && best[s] != ~0ull) atomicMin(&a.keys[(size_t)py[s] * a.width + px[s]], best[s]);
        __syncthreads();  // the stage and s_item are rewritten by the next item
    }
    stat_add(a.stats, STAT_TESTED, c_tested);
    stat_add(a.stats, STAT_INSIDE, c_inside);
}

struct ResolveArgs {
    uint32_t* counters;
    int64_t ntri;
    const unsigned long long* keys;
    unsigned long long* keys_rearm;  // non-null: keys are re-armed for the next frame as they are read
    const int32_t* tri_v;
    const int4* tri_nm;
    const float4* rv;
    const float* nrm;
    const float* pos;     // model-space positions (flat shading's face normals)
    const float* kd;
    const float* lights;
    int32_t nl;
    Mat4 normal;
    uint32_t width, height;
    bool cw;
    bool flat;            // RAST_FLAT: face normals in place of the vertex normals
    bool vec_ok;  // npx % 4 == 0 (planes stay 4-byte aligned), rgb 4-byte and depth 16-byte aligned
    uint8_t* rgb;
    float* depth;
    uint32_t* tri_id;
    unsigned long long* stats;
    const float* vcol;    // per-vertex albedo (nv * 3) or null for the material's Kd / texture
    const float* tex;     // textures (null: none), see DeviceMesh
    const long long* tex_off;
    const int2* tex_wh;
    const float* uv;
    const int32_t* tris10;
    float4* gbuf;         // deferred shading: 2 float4 per fragment record, or null to shade here
    uint32_t* gbuf_count; // deferred shading: records per block (1024 pixels)
    uint32_t* shade_index;  // deferred shading: the tile list build_shade_tiles writes
    bool keep_on_overflow;  // write nothing when the frame's bin pools overflowed
};

constexpr int kResolveThreads = 256;
constexpr int kResolveWarps = kResolveThreads / 32;
constexpr int kSpan = 128;  // consecutive pixels per warp, 4 per lane
static_assert(kResolveWarps * kSpan == kShadeBlock, "a resolve block is one block of shading records");

// CImg's linear_atXY(fx, fy, 0, c) for c = 0, 1, 2 on a normalised planar texture: the coordinates
// clamped to [0, w-1] x [0, h-1] (cimg::cut), the integer corner by truncation, and the blend
// Icc + dx*(Inc - Icc + dy*(Icc + Inn - Icn - Inc)) + dy*(Icn - Icc) in CImg's order.
__device__ __forceinline__ float3 texture_sample(const float* img, int w, int h, float fx, float fy) {
    const float wm = (float)(w - 1), hm = (float)(h - 1);
    const float nfx = fx < 0.f ? 0.f : (fx > wm ? wm : fx);
    const float nfy = fy < 0.f ? 0.f : (fy > hm ? hm : fy);
    const uint32_t x = min(__float2uint_rz(nfx), (uint32_t)(w - 1)), y = min(__float2uint_rz(nfy), (uint32_t)(h - 1));
    const float dx = sub(nfx, (float)x), dy = sub(nfy, (float)y);
    const uint32_t nx = dx > 0.f ? x + 1 : x, ny = dy > 0.f ? y + 1 : y;
    const size_t plane = (size_t)w * h;
    float r[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float* P = img + c * plane;
        const float Icc = __ldg(P + x + (size_t)y * w), Inc = __ldg(P + nx + (size_t)y * w);
        const float Icn = __ldg(P + x + (size_t)ny * w), Inn = __ldg(P + nx + (size_t)ny * w);
        const float t = add(sub(Inc, Icc), mul(dy, sub(sub(add(Icc, Inn), Icn), Inc)));
        r[c] = add(add(Icc, mul(dx, t)), mul(dy, sub(Icn, Icc)));
    }
    return make_float3(r[0], r[1], r[2]);
}

// The winning fragment's attributes as update_pixel computes them (drawing.cpp:108-140):
// barycentrics at the integer pixel, NDC depth, perspective-correct normal, normalised and flipped
// for clockwise winding, and the albedo (the material's Kd, or the perspective-correct per-vertex
// colour when the mesh has one).
__device__ __forceinline__ void fragment_attributes(const ResolveArgs& a, uint32_t x, uint32_t y, float4 v0, float4 v1,
                                                    float4 v2, float3 n0, float3 n1, float3 n2, int mat,
                                                    int32_t i0, int32_t i1, int32_t i2, int64_t tri, float& depth,
                                                    float3& nrm, float3& alb) {
    EdgeTri T;
    make_edge_tri(v0, v1, v2, T);
    const float pxf = (float)x, pyf = (float)y;
    const float e0 = sub(mul(T.d12x, sub(pyf, T.y1)), mul(T.d12y, sub(pxf, T.x1)));
    const float e1 = sub(mul(T.d20x, sub(pyf, T.y2)), mul(T.d20y, sub(pxf, T.x2)));
    const float e2 = sub(mul(T.d01x, sub(pyf, T.y0)), mul(T.d01y, sub(pxf, T.x0)));
    const float b0 = dvd(e0, T.area), b1 = dvd(e1, T.area), b2 = dvd(e2, T.area);
    depth = interp_depth(T, b0, b1, b2);

    const float i0w = mul(v0.w, b0), i1w = mul(v1.w, b1), i2w = mul(v2.w, b2);
    const float dd = dvd(1.f, add(add(i0w, i1w), i2w));
    float sx = add(add(mul(i0w, n0.x), mul(i1w, n1.x)), mul(i2w, n2.x));
    float sy = add(add(mul(i0w, n0.y), mul(i1w, n1.y)), mul(i2w, n2.y));
    float sz = add(add(mul(i0w, n0.z), mul(i1w, n1.z)), mul(i2w, n2.z));
    sx = mul(dd, sx); sy = mul(dd, sy); sz = mul(dd, sz);
    const float inv = dvd(1.0f, __fsqrt_rn(add(add(mul(sx, sx), mul(sy, sy)), mul(sz, sz))));
    nrm = make_float3(mul(sx, inv), mul(sy, inv), mul(sz, inv));
    if (a.cw) nrm = make_float3(-nrm.x, -nrm.y, -nrm.z);

    if (a.vcol) {
        const float* c0 = a.vcol + 3 * (int64_t)i0;
        const float* c1 = a.vcol + 3 * (int64_t)i1;
        const float* c2 = a.vcol + 3 * (int64_t)i2;
        float ux = add(add(mul(i0w, __ldg(c0)), mul(i1w, __ldg(c1))), mul(i2w, __ldg(c2)));
        float uy = add(add(mul(i0w, __ldg(c0 + 1)), mul(i1w, __ldg(c1 + 1))), mul(i2w, __ldg(c2 + 1)));
        float uz = add(add(mul(i0w, __ldg(c0 + 2)), mul(i1w, __ldg(c1 + 2))), mul(i2w, __ldg(c2 + 2)));
        alb = make_float3(mul(dd, ux), mul(dd, uy), mul(dd, uz));
    } else if (a.tex && __ldg(a.tex_off + mat) >= 0) {
        // drawing.cpp:166-170 (uv (0, 0) where the index is < 0) and 135, material.cpp:18-21
        float ux[3] = {0.f, 0.f, 0.f}, uy[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int32_t ui = __ldg(a.tris10 + 10 * tri + 6 + k);
            if (ui >= 0) {
                ux[k] = __ldg(a.uv + 2 * (int64_t)ui);
                uy[k] = __ldg(a.uv + 2 * (int64_t)ui + 1);
            }
        }
        const float u = mul(dd, add(add(mul(i0w, ux[0]), mul(i1w, ux[1])), mul(i2w, ux[2])));
        const float v = mul(dd, add(add(mul(i0w, uy[0]), mul(i1w, uy[1])), mul(i2w, uy[2])));
        const int2 wh = __ldg(a.tex_wh + mat);
        alb = texture_sample(a.tex + __ldg(a.tex_off + mat), wh.x, wh.y, mul(u, (float)wh.x),
                             mul(sub(1.f, v), (float)wh.y));
    } else {
        const float* kd = a.kd + 3 * (int64_t)mat;
        alb = make_float3(__ldg(kd), __ldg(kd + 1), __ldg(kd + 2));
    }
}

struct ResolveStage {
    uint32_t win_px[kSpan], win_tri[kSpan];  // compacted winners: pixel offset in the span, triangle
    float depth[kSpan];                      // per pixel offset: shaded depth and packed RGB
    uint32_t rgb[kSpan];
};

// Each warp takes kSpan consecutive pixels (4 per lane) of the flattened frame: it loads their keys
// (16-byte loads), re-arms them, compacts the pixels that have a winner, shades the
// winners one per lane so the gathers of 32 fragments are in flight together, and writes the
// frame and depth buffers 4 pixels per lane.
// kClear: RAST_CLEAR (every pixel written, the incoming depth 1.0); else read-modify-write.
template <bool kClear>
__global__ void __launch_bounds__(kResolveThreads) k_resolve(ResolveArgs a) {
    __shared__ ResolveStage stage[kResolveWarps];
    __shared__ uint32_t s_count[kResolveWarps];
    pdl_wait();
    // Deferred shading: the shading kernel may be launched once every block of this grid has
    // started (it waits for this grid's completion before it reads the records).
    pdl_launch_dependents();
    // Every earlier pass of the frame is complete here, so the status word is final. A deferred
    // frame's shading pass then finds an empty tile list and writes nothing either.
    if (a.keep_on_overflow && (a.counters[1] & (STATUS_BIN_OVERFLOW | STATUS_LARGE_OVERFLOW))) {
        if (a.shade_index && blockIdx.x == 0 && threadIdx.x == 0) {
            a.shade_index[0] = 0u;
            a.shade_index[1] = 0u;
        }
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    ResolveStage& S = stage[warp];
    const int64_t npx = (int64_t)a.width * a.height;
    const int64_t span0 = ((int64_t)blockIdx.x * kResolveWarps + warp) * kSpan;
    unsigned long long written = 0;
    const bool in_range = span0 < npx;
    {
        const int64_t p0 = span0 + 4 * lane;
        const bool full = in_range && p0 + 3 < npx;
        const bool vec = a.vec_ok && full;
        unsigned long long key[4];
        if (full) {
            const ulonglong2 k01 = *reinterpret_cast<const ulonglong2*>(a.keys + p0);
            const ulonglong2 k23 = *reinterpret_cast<const ulonglong2*>(a.keys + p0 + 2);
            key[0] = k01.x; key[1] = k01.y; key[2] = k23.x; key[3] = k23.y;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) key[k] = in_range && p0 + k < npx ? a.keys[p0 + k] : kNoWinner;
        }
        if (a.keys_rearm && in_range) {
            const unsigned long long r = kClear ? clear_key() : kArmed;
            if (full) {
                *reinterpret_cast<ulonglong2*>(a.keys_rearm + p0) = make_ulonglong2(r, r);
                *reinterpret_cast<ulonglong2*>(a.keys_rearm + p0 + 2) = make_ulonglong2(r, r);
            } else {
                for (int k = 0; k < 4; ++k)
                    if (p0 + k < npx) a.keys_rearm[p0 + k] = r;
            }
        }
        // Read-modify-write: the nearest fragment wins when it beats the incoming depth
        // (drawing.cpp:119), the depth buffer's value, read only where a fragment landed (the keys
        // of pixels outside the frame hold no fragment). For a NaN incoming depth nothing passes.
        // Clear mode: every fragment that landed beat 1.0 already.
        // A lane's four pixels are read as one 16-byte load when any fragment landed among them
        // (over the host link, where the buffers may live, four scalar loads of one line cost four
        // transactions).
        float din[4] = {0.f, 0.f, 0.f, 0.f};
        if (!kClear) {
            bool any = false;
#pragma unroll
            for (int k = 0; k < 4; ++k) any |= (uint32_t)key[k] != 0xFFFFFFFFu;
            if (vec) {
                if (any) {
                    const float4 d4 = *reinterpret_cast<const float4*>(a.depth + p0);
                    din[0] = d4.x; din[1] = d4.y; din[2] = d4.z; din[3] = d4.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if ((uint32_t)key[k] != 0xFFFFFFFFu) din[k] = a.depth[p0 + k];
            }
        }
        // compact the winners of the span
        bool win[4];
        uint32_t n_win = 0;
        const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t t = (uint32_t)(key[k] & 0xFFFFFFFFull);
            win[k] = t != 0xFFFFFFFFu;
            if (!kClear) win[k] = win[k] && din[k] == din[k] && (uint32_t)(key[k] >> 32) < depth_order(din[k]);
            if (win[k] && (int64_t)t >= a.ntri) {
                report(a.counters, 3u, t);
                win[k] = false;
            }
            const unsigned m = __ballot_sync(kFull, win[k]);
            if (win[k]) {
                const uint32_t pos = n_win + __popc(m & lt_mask);
                S.win_px[pos] = 4u * lane + k;
                S.win_tri[pos] = t;
            }
            n_win += __popc(m);
        }
        __syncwarp();
        // deferred shading: the block's winners go to its records in raster order; this warp's
        // start is the count of the warps before it
        uint32_t rec_base = 0;
        if (a.gbuf) {
            if (lane == 0) s_count[warp] = n_win;
            __syncthreads();
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < kResolveWarps; ++w) {
                const uint32_t c = s_count[w];
                before += w < warp ? c : 0u;
                total += c;
            }
            rec_base = blockIdx.x * (uint32_t)(kResolveWarps * kSpan) + before;
            if (threadIdx.x == 0) a.gbuf_count[blockIdx.x] = total;
        }
        for (uint32_t i = lane; i < n_win; i += 32) {
            const uint32_t off = S.win_px[i];
            const int64_t tt = S.win_tri[i];
            const uint32_t p = (uint32_t)(span0 + off);  // < 2^30: width, height <= 32768
            const uint32_t y = p / a.width, x = p - y * a.width;
            const int32_t i0 = __ldg(a.tri_v + 3 * tt), i1 = __ldg(a.tri_v + 3 * tt + 1), i2 = __ldg(a.tri_v + 3 * tt + 2);
            const int4 nm = __ldg(a.tri_nm + tt);
            const float4 v0 = __ldg(a.rv + i0), v1 = __ldg(a.rv + i1), v2 = __ldg(a.rv + i2);
            float3 n0, n1, n2;
            if (a.flat) {
                // flat shading: every vertex takes the face normal (model space), then the path is
                // unchanged
                const float3 f = face_normal(a.pos, i0, i1, i2);
                n0 = n1 = n2 = camera_normal(a.normal, f.x, f.y, f.z);
            } else {
                const float* q0 = a.nrm + 3 * (int64_t)nm.x;
                const float* q1 = a.nrm + 3 * (int64_t)nm.y;
                const float* q2 = a.nrm + 3 * (int64_t)nm.z;
                n0 = camera_normal(a.normal, __ldg(q0), __ldg(q0 + 1), __ldg(q0 + 2));
                n1 = camera_normal(a.normal, __ldg(q1), __ldg(q1 + 1), __ldg(q1 + 2));
                n2 = camera_normal(a.normal, __ldg(q2), __ldg(q2 + 1), __ldg(q2 + 2));
            }
            float dep;
            float3 nrm, alb;
            fragment_attributes(a, x, y, v0, v1, v2, n0, n1, n2, nm.w, i0, i1, i2, tt, dep, nrm, alb);
            S.depth[off] = dep;
            if (a.gbuf) {
                // deferred: the span's i-th record; the shading pass writes the colour
                const size_t slot = (size_t)rec_base + i;
                a.gbuf[2 * slot] = make_float4(nrm.x, nrm.y, nrm.z, alb.x);
                a.gbuf[2 * slot + 1] = make_float4(alb.y, alb.z, __uint_as_float(p), 0.f);
                S.rgb[off] = 0u;
            } else {
                S.rgb[off] = shade_lights(a.lights, a.nl, nrm, alb);
            }
        }
        written = n_win;
        __syncwarp();
        if (in_range) {
        float dep[4];
        uint32_t col[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            dep[k] = win[k] ? S.depth[4 * lane + k] : 1.0f;
            col[k] = win[k] ? S.rgb[4 * lane + k] : 0u;
        }
        const int64_t plane = npx;
        // four winners in a row (read-modify-write) are written like a cleared frame's pixels
        const bool all4 = vec && win[0] && win[1] && win[2] && win[3];
        if ((kClear && vec) || all4) {
            // every pixel is written: background 0 / 1.0 where nothing won
            *reinterpret_cast<float4*>(a.depth + p0) = make_float4(dep[0], dep[1], dep[2], dep[3]);
            uint32_t pr = 0, pg = 0, pb = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                pr |= (col[k] & 0xFFu) << (8 * k);
                pg |= ((col[k] >> 8) & 0xFFu) << (8 * k);
                pb |= ((col[k] >> 16) & 0xFFu) << (8 * k);
            }
            *reinterpret_cast<uint32_t*>(a.rgb + p0) = pr;
            *reinterpret_cast<uint32_t*>(a.rgb + plane + p0) = pg;
            *reinterpret_cast<uint32_t*>(a.rgb + 2 * plane + p0) = pb;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (p0 + k < npx && (win[k] || kClear)) {
                    a.depth[p0 + k] = dep[k];
                    a.rgb[p0 + k] = (uint8_t)(col[k] & 0xFFu);
                    a.rgb[plane + p0 + k] = (uint8_t)((col[k] >> 8) & 0xFFu);
                    a.rgb[2 * plane + p0 + k] = (uint8_t)((col[k] >> 16) & 0xFFu);
                }
            }
        }
        if (a.tri_id) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (p0 + k < npx) a.tri_id[p0 + k] = win[k] ? (uint32_t)(key[k] & 0xFFFFFFFFull) : 0xFFFFFFFFu;
        }
        }
        // lane 0 counts for the warp
        if (lane != 0) written = 0;
    }
    stat_add(a.stats, STAT_WRITTEN, written);
    if (a.gbuf) {
        // the last block to finish lists the shading tiles of all blocks
        __shared__ bool s_last;
        if (threadIdx.x == 0) {
            __threadfence();  // this block's count is visible before its ticket
            s_last = atomicAdd(&a.counters[kResolveTicket], 1u) == gridDim.x - 1;
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            build_shade_tiles(a.gbuf_count, gridDim.x, a.shade_index);
        }
    }
}

int grid_for(int64_t n, int threads, int max_blocks) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b < max_blocks ? b : max_blocks);
}

// Launches a kernel of the frame after its first with programmatic stream serialization: it may
// start while the kernel before it runs, and waits for it (pdl_wait) before anything else.
template <typename... Params, typename... Args>
cudaError_t launch_pdl(bool chained, void (*kernel)(Params...), unsigned grid, unsigned block, cudaStream_t stream,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = chained ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int TS, int TPT>
cudaError_t launch_tile(const TileArgs& ta, int n_sm, bool chained, cudaStream_t stream) {
    const int per_sm = 2048 / TPT < 8 ? 2048 / TPT : 8;
    return launch_pdl(chained, k_tile_raster<TS, TPT>, (unsigned)(n_sm * per_sm), (unsigned)TPT, stream, ta);
}

// The tile raster for tile edge TS with `threads` threads per tile (0: min(TS*TS, 256)); values
// the kernel does not take fall back to the default.
template <int TS>
cudaError_t launch_tile_threads(const TileArgs& ta, uint32_t threads, int n_sm, bool chained, cudaStream_t stream) {
    if constexpr (TS == 8) {
        return launch_tile<8, 64>(ta, n_sm, chained, stream);
    } else {
        if (threads == 64u) return launch_tile<TS, 64>(ta, n_sm, chained, stream);
        if (threads == 128u) return launch_tile<TS, 128>(ta, n_sm, chained, stream);
        if constexpr (TS == 32)
            if (threads == 512u) return launch_tile<TS, 512>(ta, n_sm, chained, stream);
        return launch_tile<TS, 256>(ta, n_sm, chained, stream);
    }
}

}  // namespace

int launch_split_triangles(const int32_t* tris10, int64_t ntri, int32_t* tri_v, int4* tri_nm, cudaStream_t stream) {
    k_split_triangles<<<grid_for(ntri, 256, 1 << 16), 256, 0, stream>>>(tris10, ntri, tri_v, tri_nm);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_arm_keys(unsigned long long* keys, int64_t n, bool clear, cudaStream_t stream) {
    k_arm_keys<<<grid_for(n, 256, 1 << 16), 256, 0, stream>>>(keys, n, clear);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_draw(const DeviceMesh& mesh, const FrameScratch& s, const DrawParams& p, cudaStream_t stream,
                cudaEvent_t* events) {
    auto mark = [&](int i) {
        if (events) cudaEventRecord(events[i], stream);
    };
    const bool clear = (p.flags & 2u) != 0;  // RAST_CLEAR
    const bool cw = (p.flags & 1u) != 0;     // RAST_WIND_CLOCKWISE
    const bool flat = (p.flags & 4u) != 0;   // RAST_FLAT
    const int64_t npx = (int64_t)p.width * p.height;
    const uint32_t n_tiles = p.tiles_x * p.tiles_y;
    const uint32_t shift = p.tile == 8 ? 3u : (p.tile == 16 ? 4u : 5u);
    int launches = 0;

    mark(0);
    mark(1);
    const FrameClear clr{s.counters,    s.clear_counter_words,
                         s.stats,       s.clear_stats ? (uint32_t)kStatWords : 0u,
                         s.shade_stats, s.clear_shade_stats && s.shade_stats ? (uint32_t)kShadeStats : 0u};
    if ((reinterpret_cast<uintptr_t>(mesh.pos) % 16u) == 0)
        k_vertex4<<<grid_for(mesh.nv / 4 + mesh.nv % 4, 256, 1 << 16), 256, 0, stream>>>(
            mesh.pos, mesh.nv, p.camera, (float)(int)p.width, (float)(int)p.height, s.rv, clr);
    else
        k_vertex<<<grid_for(mesh.nv, 256, 1 << 16), 256, 0, stream>>>(mesh.pos, mesh.nv, p.camera, (float)(int)p.width,
                                                                       (float)(int)p.height, s.rv, clr);
    ++launches;
    mark(2);

    SetupArgs sa;
    sa.tri_v = mesh.tri_v;
    sa.rv = s.rv;
    sa.ntri = mesh.ntri;
    sa.lim_x = (float)(p.width - 1u);
    sa.lim_y = (float)(p.height - 1u);
    sa.width = p.width;
    sa.height = p.height;
    sa.small_max = p.small_max;
    sa.tile_shift = shift;
    sa.tiles_x = p.tiles_x;
    sa.n_tiles = n_tiles;
    sa.cw = cw;
    sa.keys = s.keys;
    sa.large = s.large;
    sa.cap_large = s.cap_large;
    sa.counters = s.counters;
    sa.stats = s.stats;
    if (mesh.ntri > 0) {
        const unsigned blocks = (unsigned)((mesh.ntri + kSetupThreads - 1) / kSetupThreads);
        const unsigned th = (unsigned)kSetupThreads;
        cudaError_t e;
        if (p.row_chunk == 32) e = launch_pdl(p.chained, k_setup_raster<32>, blocks, th, stream, sa);
        else if (p.row_chunk == 8) e = launch_pdl(p.chained, k_setup_raster<8>, blocks, th, stream, sa);
        else e = launch_pdl(p.chained, k_setup_raster<4>, blocks, th, stream, sa);
        if (e != cudaSuccess) return -1;
        ++launches;
    }
    mark(3);

    if (launch_pdl(p.chained, k_bin_scan, 1u, 1024u, stream, (const uint32_t*)s.counters, n_tiles, s.tile_offset,
                   s.cap_entries, s.counters + 1, s.stats) != cudaSuccess)
        return -1;
    ++launches;
    mark(4);

    ScatterArgs sc;
    sc.large = s.large;
    sc.n_tiles = n_tiles;
    sc.counters = s.counters;
    sc.cursors = s.counters + kCounterHeader + n_tiles;
    sc.offset = s.tile_offset;
    sc.entries = s.entries;
    sc.cap_large = s.cap_large;
    sc.cap_entries = s.cap_entries;
    sc.tile_shift = shift;
    sc.tiles_x = p.tiles_x;
    sc.stats = s.stats;
    if (launch_pdl(p.chained, k_bin_scatter, (unsigned)grid_for(s.cap_large, 256, p.n_sm), 256u, stream, sc) != cudaSuccess)
        return -1;
    ++launches;
    mark(5);

    TileArgs ta;
    ta.large = s.large;
    ta.counters = s.counters;
    ta.offset = s.tile_offset;
    ta.entries = s.entries;
    ta.cap_entries = s.cap_entries;
    ta.cap_large = s.cap_large;
    ta.keys = s.keys;
    ta.width = p.width;
    ta.height = p.height;
    ta.tiles_x = p.tiles_x;
    ta.n_tiles = n_tiles;
    ta.stats = s.stats;
    const cudaError_t et = p.tile == 8 ? launch_tile_threads<8>(ta, p.tile_threads, p.n_sm, p.chained, stream)
                           : p.tile == 16 ? launch_tile_threads<16>(ta, p.tile_threads, p.n_sm, p.chained, stream)
                                          : launch_tile_threads<32>(ta, p.tile_threads, p.n_sm, p.chained, stream);
    if (et != cudaSuccess) return -1;
    ++launches;
    mark(6);
    if (p.before_resolve && cudaStreamWaitEvent(stream, p.before_resolve, 0) != cudaSuccess) return -1;

    ResolveArgs ra;
    ra.counters = s.counters;
    ra.ntri = mesh.ntri;
    ra.keys = s.keys;
    ra.keys_rearm = s.keys;
    ra.tri_v = mesh.tri_v;
    ra.tri_nm = mesh.tri_nm;
    ra.rv = s.rv;
    ra.nrm = mesh.nrm;
    ra.pos = mesh.pos;
    ra.kd = mesh.kd;
    ra.lights = p.lights;
    ra.nl = p.nl;
    ra.normal = p.normal;
    ra.width = p.width;
    ra.height = p.height;
    ra.cw = cw;
    ra.flat = flat;
    ra.vec_ok = (reinterpret_cast<uintptr_t>(p.rgb) % 4u) == 0 && (npx % 4) == 0 &&
                (reinterpret_cast<uintptr_t>(p.depth) % 16u) == 0;
    ra.rgb = p.rgb;
    ra.depth = p.depth;
    ra.tri_id = p.tri_id;
    ra.stats = s.stats;
    ra.vcol = mesh.vcol;
    ra.tex = mesh.tex;
    ra.tex_off = mesh.tex_off;
    ra.tex_wh = mesh.tex_wh;
    ra.uv = mesh.uv;
    ra.tris10 = mesh.tris10;
    const bool deferred = p.shader != 0;
    ra.gbuf = deferred ? s.gbuf : nullptr;
    ra.keep_on_overflow = p.keep_outputs_on_overflow;
    ra.gbuf_count = deferred ? s.gbuf_count : nullptr;
    ra.shade_index = deferred ? s.shade_index : nullptr;
    const int64_t spans = (npx + kSpan - 1) / kSpan;
    if (launch_pdl(p.chained, clear ? k_resolve<true> : k_resolve<false>, (unsigned)((spans + kResolveWarps - 1) / kResolveWarps),
                   (unsigned)kResolveThreads, stream, ra) != cudaSuccess)
        return -1;
    ++launches;
    mark(7);
    if (p.shader != 0) {
        const int n = launch_shade(s, p, (spans + kResolveWarps - 1) / kResolveWarps, stream);
        if (n < 0) return -1;
        launches += n;
    }
    mark(8);

    return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

}  // namespace rast
