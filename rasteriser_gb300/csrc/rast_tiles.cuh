// The tile list of the deferred shading pass, built by one CTA from the per-block fragment counts.
//
// The resolve pass stores the winning fragments of each 1024-pixel block in the block's own
// records (block * 1024 + i, raster order). The records, taken in block order, form one sequence
// of `fragments` records; shading tile t is records 128t .. 128t + 127 of it (the last tile may be
// shorter), so every tile but the last is full whatever the blocks' counts. The list keeps the
// exclusive prefix P of the blocks' counts and, per tile, a descriptor (b, P[b], P[b+1], P[b+2])
// for the block b holding its first record, so a record's slot in the first three blocks of its
// tile follows from the descriptor alone (shade_record_slot). The order is fixed, which makes
// every tile's contents, and so the learned shader's checked samples, the same from run to run.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rast_internal.h"

namespace rast {
namespace {

// Block-cooperative (blockDim a multiple of 32, at most 1024). index: [0] fragments, [1] tiles,
// [2..3] unused, [4 .. 4 + n_blocks] the prefix, then the tiles' first blocks.
__device__ __noinline__ void build_shade_tiles(const uint32_t* bcount, uint32_t n_blocks, uint32_t* index) {
    __shared__ uint32_t s_recs[32];
    const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = tid & 31u, warp = tid >> 5, nw = nt >> 5;
    const uint32_t per = (n_blocks + nt - 1) / nt;
    const uint32_t b0 = min(tid * per, n_blocks), b1 = min(b0 + per, n_blocks);
    uint32_t recs = 0;
    for (uint32_t b = b0; b < b1; ++b) recs += min(__ldcg(bcount + b), (uint32_t)kShadeBlock);
    uint32_t ir = recs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t r = __shfl_up_sync(0xFFFFFFFFu, ir, o);
        if ((int)lane >= o) ir += r;
    }
    if (lane == 31) s_recs[warp] = ir;
    __syncthreads();
    if (warp == 0) {
        uint32_t wr = lane < nw ? s_recs[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t r = __shfl_up_sync(0xFFFFFFFFu, wr, o);
            if ((int)lane >= o) wr += r;
        }
        if (lane < nw) s_recs[lane] = wr;
    }
    __syncthreads();
    const uint32_t total = s_recs[nw - 1];
    uint32_t* prefix = index + 4;
    uint4* desc = reinterpret_cast<uint4*>(index + kShadeTileDescWord(n_blocks));
    uint32_t p = ir - recs + (warp ? s_recs[warp - 1] : 0u);
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t c = min(__ldcg(bcount + b), (uint32_t)kShadeBlock);
        prefix[b] = p;
        p += c;
    }
    if (tid == 0) {
        index[0] = total;
        index[1] = (total + kShadeTile - 1) / kShadeTile;
        prefix[n_blocks] = total;
    }
    __syncthreads();
    // the tiles whose first record is in block b (P[b] <= 128t < P[b+1]); past the last block the
    // descriptor holds the total
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t pb = prefix[b], pe = prefix[b + 1];
        const uint32_t p2 = b + 2 <= n_blocks ? prefix[b + 2] : total;
        for (uint32_t t = (pb + kShadeTile - 1) / kShadeTile; t * kShadeTile < pe; ++t)
            desc[t] = make_uint4(b, pb, pe, p2);
    }
}

// Records in tile t, its descriptor, and the slot (block * 1024 + i) of record `row` of it
// (row < count), for the list above over n_blocks blocks.
__device__ __forceinline__ uint32_t shade_tile_count(const uint32_t* index, uint32_t t) {
    return min((uint32_t)kShadeTile, index[0] - t * (uint32_t)kShadeTile);
}
__device__ __forceinline__ uint4 shade_tile_desc(const uint32_t* index, uint32_t n_blocks, uint32_t t) {
    return reinterpret_cast<const uint4*>(index + kShadeTileDescWord(n_blocks))[t];
}
__device__ __forceinline__ size_t shade_record_slot(const uint32_t* index, uint32_t n_blocks, uint4 d, uint32_t t,
                                                    uint32_t row) {
    const uint32_t g = t * (uint32_t)kShadeTile + row;
    if (g < d.z) return (size_t)d.x * kShadeBlock + (g - d.y);
    if (g < d.w) return (size_t)(d.x + 1) * kShadeBlock + (g - d.z);
    // a tile over more than three blocks: walk the prefix on
    const uint32_t* prefix = index + 4;
    uint32_t b = d.x + 2;
    while (b + 1 < n_blocks && prefix[b + 1] <= g) ++b;
    return (size_t)b * kShadeBlock + (g - prefix[b]);
}

}  // namespace
}  // namespace rast
