// The tile list of the deferred shading pass, built by one CTA from the per-block fragment counts.
//
// The resolve pass stores the winning fragments of each 1024-pixel block in the block's own
// records (block * 1024 + i, raster order). A shading tile is up to 128 consecutive records of one
// block; tile entries are ((block * 8 + chunk) << 8) | (records - 1), so the tile's first record is
// (entry >> 8) * 128. The list is in block order, which makes every tile's contents, and so the
// learned shader's checked samples, the same from run to run.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rast_internal.h"

namespace rast {
namespace {

// Block-cooperative (blockDim a multiple of 32, at most 1024). index: [0] fragments, [1] tiles,
// [2..3] unused, then the tile entries.
__device__ __noinline__ void build_shade_tiles(const uint32_t* bcount, uint32_t n_blocks, uint32_t* index) {
    __shared__ uint32_t s_tiles[32], s_recs[32];
    const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = tid & 31u, warp = tid >> 5, nw = nt >> 5;
    const uint32_t per = (n_blocks + nt - 1) / nt;
    const uint32_t b0 = min(tid * per, n_blocks), b1 = min(b0 + per, n_blocks);
    uint32_t tiles = 0, recs = 0;
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t c = min(__ldcg(bcount + b), (uint32_t)kShadeBlock);
        tiles += (c + kShadeTile - 1) / kShadeTile;
        recs += c;
    }
    uint32_t it = tiles, ir = recs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, it, o), r = __shfl_up_sync(0xFFFFFFFFu, ir, o);
        if ((int)lane >= o) { it += t; ir += r; }
    }
    if (lane == 31) { s_tiles[warp] = it; s_recs[warp] = ir; }
    __syncthreads();
    if (warp == 0) {
        uint32_t wt = lane < nw ? s_tiles[lane] : 0u, wr = lane < nw ? s_recs[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wt, o), r = __shfl_up_sync(0xFFFFFFFFu, wr, o);
            if ((int)lane >= o) { wt += t; wr += r; }
        }
        if (lane < nw) { s_tiles[lane] = wt; s_recs[lane] = wr; }
    }
    __syncthreads();
    uint32_t t0 = it - tiles + (warp ? s_tiles[warp - 1] : 0u);
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t c = min(__ldcg(bcount + b), (uint32_t)kShadeBlock);
        for (uint32_t ch = 0; ch * kShadeTile < c; ++ch)
            index[4 + t0++] = ((b * 8u + ch) << 8) | (min((uint32_t)kShadeTile, c - ch * kShadeTile) - 1u);
    }
    if (tid == 0) {
        index[0] = s_recs[nw - 1];
        index[1] = s_tiles[nw - 1];
    }
}

}  // namespace
}  // namespace rast
