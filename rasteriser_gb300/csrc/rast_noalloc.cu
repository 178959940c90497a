// rast_draw_noalloc: one frame of the draw, with no context and no device allocation.
//
// Some callers cannot allocate device memory from inside the renderer: a host application that
// hands all device memory to its own pool and forbids allocations it does not own, or a frame loop
// that cannot take the implicit device-wide synchronisation of cudaMalloc / cudaFree. For them this
// entry point takes every input and output as a device pointer from the caller and keeps all
// intermediate buffers (split triangle indices, raster vertices, depth keys, the binned list, tile
// bins, counters) in one fixed array inside the library, kNoAllocScratchBytes large. Every GPU
// that loads the library holds that array until the process exits.
//
// The array's address is taken with cudaGetSymbolAddress the first time the entry point runs on a
// device (with that device current); that first call should come before any stream capture. All
// calls share the array, and it keeps the last call's contents: each call clears the counters and
// arms the depth keys it needs before using them. Calls whose work overlaps on the GPU (for
// example on two streams at once) race on the array; serialise them.
#include <cuda_runtime.h>

#include <cstdint>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "rast.h"
#include "rast_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Errors are reported through rast_last_error(NULL), as for rast_create.
rast_status fail(rast_status s, const std::string& msg) {
    rast::set_thread_error(msg);
    return s;
}

// Index check on the device: a triangle referring to a vertex, normal or material that does not
// exist sets status[0]. uv indices are not read by this entry point and are not checked.
__global__ void k_check_indices(const int32_t* __restrict__ tris10, int64_t ntri, int64_t nv, int64_t nn,
                                int32_t nmat, uint32_t* status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ntri; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t* t = tris10 + 10 * i;
        bool ok = t[9] >= 0 && t[9] < nmat;
        for (int k = 0; k < 3; ++k) ok = ok && t[k] >= 0 && t[k] < nv && t[3 + k] >= 0 && t[3 + k] < nn;
        if (!ok) atomicOr(status, 1u);
    }
}

// Carves `bytes` (rounded up to 256) off the scratch array.
struct Carver {
    unsigned char* base;
    size_t used = 0;
    template <typename T> T* take(size_t bytes) {
        T* p = reinterpret_cast<T*>(base + used);
        used += (bytes + 255) & ~size_t(255);
        return p;
    }
};

}  // namespace

extern "C" rast_status rast_draw_noalloc(const float* d_pos, int64_t nv, const float* d_nrm, int64_t nn,
                                         const int32_t* d_tris, int64_t ntri, const float* d_kd, int32_t nmat,
                                         const float* d_lights7, int32_t nl, const float camera[16],
                                         const float normal[16], uint32_t width, uint32_t height, uint32_t flags,
                                         uint8_t* d_rgb_planar, float* d_depth, uint32_t* d_tri_id, void* stream) {
    if (!camera || !normal || !d_rgb_planar || !d_depth) return fail(RAST_ERR_INVALID_ARG, "null matrix or buffer");
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(RAST_ERR_INVALID_ARG, "frame size out of range");
    if (nv < 0 || nn < 0 || ntri < 0 || nmat < 0 || nl < 0 || nl > 4096 || (nv && !d_pos) || (nn && !d_nrm) ||
        (ntri && !d_tris) || (nmat && !d_kd) || (nl && !d_lights7))
        return fail(RAST_ERR_INVALID_ARG, "bad count or null array");
    if (ntri >= 0xFFFFFFFFll) return fail(RAST_ERR_INVALID_ARG, "too many triangles");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(RAST_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(RAST_ERR_INVALID_ARG, "device ordinal beyond 63");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> g(g_setup_mu);
        if (!g_scratch_ptr[dev]) {
            // Set-up, once per device, with that device current: the host-side name of the array is
            // not a device address; cudaGetSymbolAddress gives the address kernels can use.
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return fail(RAST_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_ptr[dev] = p;
        }
        base = g_scratch_ptr[dev];
    }

    // Lay out the frame's fixed-size buffers first; the tile-bin entries then take every byte of
    // the array that is left, since their need depends on how much screen the triangles cover (a
    // screen-sized triangle is one entry per tile) and this entry point cannot grow them.
    const uint32_t tile = 16;
    const uint32_t tiles_x = (width + tile - 1) / tile, tiles_y = (height + tile - 1) / tile;
    const uint32_t n_tiles = tiles_x * tiles_y;
    const int64_t npx = (int64_t)width * height;
    const int64_t cap_large = ntri > 0 ? ntri : 1;
    const size_t counter_words = rast::kCounterHeader + 2 * (size_t)n_tiles;
    size_t fixed = 0;
    for (size_t b : {(size_t)12 * cap_large, (size_t)16 * cap_large, (size_t)16 * (nv > 0 ? nv : 1), (size_t)8 * npx,
                     sizeof(rast::BinnedTri) * (size_t)cap_large, 4 * counter_words, 4 * 2 * ((size_t)n_tiles + 1),
                     sizeof(unsigned long long) * rast::kStatWords, (size_t)256})
        fixed += (b + 255) & ~size_t(255);
    const size_t min_entries = 65536;
    if (fixed + 4 * min_entries > kNoAllocScratchBytes)
        return fail(RAST_ERR_INVALID_ARG, "frame needs " + std::to_string(fixed + 4 * min_entries) +
                                              " bytes of scratch; the fixed array holds " +
                                              std::to_string(kNoAllocScratchBytes));
    // the entry count travels in 32-bit counters
    const int64_t cap_entries = (int64_t)std::min<size_t>((kNoAllocScratchBytes - fixed) / 4 / 64 * 64, 0x7FFFFFFFu);

    Carver c{static_cast<unsigned char*>(base)};
    int32_t* tri_v = c.take<int32_t>((size_t)12 * cap_large);
    int4* tri_nm = c.take<int4>((size_t)16 * cap_large);
    rast::FrameScratch s;
    s.rv = c.take<float4>((size_t)16 * (nv > 0 ? nv : 1));
    s.keys = c.take<unsigned long long>((size_t)8 * npx);
    s.large = c.take<rast::BinnedTri>(sizeof(rast::BinnedTri) * (size_t)cap_large);
    s.counters = c.take<uint32_t>(4 * counter_words);
    s.tile_offset = c.take<uint32_t>(4 * 2 * ((size_t)n_tiles + 1));
    s.stats = c.take<unsigned long long>(sizeof(unsigned long long) * rast::kStatWords);
    uint32_t* check = c.take<uint32_t>(256);
    s.entries = c.take<uint32_t>((size_t)4 * cap_entries);
    s.cap_large = cap_large;
    s.cap_entries = cap_entries;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // What must start at zero: the index-check word, the counters and the statistics.
    if ((e = cudaMemsetAsync(check, 0, sizeof(uint32_t), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(s.counters, 0, 4 * counter_words, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(s.stats, 0, sizeof(unsigned long long) * rast::kStatWords, st)) != cudaSuccess)
        return fail(RAST_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    if (ntri > 0) {
        k_check_indices<<<(unsigned)((ntri + 255) / 256 < 65536 ? (ntri + 255) / 256 : 65536), 256, 0, st>>>(
            d_tris, ntri, nv, nn, nmat, check);
        uint32_t bad = 0;
        if ((e = cudaMemcpyAsync(&bad, check, sizeof bad, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return fail(RAST_ERR_CUDA, std::string("index check: ") + cudaGetErrorString(e));
        if (bad) return fail(RAST_ERR_BAD_INDEX, "a triangle refers to a vertex, normal or material that does not exist");
        if (rast::launch_split_triangles(d_tris, ntri, tri_v, tri_nm, st) < 0)
            return fail(RAST_ERR_CUDA, "split triangles launch failed");
    }
    if (rast::launch_arm_keys(s.keys, npx, (flags & RAST_CLEAR) != 0, st) < 0)
        return fail(RAST_ERR_CUDA, "arm keys launch failed");

    rast::DeviceMesh mesh;
    mesh.pos = d_pos;
    mesh.tri_v = tri_v;
    mesh.tri_nm = tri_nm;
    mesh.nrm = d_nrm;
    mesh.kd = d_kd;
    mesh.nv = nv;
    mesh.ntri = ntri;
    mesh.nn = nn;
    mesh.nmat = nmat;

    rast::DrawParams p;
    std::memcpy(p.camera.m, camera, sizeof p.camera.m);
    std::memcpy(p.normal.m, normal, sizeof p.normal.m);
    p.width = width;
    p.height = height;
    p.flags = flags;
    // the context path's defaults (rast_create): whole-row items on the per-triangle path
    p.small_max = 4096;
    p.tile = tile;
    p.row_chunk = 32;
    // after a bin overflow the resolve pass writes nothing: the caller's buffers stay as they were
    p.keep_outputs_on_overflow = true;
    p.tiles_x = tiles_x;
    p.tiles_y = tiles_y;
    int n_sm = 1;
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n_sm < 1) n_sm = 1;
    p.n_sm = n_sm;
    p.nl = nl;
    p.lights = d_lights7;
    p.rgb = d_rgb_planar;
    p.depth = d_depth;
    p.tri_id = d_tri_id;
    if (rast::launch_draw(mesh, s, p, st) < 0)
        return fail(RAST_ERR_CUDA, std::string("launch draw: ") + cudaGetErrorString(cudaGetLastError()));

    // Device-side conditions (a bin pool the fixed array cannot grow, a failed check).
    uint32_t status = 0;
    if ((e = cudaMemcpyAsync(&status, s.counters + 1, sizeof status, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(RAST_ERR_CUDA, std::string("draw: ") + cudaGetErrorString(e));
    if (status & (rast::STATUS_BIN_OVERFLOW | rast::STATUS_LARGE_OVERFLOW))
        return fail(RAST_ERR_BIN_OVERFLOW,
                    "the frame needs more tile-bin entries than the fixed array provides; the frame, depth and "
                    "triangle-id buffers were left unchanged");
    if (status) return fail(RAST_ERR_INTERNAL, "device status " + std::to_string(status));
    return RAST_OK;
}
