// Host side of librast's C ABI (include/rast.h): contexts, validation, device buffers and the
// orchestration of one draw. The kernels are in rast_kernels.cu.
#include <cuda.h>  // pointer attribute names; the driver function is reached through cudart
#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>


#include "rast_context.h"

namespace rast {
thread_local std::string g_create_error;
void set_thread_error(const std::string& msg) { g_create_error = msg; }
}  // namespace rast

using namespace rast;

namespace {

uint32_t tile_shift(uint32_t tile) { return tile == 8 ? 3u : (tile == 16 ? 4u : 5u); }

// Whether the current device reaches ordinary pageable host memory through the host's page tables
// (address translation services, as on Grace): kernels may then use such buffers in place.
bool pageable_reachable() {
    static int known[64];  // per device: 0 unknown, 1 no, 2 yes
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (known[dev] == 0) {
        int ats = 0;
        known[dev] = cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
                                 cudaSuccess &&
                             ats
                         ? 2
                         : 1;
    }
    return known[dev] == 2;
}

// Makes every page of [p, p + bytes) present and writable in the host's page tables
// (MADV_POPULATE_WRITE), so the device, translating host addresses, never has to fault a page in.
// False when the host cannot (an older kernel, a read-only or unmapped range): the caller then
// copies the buffer instead.
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23  // Linux UAPI value
#endif
bool populate_writable(const void* p, size_t bytes) {
    static const uintptr_t page = (uintptr_t)sysconf(_SC_PAGESIZE);
    if (page == 0 || (page & (page - 1)) != 0) return false;
    const uintptr_t b = (uintptr_t)p & ~(page - 1), e = ((uintptr_t)p + bytes + page - 1) & ~(page - 1);
    return madvise(reinterpret_cast<void*>(b), e - b, MADV_POPULATE_WRITE) == 0;
}

// The device address of [p, p + bytes) when the kernels can use the range in place, else nullptr:
// the whole range lies in one page-locked host allocation that the device maps (cudaHostAlloc,
// cudaHostRegister, torch's pinned memory; both ends in the same CUDA allocation, one buffer id,
// mapped contiguously), or it is ordinary pageable memory, the device translates host addresses
// (pageable_reachable) and its pages could be made present and writable (populate_writable).
void* mapped_host_range(const void* p, size_t bytes) {
    using GetAttrs = CUresult (*)(unsigned int, CUpointer_attribute*, void**, CUdeviceptr);
    static const GetAttrs get = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttributes", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return reinterpret_cast<GetAttrs>(fn);
    }();
    if (!get || !p || bytes == 0) return nullptr;
    {
        unsigned int type = 0;
        CUpointer_attribute a0 = CU_POINTER_ATTRIBUTE_MEMORY_TYPE;
        void* d0 = &type;
        // a pointer of no CUDA allocation (pageable memory) reads back type 0
        if (get(1, &a0, &d0, (CUdeviceptr)(uintptr_t)p) == CUDA_SUCCESS && type == 0)
            return pageable_reachable() && populate_writable(p, bytes) ? const_cast<void*>(p) : nullptr;
    }
    struct Ends {
        unsigned int type = 0;
        unsigned long long id = 0;
        void* dev = nullptr;
    } e[2];
    const CUdeviceptr at[2] = {(CUdeviceptr)(uintptr_t)p, (CUdeviceptr)(uintptr_t)p + (CUdeviceptr)(bytes - 1)};
    for (int i = 0; i < 2; ++i) {
        // A pointer of no CUDA allocation (pageable memory) reads back type 0 and buffer id 0.
        CUpointer_attribute attrs[3] = {CU_POINTER_ATTRIBUTE_MEMORY_TYPE, CU_POINTER_ATTRIBUTE_BUFFER_ID,
                                        CU_POINTER_ATTRIBUTE_DEVICE_POINTER};
        void* data[3] = {&e[i].type, &e[i].id, &e[i].dev};
        if (get(3, attrs, data, at[i]) != CUDA_SUCCESS || e[i].type != CU_MEMORYTYPE_HOST || !e[i].dev) return nullptr;
    }
    if (e[0].id == 0 || e[0].id != e[1].id || (uintptr_t)e[1].dev - (uintptr_t)e[0].dev != bytes - 1) return nullptr;
    return e[0].dev;
}

// Sizes the per-draw scratch for a width x height frame.
rast_status ensure_scratch(rast_ctx* c, uint32_t w, uint32_t h, uint32_t tiles) {
    const int64_t npx = (int64_t)w * h;
    RAST_CUDA(c, c->rv.reserve(sizeof(float4) * (size_t)std::max<int64_t>(c->mesh.nv, 1)));
    if (c->keys.bytes < sizeof(unsigned long long) * (size_t)npx) c->keys_armed = false;
    RAST_CUDA(c, c->keys.reserve(sizeof(unsigned long long) * (size_t)npx));
    c->cap_large = std::max<int64_t>(c->mesh.ntri, 1);
    RAST_CUDA(c, c->large.reserve(sizeof(rast::BinnedTri) * (size_t)c->cap_large));
    RAST_CUDA(c, c->counters.reserve(sizeof(uint32_t) * (rast::kCounterHeader + 2 * (size_t)tiles)));
    RAST_CUDA(c, c->tile_offset.reserve(sizeof(uint32_t) * 2 * ((size_t)tiles + 1)));
    if (c->cap_entries == 0)
        c->cap_entries = c->bin_capacity > 0 ? c->bin_capacity : std::max<int64_t>(1 << 20, 2 * c->mesh.ntri);
    RAST_CUDA(c, c->entries.reserve(sizeof(uint32_t) * (size_t)c->cap_entries));
    RAST_CUDA(c, c->stats.reserve(sizeof(unsigned long long) * rast::kStatWords));
    if (c->shader != RAST_SHADER_EXACT) {
        const int64_t blocks = (npx + rast::kShadeBlock - 1) / rast::kShadeBlock;
        RAST_CUDA(c, c->gbuf.reserve(2 * sizeof(float4) * (size_t)blocks * rast::kShadeBlock));
        RAST_CUDA(c, c->gbuf_count.reserve(sizeof(uint32_t) * (size_t)blocks));
        RAST_CUDA(c, c->shade_index.reserve(sizeof(uint32_t) * (size_t)rast::kShadeIndexWords(blocks)));
        RAST_CUDA(c, c->shade_stats.reserve(sizeof(unsigned long long) * rast::kShadeStats));
    }
    return RAST_OK;
}

rast_status enqueue_draw(rast_ctx* c, const float* camera, const float* normal, uint32_t w, uint32_t h,
                         uint32_t flags, uint8_t* d_rgb, float* d_depth, uint32_t* d_ids) {
    if (!c->has_mesh) return fail(c, RAST_ERR_NO_MESH, "no mesh uploaded");
    if (c->shader == RAST_SHADER_LEARNED) {
        if (!c->mlp_ready) return fail(c, RAST_ERR_INVALID_ARG, "learned shading needs trained or loaded weights");
        if (c->mlp_nl != c->nl || c->mlp_lights_hash != rast::lights_hash(c->lights_host.data(), c->nl))
            return fail(c, RAST_ERR_INVALID_ARG, "the MLP was trained for another light rig");
    }
    const uint32_t tiles_x = (w + c->tile - 1) / c->tile, tiles_y = (h + c->tile - 1) / c->tile;
    const uint32_t n_tiles = tiles_x * tiles_y;
    rast_status st = ensure_scratch(c, w, h, n_tiles);
    if (st != RAST_OK) return st;
    const int64_t npx = (int64_t)w * h;
    const bool clear = (flags & RAST_CLEAR) != 0;
    if (!c->keys_armed || c->keys_px != npx || c->keys_clear != clear) {
        if (rast::launch_arm_keys(c->keys.as<unsigned long long>(), npx, clear, c->stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "arm keys");
    }
    rast::FrameScratch s;
    s.rv = c->rv.as<float4>();
    s.keys = c->keys.as<unsigned long long>();
    s.large = c->large.as<rast::BinnedTri>();
    s.counters = c->counters.as<uint32_t>();
    s.tile_offset = c->tile_offset.as<uint32_t>();
    s.entries = c->entries.as<uint32_t>();
    s.stats = c->stats.as<unsigned long long>();
    s.cap_large = c->cap_large;
    s.cap_entries = c->cap_entries;
    // the counters (header, tile counts and cursors) and statistics start at zero: the frame's
    // first kernel clears them
    s.clear_counter_words = (uint32_t)(rast::kCounterHeader + 2 * (size_t)n_tiles);
    s.clear_stats = true;
    if (c->shader != RAST_SHADER_EXACT) {
        s.gbuf = c->gbuf.as<float4>();
        s.gbuf_count = c->gbuf_count.as<uint32_t>();
        s.shade_index = c->shade_index.as<uint32_t>();
        s.shade_stats = c->shade_stats.as<unsigned long long>();
        s.clear_shade_stats = true;
    }

    rast::DrawParams p;
    std::memcpy(p.camera.m, camera, sizeof p.camera.m);
    std::memcpy(p.normal.m, normal, sizeof p.normal.m);
    p.width = w;
    p.height = h;
    p.flags = flags;
    p.small_max = c->small_max;
    p.tile = c->tile;
    p.row_chunk = c->row_chunk;
    p.tile_threads = c->tile_threads;
    p.before_resolve = c->before_resolve;
    p.keep_outputs_on_overflow = c->keep_outputs;
    p.tiles_x = tiles_x;
    p.tiles_y = tiles_y;
    p.n_sm = c->n_sm;
    p.nl = c->nl;
    p.lights = c->lights.as<float>();
    p.rgb = d_rgb;
    p.depth = d_depth;
    p.tri_id = d_ids;
    p.shader = c->shader;
    p.mlp = c->mlp_image.ptr;
    p.mlp_net = c->mlp_net;
    p.mlp_samples = c->mlp_samples;
    p.mlp_bound = (float)c->mlp_bound_milli * 1e-3f;
    p.mlp_stall_test = c->test_shade_stall;
    if (c->timing && !c->ev_made) {
        for (auto& e : c->ev) RAST_CUDA(c, cudaEventCreate(&e));
        c->ev_made = true;
    }
    const int n = rast::launch_draw(c->mesh, s, p, c->stream, c->timing ? c->ev : nullptr);
    c->ev_recorded = c->timing;
    if (n < 0) return cuda_fail(c, cudaGetLastError(), "launch draw");
    c->replay_valid = p.shader != RAST_SHADER_EXACT;
    if (c->replay_valid) {
        c->replay_s = s;
        c->replay_p = p;
        c->replay_p.before_resolve = nullptr;
        c->replay_blocks = (npx + rast::kShadeBlock - 1) / rast::kShadeBlock;
    }
    c->last_launches = (uint64_t)n;
    c->last_in_place = false;
    c->keys_armed = true;  // the resolve pass re-arms every key it reads
    c->keys_clear = clear;
    c->keys_px = npx;
    return RAST_OK;
}

// Reads the device status word and clears it; grows the bin pool after an overflow.
rast_status collect_status(rast_ctx* c) {
    if (!c->counters.ptr) return RAST_OK;
    uint32_t status = 0;
    RAST_CUDA(c, cudaMemcpy(&status, c->counters.as<uint32_t>() + 1, sizeof status, cudaMemcpyDeviceToHost));
    if (status & rast::STATUS_BIN_OVERFLOW) {
        unsigned long long need = 0;
        RAST_CUDA(c, cudaMemcpy(&need,
                                c->stats.as<unsigned long long>() +
                                    (size_t)rast::STAT_BIN_ENTRIES * rast::kStatSlots * rast::kSlotWords,
                                sizeof need, cudaMemcpyDeviceToHost));
        c->cap_entries = std::max<int64_t>((int64_t)need + (int64_t)need / 4, 2 * c->cap_entries);
        RAST_CUDA(c, c->entries.reserve(sizeof(uint32_t) * (size_t)c->cap_entries));
        uint32_t zero = 0;
        RAST_CUDA(c, cudaMemcpy(c->counters.as<uint32_t>() + 1, &zero, sizeof zero, cudaMemcpyHostToDevice));
        c->keys_armed = false;
        return fail(c, RAST_ERR_BIN_OVERFLOW, "tile-bin pool overflowed; it was grown to " +
                                                  std::to_string(c->cap_entries) + " entries, draw again");
    }
    if (status & rast::STATUS_SHADE_TIMEOUT) {
        uint32_t zero = 0;
        RAST_CUDA(c, cudaMemcpy(c->counters.as<uint32_t>() + 1, &zero, sizeof zero, cudaMemcpyHostToDevice));
        return fail(c, RAST_ERR_TIMEOUT, "learned shader: a tensor-core MMA did not complete in time");
    }
    if (status & rast::STATUS_CHECK_FAILED) {
        uint32_t w[2] = {0, 0};
        RAST_CUDA(c, cudaMemcpy(w, c->counters.as<uint32_t>() + 2, sizeof w, cudaMemcpyDeviceToHost));
        return fail(c, RAST_ERR_INTERNAL, "device check " + std::to_string(w[0]) + " failed (detail " +
                                              std::to_string(w[1]) + ")");
    }
    if (status) return fail(c, RAST_ERR_INTERNAL, "device status " + std::to_string(status));
    return RAST_OK;
}

bool valid_matrix_args(const float* camera, const float* normal) { return camera && normal; }

}  // namespace

extern "C" {

int rast_abi_version(void) { return RAST_ABI_VERSION; }

const char* rast_status_string(rast_status s) {
    switch (s) {
        case RAST_OK: return "ok";
        case RAST_ERR_INVALID_ARG: return "invalid argument";
        case RAST_ERR_BAD_INDEX: return "index out of range";
        case RAST_ERR_NO_MESH: return "no mesh";
        case RAST_ERR_CUDA: return "CUDA error";
        case RAST_ERR_OUT_OF_MEMORY: return "out of device memory";
        case RAST_ERR_BIN_OVERFLOW: return "tile-bin pool overflow";
        case RAST_ERR_TIMEOUT: return "device wait timed out";
        case RAST_ERR_NO_DEVICE: return "no CUDA device";
        case RAST_ERR_INTERNAL: return "device consistency check failed";
    }
    return "unknown status";
}

const char* rast_last_error(const rast_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

rast_status rast_create(rast_ctx** out, int device) {
    if (!out) return fail(nullptr, RAST_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(nullptr, RAST_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    if (device < 0 || device >= n) return fail(nullptr, RAST_ERR_INVALID_ARG, "device ordinal out of range");
    DeviceGuard g(device);
    rast_ctx* c = new rast_ctx();
    c->device = device;
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(nullptr, RAST_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    if (cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || c->n_sm < 1)
        c->n_sm = 1;
    *out = c;
    return RAST_OK;
}

void rast_destroy(rast_ctx* c) {
    if (!c) return;
    DeviceGuard g(c->device);
    cudaStreamSynchronize(c->stream);
    for (DevBuf* b : {&c->pos, &c->tris10, &c->tri_v, &c->tri_nm, &c->nrm, &c->kd, &c->lights, &c->rv, &c->keys,
                      &c->large, &c->counters, &c->tile_offset, &c->entries, &c->stats, &c->d_rgb, &c->d_depth,
                      &c->d_ids, &c->vcol, &c->uvbuf, &c->texbuf, &c->tex_offbuf, &c->tex_whbuf, &c->gbuf, &c->gbuf_count, &c->shade_index, &c->shade_stats, &c->view_mm,
                      &c->mlp_image})
        b->release();
    if (c->ev_made)
        for (auto& e : c->ev) cudaEventDestroy(e);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    for (auto& l : c->lanes) {
        for (DevBuf* b : {&l->rv, &l->keys, &l->large, &l->counters, &l->tile_offset, &l->entries}) b->release();
        if (l->done) cudaEventDestroy(l->done);
        if (l->stream) cudaStreamDestroy(l->stream);
    }
    for (auto& m : c->meshes)
        for (DevBuf* b : {&m->pos, &m->tris10, &m->tri_v, &m->tri_nm, &m->nrm, &m->kd}) b->release();
    c->batch_stats.release();
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    for (DevBuf* b : {&c->d_rgb_in, &c->d_depth_in}) b->release();
    if (c->ev_depth_in) cudaEventDestroy(c->ev_depth_in);
    if (c->ev_rgb_in) cudaEventDestroy(c->ev_rgb_in);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

rast_status rast_set_stream(rast_ctx* c, void* stream) {
    if (!c) return RAST_ERR_INVALID_ARG;
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    return RAST_OK;
}

void* rast_get_stream(const rast_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

rast_status rast_upload_mesh(rast_ctx* c, const float* pos, int64_t nv, const float* nrm, int64_t nn, const float* uv,
                             int64_t nuv, const int32_t* tris, int64_t ntri, const float* kd, int32_t nmat) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (nv < 0 || nn < 0 || nuv < 0 || ntri < 0 || nmat < 0) return fail(c, RAST_ERR_INVALID_ARG, "negative count");
    if ((nv && !pos) || (nn && !nrm) || (nuv && !uv) || (ntri && !tris) || (nmat && !kd))
        return fail(c, RAST_ERR_INVALID_ARG, "null array with a nonzero count");
    std::string msg;
    rast_status st = check_index(tris, ntri, nv, nn, nuv, nmat, msg);
    if (st != RAST_OK) return fail(c, st, msg);
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    c->has_mesh = false;
    c->has_vcol = false;
    c->mesh.vcol = nullptr;
    if (c->graph_exec) {  // a recorded batch may refer to the mesh being replaced
        cudaGraphExecDestroy(c->graph_exec);
        c->graph_exec = nullptr;
        c->graph_key.clear();
    }
    RAST_CUDA(c, c->pos.reserve(sizeof(float) * 3 * (size_t)std::max<int64_t>(nv, 1)));
    RAST_CUDA(c, c->nrm.reserve(sizeof(float) * 3 * (size_t)std::max<int64_t>(nn, 1)));
    RAST_CUDA(c, c->kd.reserve(sizeof(float) * 3 * (size_t)std::max<int32_t>(nmat, 1)));
    RAST_CUDA(c, c->tris10.reserve(sizeof(int32_t) * 10 * (size_t)std::max<int64_t>(ntri, 1)));
    RAST_CUDA(c, c->tri_v.reserve(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(ntri, 1)));
    RAST_CUDA(c, c->tri_nm.reserve(sizeof(int4) * (size_t)std::max<int64_t>(ntri, 1)));
    if (nv) RAST_CUDA(c, cudaMemcpyAsync(c->pos.ptr, pos, sizeof(float) * 3 * nv, cudaMemcpyHostToDevice, c->stream));
    if (nn) RAST_CUDA(c, cudaMemcpyAsync(c->nrm.ptr, nrm, sizeof(float) * 3 * nn, cudaMemcpyHostToDevice, c->stream));
    if (nmat) RAST_CUDA(c, cudaMemcpyAsync(c->kd.ptr, kd, sizeof(float) * 3 * nmat, cudaMemcpyHostToDevice, c->stream));
    if (ntri) {
        RAST_CUDA(c, cudaMemcpyAsync(c->tris10.ptr, tris, sizeof(int32_t) * 10 * ntri, cudaMemcpyHostToDevice, c->stream));
        if (rast::launch_split_triangles(c->tris10.as<int32_t>(), ntri, c->tri_v.as<int32_t>(), c->tri_nm.as<int4>(),
                                         c->stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "split triangles");
    }
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    RAST_CUDA(c, c->uvbuf.reserve(sizeof(float) * 2 * (size_t)std::max<int64_t>(nuv, 1)));
    if (nuv) RAST_CUDA(c, cudaMemcpy(c->uvbuf.ptr, uv, sizeof(float) * 2 * nuv, cudaMemcpyHostToDevice));
    c->tex_host.assign((size_t)nmat, std::vector<float>());
    c->tex_dims.assign((size_t)nmat, make_int2(0, 0));
    c->mesh.tex = nullptr;
    c->mesh.tex_off = nullptr;
    c->mesh.tex_wh = nullptr;
    c->mesh.uv = c->uvbuf.as<float>();
    c->mesh.tris10 = c->tris10.as<int32_t>();
    c->mesh.pos = c->pos.as<float>();
    c->mesh.tri_v = c->tri_v.as<int32_t>();
    c->mesh.tri_nm = c->tri_nm.as<int4>();
    c->mesh.nrm = c->nrm.as<float>();
    c->mesh.kd = c->kd.as<float>();
    c->mesh.nv = nv;
    c->mesh.ntri = ntri;
    c->mesh.nn = nn;
    c->mesh.nmat = nmat;
    c->has_mesh = true;
    c->cap_entries = 0;  // re-sized for the new mesh on the next draw
    return RAST_OK;
}

rast_status rast_upload_vertex_albedo(rast_ctx* c, const float* rgb3, int64_t nv) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (!c->has_mesh) return fail(c, RAST_ERR_NO_MESH, "no mesh uploaded");
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!rgb3 && nv == 0) {
        c->has_vcol = false;
        c->mesh.vcol = nullptr;
        return RAST_OK;
    }
    if (!rgb3 || nv != c->mesh.nv) return fail(c, RAST_ERR_INVALID_ARG, "vertex albedo needs one rgb per mesh vertex");
    RAST_CUDA(c, c->vcol.reserve(sizeof(float) * 3 * (size_t)std::max<int64_t>(nv, 1)));
    if (nv) RAST_CUDA(c, cudaMemcpy(c->vcol.ptr, rgb3, sizeof(float) * 3 * nv, cudaMemcpyHostToDevice));
    c->has_vcol = true;
    c->mesh.vcol = c->vcol.as<float>();
    return RAST_OK;
}

rast_status rast_upload_texture(rast_ctx* c, int32_t material, const float* texels, uint32_t w, uint32_t h,
                                uint32_t channels) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (!c->has_mesh) return fail(c, RAST_ERR_NO_MESH, "no mesh uploaded");
    if (material < 0 || material >= c->mesh.nmat) return fail(c, RAST_ERR_INVALID_ARG, "material out of range");
    if (texels && (w == 0 || h == 0 || w > 65536 || h > 65536 || channels < 3 || channels > 4))
        return fail(c, RAST_ERR_INVALID_ARG, "texture needs 3 or 4 channels and 1..65536 pixels a side");
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<float>& t = c->tex_host[(size_t)material];
    if (!texels) {
        t.clear();
        c->tex_dims[(size_t)material] = make_int2(0, 0);
    } else {
        // material.h:21, diffuse_texture.normalize(0.f, 1.f): CImg takes the smallest and largest
        // value over every channel (with < and >), fills with 0 when they are equal, leaves an image
        // already spanning 0..1 as it is, and otherwise maps v to (v - m) / (M - m) * (1 - 0) + 0.
        const size_t plane = (size_t)w * h, n = plane * channels;
        float m = texels[0], M = texels[0];
        for (size_t i = 1; i < n; ++i) {
            if (texels[i] < m) m = texels[i];
            if (texels[i] > M) M = texels[i];
        }
        t.assign(3 * plane, 0.f);
        if (!(m == M))
            for (size_t i = 0; i < 3 * plane; ++i)
                t[i] = (m != 0.f || M != 1.f) ? (texels[i] - m) / (M - m) * (1.f - 0.f) + 0.f : texels[i];
        c->tex_dims[(size_t)material] = make_int2((int)w, (int)h);
    }
    // device tables
    std::vector<long long> off((size_t)c->mesh.nmat, -1);
    size_t total = 0;
    for (size_t i = 0; i < c->tex_host.size(); ++i)
        if (!c->tex_host[i].empty()) {
            off[i] = (long long)total;
            total += c->tex_host[i].size();
        }
    if (total == 0) {
        c->mesh.tex = nullptr;
        c->mesh.tex_off = nullptr;
        c->mesh.tex_wh = nullptr;
        return RAST_OK;
    }
    RAST_CUDA(c, c->texbuf.reserve(sizeof(float) * total));
    RAST_CUDA(c, c->tex_offbuf.reserve(sizeof(long long) * off.size()));
    RAST_CUDA(c, c->tex_whbuf.reserve(sizeof(int2) * off.size()));
    for (size_t i = 0; i < c->tex_host.size(); ++i)
        if (off[i] >= 0)
            RAST_CUDA(c, cudaMemcpy(c->texbuf.as<float>() + off[i], c->tex_host[i].data(),
                                    sizeof(float) * c->tex_host[i].size(), cudaMemcpyHostToDevice));
    RAST_CUDA(c, cudaMemcpy(c->tex_offbuf.ptr, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice));
    RAST_CUDA(c, cudaMemcpy(c->tex_whbuf.ptr, c->tex_dims.data(), sizeof(int2) * off.size(), cudaMemcpyHostToDevice));
    c->mesh.tex = c->texbuf.as<float>();
    c->mesh.tex_off = c->tex_offbuf.as<long long>();
    c->mesh.tex_wh = c->tex_whbuf.as<int2>();
    return RAST_OK;
}

rast_status rast_set_lights(rast_ctx* c, const float* lights7, int32_t n) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (n < 0 || n > kMaxLights || (n && !lights7)) return fail(c, RAST_ERR_INVALID_ARG, "bad light count or pointer");
    DeviceGuard g(c->device);
    RAST_CUDA(c, c->lights.reserve(sizeof(float) * 7 * (size_t)std::max(n, 1)));
    if (n)
        RAST_CUDA(c, cudaMemcpyAsync(c->lights.ptr, lights7, sizeof(float) * 7 * n, cudaMemcpyHostToDevice, c->stream));
    // The host array may be reused by the caller as soon as this returns.
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    c->nl = n;
    c->lights_host.assign(lights7, lights7 + 7 * (size_t)n);
    return RAST_OK;
}

rast_status rast_draw_device(rast_ctx* c, const float camera[16], const float normal[16], uint32_t w, uint32_t h,
                             uint32_t flags, uint8_t* d_rgb, float* d_depth, uint32_t* d_ids) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (!valid_matrix_args(camera, normal) || !d_rgb || !d_depth)
        return fail(c, RAST_ERR_INVALID_ARG, "null matrix or buffer");
    if (w == 0 || h == 0 || w > kMaxDim || h > kMaxDim) return fail(c, RAST_ERR_INVALID_ARG, "frame size out of range");
    DeviceGuard g(c->device);
    return enqueue_draw(c, camera, normal, w, h, flags, d_rgb, d_depth, d_ids);
}

rast_status rast_draw(rast_ctx* c, const float camera[16], const float normal[16], uint32_t w, uint32_t h,
                      uint32_t flags, uint8_t* rgb, float* depth, uint32_t* ids) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (!valid_matrix_args(camera, normal) || !rgb || !depth)
        return fail(c, RAST_ERR_INVALID_ARG, "null matrix or buffer");
    if (w == 0 || h == 0 || w > kMaxDim || h > kMaxDim) return fail(c, RAST_ERR_INVALID_ARG, "frame size out of range");
    DeviceGuard g(c->device);
    const size_t npx = (size_t)w * h;
    const bool rmw = !(flags & RAST_CLEAR);
    if (!c->h_status) RAST_CUDA(c, cudaMallocHost(&c->h_status, sizeof(uint32_t)));
    // Host buffers the device reaches (page-locked memory it maps; pageable memory where it
    // translates host addresses) are used in place: the resolve pass reads the incoming depth
    // where a fragment landed and writes the frame's pixels (read-modify-write: only the winners;
    // deferred shading then writes their colour) straight into the host buffers, so no
    // frame-sized copy crosses the link. After a bin-pool overflow nothing is written, and the
    // redraw starts from the same buffers.
    if (c->host_in_place) {
        uint8_t* hr = static_cast<uint8_t*>(mapped_host_range(rgb, 3 * npx));
        float* hd = static_cast<float*>(mapped_host_range(depth, sizeof(float) * npx));
        uint32_t* hi = ids ? static_cast<uint32_t*>(mapped_host_range(ids, sizeof(uint32_t) * npx)) : nullptr;
        if (hr && hd && (!ids || hi)) {
            for (int attempt = 0; attempt < 3; ++attempt) {
                c->keep_outputs = true;
                rast_status st = enqueue_draw(c, camera, normal, w, h, flags, hr, hd, hi);
                c->keep_outputs = false;
                if (st != RAST_OK) return st;
                c->last_in_place = true;
                RAST_CUDA(c, cudaMemcpyAsync(c->h_status, c->counters.as<uint32_t>() + 1, sizeof(uint32_t),
                                             cudaMemcpyDeviceToHost, c->stream));
                RAST_CUDA(c, cudaStreamSynchronize(c->stream));
                if (*c->h_status == 0u) return RAST_OK;
                st = collect_status(c);
                if (st == RAST_ERR_BIN_OVERFLOW) continue;  // pool grown; the buffers are untouched
                return st;
            }
            return fail(c, RAST_ERR_BIN_OVERFLOW, "tile-bin pool still overflowing after regrowth");
        }
    }
    // Otherwise the buffers are copied through device memory.
    RAST_CUDA(c, c->d_rgb.reserve(3 * npx));
    RAST_CUDA(c, c->d_depth.reserve(sizeof(float) * npx));
    if (ids) RAST_CUDA(c, c->d_ids.reserve(sizeof(uint32_t) * npx));
    if (rmw) {
        RAST_CUDA(c, c->d_rgb_in.reserve(3 * npx));
        RAST_CUDA(c, c->d_depth_in.reserve(sizeof(float) * npx));
        if (!c->copy_stream) RAST_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        if (!c->ev_depth_in) RAST_CUDA(c, cudaEventCreateWithFlags(&c->ev_depth_in, cudaEventDisableTiming));
        if (!c->ev_rgb_in) RAST_CUDA(c, cudaEventCreateWithFlags(&c->ev_rgb_in, cudaEventDisableTiming));
    }
    for (int attempt = 0; attempt < 3; ++attempt) {
        // The inputs are needed only by the resolve pass (the incoming depth each winner must beat,
        // the colour of the pixels nothing wins), so they are uploaded on the copy stream while the
        // first passes run. Both are also kept on the device, so a redraw after a bin overflow
        // starts from them again.
        if (rmw && attempt == 0) {
            RAST_CUDA(c, cudaEventRecord(c->ev_depth_in, c->stream));  // after earlier work on the stream
            RAST_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->ev_depth_in, 0));
            RAST_CUDA(c, cudaMemcpyAsync(c->d_depth.ptr, depth, sizeof(float) * npx, cudaMemcpyHostToDevice,
                                         c->copy_stream));
            RAST_CUDA(c, cudaMemcpyAsync(c->d_rgb.ptr, rgb, 3 * npx, cudaMemcpyHostToDevice, c->copy_stream));
            RAST_CUDA(c, cudaMemcpyAsync(c->d_depth_in.ptr, c->d_depth.ptr, sizeof(float) * npx,
                                         cudaMemcpyDeviceToDevice, c->copy_stream));
            RAST_CUDA(c, cudaMemcpyAsync(c->d_rgb_in.ptr, c->d_rgb.ptr, 3 * npx, cudaMemcpyDeviceToDevice, c->copy_stream));
            RAST_CUDA(c, cudaEventRecord(c->ev_rgb_in, c->copy_stream));
        } else if (rmw) {
            RAST_CUDA(c, cudaMemcpyAsync(c->d_depth.ptr, c->d_depth_in.ptr, sizeof(float) * npx,
                                         cudaMemcpyDeviceToDevice, c->stream));
            RAST_CUDA(c, cudaMemcpyAsync(c->d_rgb.ptr, c->d_rgb_in.ptr, 3 * npx, cudaMemcpyDeviceToDevice, c->stream));
            RAST_CUDA(c, cudaEventRecord(c->ev_rgb_in, c->stream));
        }
        c->before_resolve = rmw ? c->ev_rgb_in : nullptr;
        rast_status st = enqueue_draw(c, camera, normal, w, h, flags, c->d_rgb.as<uint8_t>(), c->d_depth.as<float>(),
                                      ids ? c->d_ids.as<uint32_t>() : nullptr);
        c->before_resolve = nullptr;
        if (st != RAST_OK) return st;
        // the outputs and the status word, read back in one wait
        RAST_CUDA(c, cudaMemcpyAsync(rgb, c->d_rgb.ptr, 3 * npx, cudaMemcpyDeviceToHost, c->stream));
        RAST_CUDA(c, cudaMemcpyAsync(depth, c->d_depth.ptr, sizeof(float) * npx, cudaMemcpyDeviceToHost, c->stream));
        if (ids) RAST_CUDA(c, cudaMemcpyAsync(ids, c->d_ids.ptr, sizeof(uint32_t) * npx, cudaMemcpyDeviceToHost, c->stream));
        RAST_CUDA(c, cudaMemcpyAsync(c->h_status, c->counters.as<uint32_t>() + 1, sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, c->stream));
        RAST_CUDA(c, cudaStreamSynchronize(c->stream));
        if (*c->h_status == 0u) return RAST_OK;
        st = collect_status(c);
        if (st == RAST_ERR_BIN_OVERFLOW) continue;  // pool grown; draw again from the same inputs
        return st;
    }
    return fail(c, RAST_ERR_BIN_OVERFLOW, "tile-bin pool still overflowing after regrowth");
}

rast_status rast_sync(rast_ctx* c) {
    if (!c) return RAST_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    const rast_status st = collect_status(c);
    const rast_status sb = c->lanes.empty() ? RAST_OK : collect_batch_status(c);
    return st != RAST_OK ? st : sb;
}

rast_status rast_time_shading(rast_ctx* c, int32_t repeats, float* us_per_pass) {
    if (!c || !us_per_pass || repeats < 1 || repeats > 100000) return RAST_ERR_INVALID_ARG;
    if (!c->replay_valid) return fail(c, RAST_ERR_INVALID_ARG, "the last draw did not shade in a separate pass");
    DeviceGuard g(c->device);
    cudaEvent_t e0, e1;
    RAST_CUDA(c, cudaEventCreate(&e0));
    RAST_CUDA(c, cudaEventCreate(&e1));
    rast_status st = RAST_OK;
    float ms = 0.f;
    if (cudaEventRecord(e0, c->stream) != cudaSuccess) st = cuda_fail(c, cudaGetLastError(), "event");
    for (int32_t i = 0; st == RAST_OK && i < repeats; ++i)
        if (rast::launch_shade(c->replay_s, c->replay_p, c->replay_blocks, c->stream) < 0)
            st = cuda_fail(c, cudaGetLastError(), "shading pass");
    if (st == RAST_OK && (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        st = cuda_fail(c, cudaGetLastError(), "timing");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != RAST_OK) return st;
    *us_per_pass = 1000.f * ms / (float)repeats;
    return collect_status(c);
}

rast_status rast_get_stats(rast_ctx* c, uint64_t out[8]) {
    if (!c || !out) return RAST_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(uint64_t) * 8);
    if (!c->stats.ptr) return RAST_OK;
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<unsigned long long> s(rast::kStatWords);
    RAST_CUDA(c, cudaMemcpy(s.data(), c->stats.ptr, sizeof(unsigned long long) * s.size(), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 8; ++i)
        for (int k = 0; k < rast::kStatSlots; ++k) out[i] += s[((size_t)i * rast::kStatSlots + k) * rast::kSlotWords];
    out[rast::STAT_LAUNCHES] = c->last_launches;
    out[rast::STAT_HOST_IN_PLACE] = c->last_in_place ? 1 : 0;
    return RAST_OK;
}

rast_status rast_set_option(rast_ctx* c, int option, int64_t value) {
    if (!c) return RAST_ERR_INVALID_ARG;
    switch (option) {
        case RAST_OPT_SMALL_MAX_PIXELS:
            if (value < 1 || value > 65536) return fail(c, RAST_ERR_INVALID_ARG, "small_max out of range");
            c->small_max = (uint32_t)value;
            return RAST_OK;
        case RAST_OPT_TILE_SIZE:
            if (value != 8 && value != 16 && value != 32) return fail(c, RAST_ERR_INVALID_ARG, "tile must be 8, 16 or 32");
            c->tile = (uint32_t)value;
            return RAST_OK;
        case RAST_OPT_ROW_CHUNK:
            if (value != 4 && value != 8 && value != 32)
                return fail(c, RAST_ERR_INVALID_ARG, "row chunk must be 4, 8 or 32");
            c->row_chunk = (uint32_t)value;
            return RAST_OK;
        case RAST_OPT_STAGE_TIMING:
            if (value != 0 && value != 1) return fail(c, RAST_ERR_INVALID_ARG, "stage timing is 0 or 1");
            c->timing = value == 1;
            return RAST_OK;
        case RAST_OPT_BIN_CAPACITY:
            if (value < 0 || value > (int64_t)1 << 31) return fail(c, RAST_ERR_INVALID_ARG, "bin capacity out of range");
            c->bin_capacity = value;
            c->cap_entries = 0;
            return RAST_OK;
        case RAST_OPT_SHADER:
            if (value != RAST_SHADER_EXACT && value != RAST_SHADER_EXACT_DEFERRED && value != RAST_SHADER_LEARNED)
                return fail(c, RAST_ERR_INVALID_ARG, "unknown shader");
            c->shader = (int32_t)value;
            return RAST_OK;
        case RAST_OPT_MLP_SAMPLES:
            if (value < 0 || value > 4) return fail(c, RAST_ERR_INVALID_ARG, "MLP check samples must be 0..4");
            c->mlp_samples = (int32_t)value;
            return RAST_OK;
        case RAST_OPT_MLP_BOUND_MILLI:
            if (value < 0 || value > 255000) return fail(c, RAST_ERR_INVALID_ARG, "MLP bound out of range");
            c->mlp_bound_milli = (int32_t)value;
            return RAST_OK;
        case RAST_OPT_TILE_THREADS:
            if (value != 0 && value != 64 && value != 128 && value != 256 && value != 512)
                return fail(c, RAST_ERR_INVALID_ARG, "threads per tile must be 0, 64, 128, 256 or 512");
            c->tile_threads = (uint32_t)value;
            return RAST_OK;
        case RAST_OPT_TEST_SHADE_STALL:
            if (value != 0 && value != 1) return fail(c, RAST_ERR_INVALID_ARG, "shade stall test is 0 or 1");
            c->test_shade_stall = value == 1;
            return RAST_OK;
        case RAST_OPT_HOST_IN_PLACE:
            if (value != 0 && value != 1) return fail(c, RAST_ERR_INVALID_ARG, "host in place is 0 or 1");
            c->host_in_place = value == 1;
            return RAST_OK;
        case RAST_OPT_MLP_NETWORK:
            if (value != rast::kMlpNetCompact && value != rast::kMlpNetWide)
                return fail(c, RAST_ERR_INVALID_ARG, "MLP network is 0 (compact) or 1 (wide)");
            c->mlp_train_net = (int32_t)value;
            return RAST_OK;
    }
    return fail(c, RAST_ERR_INVALID_ARG, "unknown option");
}

rast_status rast_get_option(rast_ctx* c, int option, int64_t* value) {
    if (!c || !value) return RAST_ERR_INVALID_ARG;
    switch (option) {
        case RAST_OPT_SMALL_MAX_PIXELS: *value = c->small_max; return RAST_OK;
        case RAST_OPT_TILE_SIZE: *value = c->tile; return RAST_OK;
        case RAST_OPT_BIN_CAPACITY: *value = c->cap_entries ? c->cap_entries : c->bin_capacity; return RAST_OK;
        case RAST_OPT_STAGE_TIMING: *value = c->timing ? 1 : 0; return RAST_OK;
        case RAST_OPT_ROW_CHUNK: *value = c->row_chunk; return RAST_OK;
        case RAST_OPT_SHADER: *value = c->shader; return RAST_OK;
        case RAST_OPT_MLP_SAMPLES: *value = c->mlp_samples; return RAST_OK;
        case RAST_OPT_MLP_BOUND_MILLI: *value = c->mlp_bound_milli; return RAST_OK;
        case RAST_OPT_TEST_SHADE_STALL: *value = c->test_shade_stall ? 1 : 0; return RAST_OK;
        case RAST_OPT_TILE_THREADS: *value = c->tile_threads; return RAST_OK;
        case RAST_OPT_HOST_IN_PLACE: *value = c->host_in_place ? 1 : 0; return RAST_OK;
        case RAST_OPT_MLP_NETWORK: *value = c->mlp_train_net; return RAST_OK;
    }
    return fail(c, RAST_ERR_INVALID_ARG, "unknown option");
}

rast_status rast_get_device_status(rast_ctx* c, uint32_t out[4]) {
    if (!c || !out) return RAST_ERR_INVALID_ARG;
    for (int i = 0; i < 4; ++i) out[i] = 0;
    if (!c->counters.ptr) return RAST_OK;
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    RAST_CUDA(c, cudaMemcpy(out, c->counters.ptr, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return RAST_OK;
}

rast_status rast_get_stage_times(rast_ctx* c, float out_ms[9]) {
    if (!c || !out_ms) return RAST_ERR_INVALID_ARG;
    for (int i = 0; i < 9; ++i) out_ms[i] = 0.f;
    if (!c->ev_recorded) return fail(c, RAST_ERR_INVALID_ARG, "no timed draw (set RAST_OPT_STAGE_TIMING first)");
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaEventSynchronize(c->ev[8]));
    for (int i = 0; i < 8; ++i) RAST_CUDA(c, cudaEventElapsedTime(&out_ms[i], c->ev[i], c->ev[i + 1]));
    RAST_CUDA(c, cudaEventElapsedTime(&out_ms[8], c->ev[0], c->ev[8]));
    return RAST_OK;
}

rast_status rast_depth_to_u8(rast_ctx* c, const float* d_depth, uint32_t w, uint32_t h, uint8_t* d_out) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (!d_depth || !d_out || w == 0 || h == 0 || w > kMaxDim || h > kMaxDim)
        return fail(c, RAST_ERR_INVALID_ARG, "bad depth view arguments");
    DeviceGuard g(c->device);
    RAST_CUDA(c, c->view_mm.reserve(2 * sizeof(uint32_t)));
    if (rast::launch_depth_view(d_depth, (int64_t)w * h, c->view_mm.as<uint32_t>(), d_out, c->n_sm, c->stream) < 0)
        return cuda_fail(c, cudaGetLastError(), "depth view");
    return RAST_OK;
}

rast_status rast_depth_to_u8_host(rast_ctx* c, const float* depth, uint32_t w, uint32_t h, uint8_t* out) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (!depth || !out || w == 0 || h == 0 || w > kMaxDim || h > kMaxDim)
        return fail(c, RAST_ERR_INVALID_ARG, "bad depth view arguments");
    DeviceGuard g(c->device);
    const size_t npx = (size_t)w * h;
    RAST_CUDA(c, c->d_depth.reserve(sizeof(float) * npx));
    RAST_CUDA(c, c->d_rgb.reserve(3 * npx));
    RAST_CUDA(c, cudaMemcpyAsync(c->d_depth.ptr, depth, sizeof(float) * npx, cudaMemcpyHostToDevice, c->stream));
    const rast_status st = rast_depth_to_u8(c, c->d_depth.as<float>(), w, h, c->d_rgb.as<uint8_t>());
    if (st != RAST_OK) return st;
    RAST_CUDA(c, cudaMemcpyAsync(out, c->d_rgb.ptr, npx, cudaMemcpyDeviceToHost, c->stream));
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    return RAST_OK;
}

rast_status rast_spin(rast_ctx* c, const rast_spin_desc* d, uint8_t* last_rgb, float* last_depth, double* seconds) {
    if (!c || !d) return RAST_ERR_INVALID_ARG;
    if (d->width == 0 || d->height == 0 || d->width > kMaxDim || d->height > kMaxDim || d->frames < 1 ||
        d->nl < 0 || d->nl > kMaxLights || (d->nl && !d->lights7))
        return fail(c, RAST_ERR_INVALID_ARG, "bad spin arguments");
    DeviceGuard g(c->device);
    const uint32_t w = d->width, h = d->height;
    const size_t npx = (size_t)w * h;
    float model[16], view[16], mv[16], cam[16], nm[16];
    float angles[3] = {d->angles[0], d->angles[1], d->angles[2]};
    rast_status st = rast_frame_matrices(w, h, d->scale, d->disp, angles, d->fovy_deg, d->z_near, d->z_far, model,
                                         view, mv, cam, nm);
    if (st != RAST_OK) return fail(c, st, "frame matrices");
    std::vector<float> lt(7 * (size_t)std::max(d->nl, 1));
    if (d->nl) {
        st = rast_transform_lights(view, d->lights7, d->nl, lt.data());
        if (st != RAST_OK) return fail(c, st, "lights");
    }
    st = rast_set_lights(c, lt.data(), d->nl);
    if (st != RAST_OK) return st;
    RAST_CUDA(c, c->d_rgb.reserve(3 * npx));
    RAST_CUDA(c, c->d_depth.reserve(sizeof(float) * npx));
    const uint32_t flags = (d->flags & (RAST_WIND_CLOCKWISE | RAST_FLAT)) | RAST_CLEAR;
    const auto t0 = std::chrono::steady_clock::now();
    for (int32_t k = 0; k < d->frames; ++k) {
        angles[1] = d->angles[1] + (float)k * d->step;
        st = rast_frame_matrices(w, h, d->scale, d->disp, angles, d->fovy_deg, d->z_near, d->z_far, model, view, mv,
                                 cam, nm);
        if (st != RAST_OK) return fail(c, st, "frame matrices");
        st = enqueue_draw(c, cam, nm, w, h, flags, c->d_rgb.as<uint8_t>(), c->d_depth.as<float>(), nullptr);
        if (st != RAST_OK) return st;
    }
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    st = collect_status(c);
    if (st != RAST_OK) return st;
    if (last_rgb) RAST_CUDA(c, cudaMemcpy(last_rgb, c->d_rgb.ptr, 3 * npx, cudaMemcpyDeviceToHost));
    if (last_depth) RAST_CUDA(c, cudaMemcpy(last_depth, c->d_depth.ptr, sizeof(float) * npx, cudaMemcpyDeviceToHost));
    if (seconds) *seconds = s;
    return RAST_OK;
}

rast_status rast_get_shade_stats(rast_ctx* c, uint64_t out[4]) {
    if (!c || !out) return RAST_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(uint64_t) * 4);
    if (!c->shade_stats.ptr) return RAST_OK;
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    unsigned long long s[rast::kShadeStats];
    RAST_CUDA(c, cudaMemcpy(s, c->shade_stats.ptr, sizeof s, cudaMemcpyDeviceToHost));
    out[0] = s[0];
    out[1] = s[1];
    out[2] = s[2];
    float e;
    const uint32_t bits = (uint32_t)s[3];
    std::memcpy(&e, &bits, sizeof e);
    out[3] = (uint64_t)((double)e * 1e6 + 0.5);
    return RAST_OK;
}

}  // extern "C"
