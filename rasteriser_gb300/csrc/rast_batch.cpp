// Batched drawing: many frames (different meshes, sizes, transforms and light rigs) enqueued on
// several streams ("lanes") of one context, optionally recorded once into a CUDA graph that is
// then launched as a whole; and the autotuner that picks tile size, per-triangle-path limit, row
// chunk and bin capacity for such a batch by timing it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "rast_context.h"

using namespace rast;

namespace {

const DeviceMesh* mesh_of(rast_ctx* c, int32_t id) {
    if (id == 0) return c->has_mesh ? &c->mesh : nullptr;
    if (id < 0 || (size_t)id > c->meshes.size()) return nullptr;
    return &c->meshes[(size_t)id - 1]->dm;
}

void drop_graph(rast_ctx* c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
    c->graph_key.clear();
}

uint32_t tiles_of(const rast_ctx* c, const rast_frame_desc& f) {
    return ((f.width + c->tile - 1) / c->tile) * ((f.height + c->tile - 1) / c->tile);
}

// Creates the lanes and sizes each one's scratch for the largest of the frames it will draw.
rast_status prepare_lanes(rast_ctx* c, const rast_frame_desc* frames, int32_t n, int32_t lanes) {
    while ((int32_t)c->lanes.size() < lanes) {
        std::unique_ptr<Lane> l(new Lane());
        RAST_CUDA(c, cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking));
        RAST_CUDA(c, cudaEventCreateWithFlags(&l->done, cudaEventDisableTiming));
        c->lanes.push_back(std::move(l));
    }
    if (!c->fork_ev) RAST_CUDA(c, cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
    for (int32_t li = 0; li < lanes; ++li) {
        Lane& L = *c->lanes[li];
        int64_t nv = 1, ntri = 1, npx = 1, tiles = 1;
        for (int32_t i = li; i < n; i += lanes) {
            const DeviceMesh* m = mesh_of(c, frames[i].mesh);
            nv = std::max(nv, m->nv);
            ntri = std::max(ntri, m->ntri);
            npx = std::max(npx, (int64_t)frames[i].width * frames[i].height);
            tiles = std::max<int64_t>(tiles, tiles_of(c, frames[i]));
        }
        const void* before[6] = {L.rv.ptr, L.keys.ptr, L.large.ptr, L.counters.ptr, L.tile_offset.ptr, L.entries.ptr};
        RAST_CUDA(c, L.rv.reserve(sizeof(float4) * (size_t)nv));
        RAST_CUDA(c, L.keys.reserve(sizeof(unsigned long long) * (size_t)npx));
        L.cap_large = std::max(L.cap_large, ntri);
        RAST_CUDA(c, L.large.reserve(sizeof(BinnedTri) * (size_t)L.cap_large));
        RAST_CUDA(c, L.counters.reserve(sizeof(uint32_t) * (kCounterHeader + 2 * (size_t)tiles)));
        RAST_CUDA(c, L.tile_offset.reserve(sizeof(uint32_t) * 2 * ((size_t)tiles + 1)));
        if (L.cap_entries == 0)
            L.cap_entries = c->bin_capacity > 0 ? c->bin_capacity : std::max<int64_t>(1 << 20, 2 * ntri);
        RAST_CUDA(c, L.entries.reserve(sizeof(uint32_t) * (size_t)L.cap_entries));
        const void* after[6] = {L.rv.ptr, L.keys.ptr, L.large.ptr, L.counters.ptr, L.tile_offset.ptr, L.entries.ptr};
        if (std::memcmp(before, after, sizeof before) != 0) drop_graph(c);
    }
    RAST_CUDA(c, c->batch_stats.reserve(sizeof(unsigned long long) * kStatWords * (size_t)std::max(n, 1)));
    return RAST_OK;
}

// Enqueues the batch: fork the lanes off the context stream, frame i on lane i % lanes, join.
rast_status enqueue_batch(rast_ctx* c, const rast_frame_desc* frames, int32_t n, int32_t lanes) {
    RAST_CUDA(c, cudaMemsetAsync(c->batch_stats.ptr, 0, sizeof(unsigned long long) * kStatWords * (size_t)n,
                                 c->stream));
    RAST_CUDA(c, cudaEventRecord(c->fork_ev, c->stream));
    for (int32_t li = 0; li < lanes; ++li) RAST_CUDA(c, cudaStreamWaitEvent(c->lanes[li]->stream, c->fork_ev, 0));
    std::vector<bool> first(lanes, true);
    for (int32_t i = 0; i < n; ++i) {
        const rast_frame_desc& f = frames[i];
        const int32_t li = i % lanes;
        Lane& L = *c->lanes[li];
        const uint32_t tiles_x = (f.width + c->tile - 1) / c->tile, tiles_y = (f.height + c->tile - 1) / c->tile;
        const uint32_t n_tiles = tiles_x * tiles_y;
        uint32_t* counters = L.counters.as<uint32_t>();
        const size_t words = kCounterHeader + 2 * (size_t)n_tiles;
        if (first[li]) {
            RAST_CUDA(c, cudaMemsetAsync(counters, 0, sizeof(uint32_t) * words, L.stream));
            first[li] = false;
        } else {
            // Keep the status words [1..3] of earlier frames on this lane; clear the rest.
            RAST_CUDA(c, cudaMemsetAsync(counters, 0, sizeof(uint32_t), L.stream));
            RAST_CUDA(c, cudaMemsetAsync(counters + 4, 0, sizeof(uint32_t) * (words - 4), L.stream));
        }
        const int64_t npx = (int64_t)f.width * f.height;
        if (rast::launch_arm_keys(L.keys.as<unsigned long long>(), npx, (f.flags & RAST_CLEAR) != 0, L.stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "arm keys");
        FrameScratch s;
        s.rv = L.rv.as<float4>();
        s.keys = L.keys.as<unsigned long long>();
        s.large = L.large.as<BinnedTri>();
        s.counters = counters;
        s.tile_offset = L.tile_offset.as<uint32_t>();
        s.entries = L.entries.as<uint32_t>();
        s.stats = c->batch_stats.as<unsigned long long>() + (size_t)kStatWords * i;
        s.cap_large = L.cap_large;
        s.cap_entries = L.cap_entries;
        DrawParams p;
        std::memcpy(p.camera.m, f.camera, sizeof p.camera.m);
        std::memcpy(p.normal.m, f.normal, sizeof p.normal.m);
        p.width = f.width;
        p.height = f.height;
        p.flags = f.flags;
        p.small_max = c->small_max;
        p.tile = c->tile;
        p.row_chunk = c->row_chunk;
        p.tile_threads = c->tile_threads;
        p.chained = false;
        p.tiles_x = tiles_x;
        p.tiles_y = tiles_y;
        p.n_sm = c->n_sm;
        p.nl = f.nl;
        p.lights = f.d_lights7;
        p.rgb = f.d_rgb_planar;
        p.depth = f.d_depth;
        p.tri_id = f.d_tri_id;
        if (rast::launch_draw(*mesh_of(c, f.mesh), s, p, L.stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "launch draw");
    }
    for (int32_t li = 0; li < lanes; ++li) {
        RAST_CUDA(c, cudaEventRecord(c->lanes[li]->done, c->lanes[li]->stream));
        RAST_CUDA(c, cudaStreamWaitEvent(c->stream, c->lanes[li]->done, 0));
    }
    return RAST_OK;
}

std::vector<unsigned char> batch_key(const rast_ctx* c, const rast_frame_desc* frames, int32_t n, int32_t lanes) {
    std::vector<unsigned char> k((const unsigned char*)frames, (const unsigned char*)(frames + n));
    const int64_t extra[8] = {n, lanes, c->tile, c->small_max, c->row_chunk, c->tile_threads,
                              (int64_t)(uintptr_t)c->stream, (int64_t)(uintptr_t)c->batch_stats.ptr};
    k.insert(k.end(), (const unsigned char*)extra, (const unsigned char*)(extra + 8));
    return k;
}

}  // namespace

extern "C" rast_status rast_add_mesh(rast_ctx* c, const float* pos, int64_t nv, const float* nrm, int64_t nn,
                                     const float* uv, int64_t nuv, const int32_t* tris, int64_t ntri, const float* kd,
                                     int32_t nmat, int32_t* mesh_id) {
    if (!c || !mesh_id) return RAST_ERR_INVALID_ARG;
    if (nv < 0 || nn < 0 || nuv < 0 || ntri < 0 || nmat < 0) return fail(c, RAST_ERR_INVALID_ARG, "negative count");
    if ((nv && !pos) || (nn && !nrm) || (nuv && !uv) || (ntri && !tris) || (nmat && !kd))
        return fail(c, RAST_ERR_INVALID_ARG, "null array with a nonzero count");
    std::string msg;
    rast_status st = check_index(tris, ntri, nv, nn, nuv, nmat, msg);
    if (st != RAST_OK) return fail(c, st, msg);
    DeviceGuard g(c->device);
    std::unique_ptr<MeshBuf> m(new MeshBuf());
    RAST_CUDA(c, m->pos.reserve(sizeof(float) * 3 * (size_t)std::max<int64_t>(nv, 1)));
    RAST_CUDA(c, m->nrm.reserve(sizeof(float) * 3 * (size_t)std::max<int64_t>(nn, 1)));
    RAST_CUDA(c, m->kd.reserve(sizeof(float) * 3 * (size_t)std::max<int32_t>(nmat, 1)));
    RAST_CUDA(c, m->tris10.reserve(sizeof(int32_t) * 10 * (size_t)std::max<int64_t>(ntri, 1)));
    RAST_CUDA(c, m->tri_v.reserve(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(ntri, 1)));
    RAST_CUDA(c, m->tri_nm.reserve(sizeof(int4) * (size_t)std::max<int64_t>(ntri, 1)));
    if (nv) RAST_CUDA(c, cudaMemcpy(m->pos.ptr, pos, sizeof(float) * 3 * nv, cudaMemcpyHostToDevice));
    if (nn) RAST_CUDA(c, cudaMemcpy(m->nrm.ptr, nrm, sizeof(float) * 3 * nn, cudaMemcpyHostToDevice));
    if (nmat) RAST_CUDA(c, cudaMemcpy(m->kd.ptr, kd, sizeof(float) * 3 * nmat, cudaMemcpyHostToDevice));
    if (ntri) {
        RAST_CUDA(c, cudaMemcpy(m->tris10.ptr, tris, sizeof(int32_t) * 10 * ntri, cudaMemcpyHostToDevice));
        if (rast::launch_split_triangles(m->tris10.as<int32_t>(), ntri, m->tri_v.as<int32_t>(), m->tri_nm.as<int4>(),
                                         c->stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "split triangles");
        RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    m->dm.pos = m->pos.as<float>();
    m->dm.tri_v = m->tri_v.as<int32_t>();
    m->dm.tri_nm = m->tri_nm.as<int4>();
    m->dm.nrm = m->nrm.as<float>();
    m->dm.kd = m->kd.as<float>();
    m->dm.nv = nv;
    m->dm.ntri = ntri;
    m->dm.nn = nn;
    m->dm.nmat = nmat;
    c->meshes.push_back(std::move(m));
    *mesh_id = (int32_t)c->meshes.size();
    return RAST_OK;
}

extern "C" rast_status rast_draw_batch(rast_ctx* c, const rast_frame_desc* frames, int32_t n, int32_t lanes,
                                       uint32_t batch_flags) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (n < 1 || !frames || lanes < 1 || lanes > 64) return fail(c, RAST_ERR_INVALID_ARG, "bad frame or lane count");
    for (int32_t i = 0; i < n; ++i) {
        const rast_frame_desc& f = frames[i];
        if (!mesh_of(c, f.mesh)) return fail(c, RAST_ERR_NO_MESH, "frame " + std::to_string(i) + ": no such mesh");
        if (f.width == 0 || f.height == 0 || f.width > kMaxDim || f.height > kMaxDim)
            return fail(c, RAST_ERR_INVALID_ARG, "frame " + std::to_string(i) + ": size out of range");
        if (!f.d_rgb_planar || !f.d_depth || f.nl < 0 || f.nl > kMaxLights || (f.nl && !f.d_lights7))
            return fail(c, RAST_ERR_INVALID_ARG, "frame " + std::to_string(i) + ": bad buffers or lights");
    }
    lanes = std::min(lanes, n);
    DeviceGuard g(c->device);
    rast_status st = prepare_lanes(c, frames, n, lanes);
    if (st != RAST_OK) return st;
    c->batch_frames = n;
    c->last_launches = 0;
    c->last_in_place = false;
    if (!(batch_flags & RAST_BATCH_GRAPH)) return enqueue_batch(c, frames, n, lanes);

    std::vector<unsigned char> key = batch_key(c, frames, n, lanes);
    if (!c->graph_exec || key != c->graph_key) {
        drop_graph(c);
        RAST_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        st = enqueue_batch(c, frames, n, lanes);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (st != RAST_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
        const cudaError_t ei = cudaGraphInstantiate(&c->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            c->graph_exec = nullptr;
            return cuda_fail(c, ei, "cudaGraphInstantiate");
        }
        c->graph_key = std::move(key);
    }
    RAST_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream));
    return RAST_OK;
}

extern "C" rast_status rast_get_batch_stats(rast_ctx* c, uint64_t* out) {
    if (!c || !out) return RAST_ERR_INVALID_ARG;
    if (c->batch_frames <= 0) return fail(c, RAST_ERR_INVALID_ARG, "no batch drawn");
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<unsigned long long> s((size_t)kStatWords * c->batch_frames);
    RAST_CUDA(c, cudaMemcpy(s.data(), c->batch_stats.ptr, sizeof(unsigned long long) * s.size(), cudaMemcpyDeviceToHost));
    for (int32_t f = 0; f < c->batch_frames; ++f)
        for (int i = 0; i < 8; ++i) {
            uint64_t v = 0;
            for (int k = 0; k < kStatSlots; ++k) v += s[(size_t)kStatWords * f + ((size_t)i * kStatSlots + k) * kSlotWords];
            out[8 * f + i] = v;
        }
    return RAST_OK;
}

// Reads and clears the status words of the lanes; grows their bin pools after an overflow.
rast_status rast::collect_batch_status(rast_ctx* c) {
    rast_status result = RAST_OK;
    for (auto& lp : c->lanes) {
        Lane& L = *lp;
        if (!L.counters.ptr) continue;
        uint32_t w[3] = {0, 0, 0};
        RAST_CUDA(c, cudaMemcpy(w, L.counters.as<uint32_t>() + 1, sizeof w, cudaMemcpyDeviceToHost));
        if (!w[0]) continue;
        const uint32_t zero[3] = {0, 0, 0};
        RAST_CUDA(c, cudaMemcpy(L.counters.as<uint32_t>() + 1, zero, sizeof zero, cudaMemcpyHostToDevice));
        if (w[0] & STATUS_BIN_OVERFLOW) {
            // Grow to what the largest frame of the batch needed, with a quarter in reserve.
            int64_t need = 0;
            if (c->batch_frames > 0) {
                std::vector<uint64_t> st((size_t)8 * c->batch_frames);
                if (rast_get_batch_stats(c, st.data()) == RAST_OK)
                    for (int32_t f = 0; f < c->batch_frames; ++f) need = std::max<int64_t>(need, (int64_t)st[8 * f + 5]);
            }
            L.cap_entries = std::max<int64_t>(need + need / 4, 2 * L.cap_entries);
            RAST_CUDA(c, L.entries.reserve(sizeof(uint32_t) * (size_t)L.cap_entries));
            drop_graph(c);
            result = fail(c, RAST_ERR_BIN_OVERFLOW, "a lane's tile-bin pool overflowed; it was grown, draw again");
        } else if (result == RAST_OK) {
            result = fail(c, RAST_ERR_INTERNAL, "device check " + std::to_string(w[1]) + " failed (detail " +
                                                    std::to_string(w[2]) + ")");
        }
    }
    return result;
}

extern "C" rast_status rast_autotune(rast_ctx* c, const rast_frame_desc* frames, int32_t n, int32_t lanes,
                                     int32_t repeats, int64_t out[5]) {
    if (!c || !out || repeats < 1) return RAST_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    const uint32_t tiles[3] = {8, 16, 32};
    const uint32_t smalls[3] = {256, 1024, 4096};
    const uint32_t chunks[3] = {4, 8, 32};
    const uint32_t threads[4] = {64, 128, 256, 512};
    cudaEvent_t t0, t1;
    RAST_CUDA(c, cudaEventCreate(&t0));
    RAST_CUDA(c, cudaEventCreate(&t1));
    float best = 1e30f;
    uint32_t bt = c->tile, bs = c->small_max, bc = c->row_chunk, bth = c->tile_threads;
    rast_status st = RAST_OK;
    // the batch's time with the context's current options (they are the ones being tried)
    auto time_batch = [&](float& ms) -> rast_status {
        rast_status s = RAST_OK;
        // the first run records the graph and settles the bin pools
        for (int attempt = 0; attempt < 4; ++attempt) {
            s = rast_draw_batch(c, frames, n, lanes, RAST_BATCH_GRAPH);
            if (s != RAST_OK) return s;
            RAST_CUDA(c, cudaStreamSynchronize(c->stream));
            s = collect_batch_status(c);
            if (s != RAST_ERR_BIN_OVERFLOW) break;
        }
        if (s != RAST_OK) return s;
        RAST_CUDA(c, cudaEventRecord(t0, c->stream));
        for (int r = 0; r < repeats; ++r) {
            s = rast_draw_batch(c, frames, n, lanes, RAST_BATCH_GRAPH);
            if (s != RAST_OK) return s;
        }
        RAST_CUDA(c, cudaEventRecord(t1, c->stream));
        RAST_CUDA(c, cudaEventSynchronize(t1));
        RAST_CUDA(c, cudaEventElapsedTime(&ms, t0, t1));
        return RAST_OK;
    };
    // stage 1: tile size, per-triangle limit and row chunk, with the default threads per tile
    c->tile_threads = 0;
    for (uint32_t t : tiles)
        for (uint32_t sm : smalls)
            for (uint32_t ch : chunks) {
                c->tile = t;
                c->small_max = sm;
                c->row_chunk = ch;
                float ms = 0.f;
                if ((st = time_batch(ms)) != RAST_OK) goto done;
                if (ms < best) {
                    best = ms;
                    bt = t;
                    bs = sm;
                    bc = ch;
                    bth = 0;
                }
            }
    // stage 2: threads per tile for the fastest of those (tile 8 has one choice)
    c->tile = bt;
    c->small_max = bs;
    c->row_chunk = bc;
    if (bt != 8)
        for (uint32_t th : threads) {
            if (th == 512 && bt != 32) continue;
            c->tile_threads = th;
            float ms = 0.f;
            if ((st = time_batch(ms)) != RAST_OK) goto done;
            if (ms < best) {
                best = ms;
                bth = th;
            }
        }
done:
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    c->tile = bt;
    c->small_max = bs;
    c->row_chunk = bc;
    c->tile_threads = bth;
    drop_graph(c);
    if (st != RAST_OK) return st;
    int64_t cap = 0;
    for (auto& lp : c->lanes) cap = std::max(cap, lp->cap_entries);
    out[0] = bt;
    out[1] = bs;
    out[2] = bc;
    out[3] = cap;
    out[4] = bth ? bth : std::min<uint32_t>(bt * bt, 256u);
    return RAST_OK;
}
