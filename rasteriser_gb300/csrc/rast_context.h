// Internal: the context behind the C ABI and the host helpers shared by rast_api.cpp and
// rast_batch.cpp. Not installed.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "rast.h"
#include "rast_internal.h"
#include "rast_mlp.h"

namespace rast {

// A device allocation that grows and never shrinks.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t want) {
        if (want <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};


// A mesh uploaded for batched drawing (rast_add_mesh); mesh 0 is the context's own mesh.
struct MeshBuf {
    DevBuf pos, tris10, tri_v, tri_nm, nrm, kd;
    DeviceMesh dm;
};

// One stream of a batch and the scratch its frames use one after another.
struct Lane {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf rv, keys, large, counters, tile_offset, entries;
    int64_t cap_large = 0, cap_entries = 0;
};

}  // namespace rast

using rast::DevBuf;

struct rast_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;

    // mesh
    DevBuf pos, tris10, tri_v, tri_nm, nrm, kd;
    rast::DeviceMesh mesh;
    bool has_mesh = false;

    // per-vertex albedo (rast_upload_vertex_albedo), nv * 3
    DevBuf vcol;
    bool has_vcol = false;

    // uvs and textures (rast_upload_texture): normalised planes per material, on the device
    // concatenated with per-material offsets and sizes
    DevBuf uvbuf, texbuf, tex_offbuf, tex_whbuf;
    std::vector<std::vector<float>> tex_host;
    std::vector<int2> tex_dims;

    // lights
    DevBuf lights;
    int32_t nl = 0;
    std::vector<float> lights_host;  // the records last set, for the learned shader's rig check

    // per-draw scratch
    DevBuf rv, keys, large, counters, tile_offset, entries, stats;
    int64_t cap_large = 0, cap_entries = 0;
    bool keys_armed = false;  // keys[0, keys_px) hold the armed value of keys_clear's mode
    bool keys_clear = false;
    int64_t keys_px = 0;

    // host-pointer draws stage through these
    DevBuf d_rgb, d_depth, d_ids;
    // host draws: copies of the read-modify-write inputs (for a redraw after a bin overflow), the
    // stream that uploads the colour input beside the first passes, and the status word's landing
    DevBuf d_rgb_in, d_depth_in;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_depth_in = nullptr, ev_rgb_in = nullptr;
    uint32_t* h_status = nullptr;
    cudaEvent_t before_resolve = nullptr;  // set by rast_draw for the draw it enqueues
    bool keep_outputs = false;             // set by rast_draw when the kernels use its host buffers

    // deferred shading
    int32_t shader = 0;           // RAST_SHADER_*
    int32_t mlp_samples = 2;      // RAST_OPT_MLP_SAMPLES
    int32_t mlp_bound_milli = 500;  // RAST_OPT_MLP_BOUND_MILLI
    bool test_shade_stall = false;  // RAST_OPT_TEST_SHADE_STALL
    bool host_in_place = true;      // RAST_OPT_HOST_IN_PLACE
    // the last draw's deferred shading pass, for rast_time_shading
    bool replay_valid = false;
    rast::FrameScratch replay_s;
    rast::DrawParams replay_p;
    int64_t replay_blocks = 0;
    DevBuf gbuf, gbuf_count, shade_index, shade_stats;
    DevBuf view_mm;  // rast_depth_to_u8: the depth range

    // learned shader state (rast_mlp.cpp)
    DevBuf mlp_image;             // the weights' device image (rast::MlpNet), then the check table
    int32_t mlp_net = 0;          // the network of the installed weights (kMlpNetCompact or kMlpNetWide)
    int32_t mlp_train_net = 0;    // RAST_OPT_MLP_NETWORK: the network rast_mlp_train builds
    bool mlp_ready = false;
    uint64_t mlp_lights_hash = 0;
    int32_t mlp_nl = 0;
    float mlp_scale = 1.f;
    float mlp_loss = 0.f;
    std::vector<float> mlp_q;     // rounded parameters of the current weights (MlpNet::kParams)

    // options
    uint32_t small_max = 4096;
    uint32_t tile = 16;
    uint32_t row_chunk = 32;
    uint32_t tile_threads = 0;  // RAST_OPT_TILE_THREADS
    int64_t bin_capacity = 0;  // 0: sized from the mesh

    uint64_t last_launches = 0;
    bool last_in_place = false;     // the last draw wrote rast_draw's host buffers in place
    int n_sm = 1;

    // batched drawing
    std::vector<std::unique_ptr<rast::MeshBuf>> meshes;  // ids 1.., rast_add_mesh
    std::vector<std::unique_ptr<rast::Lane>> lanes;
    DevBuf batch_stats;
    int32_t batch_frames = 0;
    cudaEvent_t fork_ev = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<unsigned char> graph_key;  // the batch the instantiated graph records

    // stage timing
    bool timing = false;
    cudaEvent_t ev[9] = {};
    bool ev_made = false;
    bool ev_recorded = false;
};

namespace rast {

extern thread_local std::string g_create_error;

inline rast_status fail(rast_ctx* c, rast_status s, const std::string& msg) {
    if (c) c->err = msg;
    else g_create_error = msg;
    return s;
}

inline rast_status cuda_fail(rast_ctx* c, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(c, e == cudaErrorMemoryAllocation ? RAST_ERR_OUT_OF_MEMORY : RAST_ERR_CUDA, m);
}

}  // namespace rast

#define RAST_CUDA(ctx, call)                                      \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return rast::cuda_fail((ctx), e_, #call); \
    } while (0)

namespace rast {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

constexpr uint32_t kMaxDim = 32768;
constexpr int32_t kMaxLights = 4096;

inline rast_status check_index(const int32_t* tris, int64_t ntri, int64_t nv, int64_t nn, int64_t nuv, int32_t nmat,
                        std::string& msg) {
    if (ntri >= 0xFFFFFFFFll) {
        msg = "too many triangles (the triangle index must fit in 32 bits)";
        return RAST_ERR_INVALID_ARG;
    }
    for (int64_t i = 0; i < ntri; ++i) {
        const int32_t* t = tris + 10 * i;
        for (int k = 0; k < 3; ++k) {
            if (t[k] < 0 || t[k] >= nv) {
                msg = "triangle " + std::to_string(i) + " vertex index " + std::to_string(t[k]) + " out of range";
                return RAST_ERR_BAD_INDEX;
            }
            if (t[3 + k] < 0 || t[3 + k] >= nn) {
                msg = "triangle " + std::to_string(i) + " normal index " + std::to_string(t[3 + k]) + " out of range";
                return RAST_ERR_BAD_INDEX;
            }
            if (t[6 + k] >= nuv) {
                msg = "triangle " + std::to_string(i) + " uv index " + std::to_string(t[6 + k]) + " out of range";
                return RAST_ERR_BAD_INDEX;
            }
        }
        if (t[9] < 0 || t[9] >= nmat) {
            msg = "triangle " + std::to_string(i) + " material " + std::to_string(t[9]) + " out of range";
            return RAST_ERR_BAD_INDEX;
        }
    }
    return RAST_OK;
}

// Status of the lanes of the last batch (rast_batch.cpp).
rast_status collect_batch_status(rast_ctx* c);

}  // namespace rast
