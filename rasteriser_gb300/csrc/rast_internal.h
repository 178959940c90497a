// Internal interface between the host side of librast (rast_api.cpp) and its kernels
// (rast_kernels.cu). Not installed; the public interface is include/rast.h.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace rast {

// Raster-space vertex of the reference (geometry.cpp:135-142): x, y in pixels, NDC z, 1/w_clip.
// Stored as float4 so a gather is one 16-byte load.

// One triangle on the binned path: everything the per-tile raster needs, 64 bytes.
struct alignas(16) BinnedTri {
    float x0, y0, x1, y1;   // raster xy of vertices 0, 1
    float x2, y2, z0, z1;   // raster xy of vertex 2, NDC z of vertices 0, 1
    float z2, area, thr, sgn;  // NDC z of vertex 2; barycentric denominator; early-reject bound
    uint32_t tri, tl, br, pad; // triangle index; bounding box corners packed as x | y << 16
};

struct Mat4 { float m[16]; };  // column major, m[c*4 + r]

// Statistics counters. Each counter is spread over kStatSlots slots, kSlotWords 64-bit words
// (128 bytes) apart; warps add into slot (warp id mod kStatSlots), so no counter is a single hot
// address and no kernel needs a block barrier to reduce them. The host sums the slots.
constexpr int kStatCounters = 8;
constexpr int kStatSlots = 32;
constexpr int kSlotWords = 16;
constexpr int kStatWords = kStatCounters * kStatSlots * kSlotWords;

enum StatIndex : int {
    STAT_FRONT = 0, STAT_TESTED = 1, STAT_INSIDE = 2, STAT_WRITTEN = 3,
    STAT_BINNED_TRIS = 4, STAT_BIN_ENTRIES = 5, STAT_LAUNCHES = 6, STAT_HOST_IN_PLACE = 7
};

// Device status word bits (counters[1]); counters[2] and [3] hold the code and detail of the
// first failed internal check.
enum StatusBits : uint32_t {
    STATUS_BIN_OVERFLOW = 1u, STATUS_LARGE_OVERFLOW = 2u, STATUS_CHECK_FAILED = 4u,
    STATUS_SHADE_TIMEOUT = 8u  // the learned shader gave up waiting for a tensor-core MMA
};

// Words of FrameScratch::counters before the per-tile counts:
//   [0] binned triangles   [1] status bits   [2] first failed check   [3] its detail
//   [4] next tile-raster work item           [5..7] unused
constexpr int kCounterHeader = 8;

// Binned triangles per tile-raster work item.
constexpr int kTileChunk = 64;

struct DeviceMesh {
    const float* pos = nullptr;      // nv * 3
    const int32_t* tri_v = nullptr;  // ntri * 3 vertex indices
    const int4* tri_nm = nullptr;    // ntri: normal indices 0..2, material
    const float* nrm = nullptr;      // nn * 3
    const float* kd = nullptr;       // nmat * 3
    const float* vcol = nullptr;     // nv * 3 per-vertex albedo, or null
    // textures (null when no material has one): per material the offset of its normalised texels
    // in tex (-1: none) and its width, height; the uvs and the triangles' uv indices
    const float* tex = nullptr;
    const long long* tex_off = nullptr;
    const int2* tex_wh = nullptr;
    const float* uv = nullptr;       // nuv * 2
    const int32_t* tris10 = nullptr; // ntri * 10, the Triangle records (uv indices at 6..8)
    int64_t nv = 0, ntri = 0, nn = 0;
    int32_t nmat = 0;
};

// Per-draw scratch owned by the context.
struct FrameScratch {
    float4* rv = nullptr;               // nv raster vertices
    unsigned long long* keys = nullptr; // W*H packed (order-preserving depth << 32 | triangle)
    BinnedTri* large = nullptr;         // binned triangles, capacity cap_large
    uint32_t* counters = nullptr;       // kCounterHeader words, n_tiles counts, n_tiles cursors
    uint32_t* tile_offset = nullptr;    // n_tiles + 1 entry offsets, then n_tiles + 1 work-item offsets
    uint32_t* entries = nullptr;        // bin entries, capacity cap_entries
    unsigned long long* stats = nullptr;  // kStatWords
    int64_t cap_large = 0, cap_entries = 0;
    // Cleared by the frame's first kernel when nonzero / set (the caller then skips its own
    // clears): the first clear_counter_words words of counters, stats, and shade_stats.
    uint32_t clear_counter_words = 0;
    bool clear_stats = false;
    bool clear_shade_stats = false;
    // deferred shading (DrawParams::shader != 0)
    float4* gbuf = nullptr;             // 2 float4 per record: (normal xyz, albedo r), (albedo gb, pixel, 0)
    uint32_t* gbuf_count = nullptr;     // records per block of 1024 pixels
    uint32_t* shade_index = nullptr;    // kShadeIndexWords(blocks): the tiles of the shading pass
    unsigned long long* shade_stats = nullptr;  // kShadeStats counters of the learned shader
};

// Deferred shading. The resolve pass stores the winning fragments of each block of 1024 pixels
// in the block's records (block * 1024 + i, raster order) with the block's count; the last block
// to finish lists the shading tiles (rast_tiles.cuh), up to 128 records of one block each.
constexpr int kShadeTile = 128;
constexpr int kShadeBlock = 1024;
// shade_index layout: [0] fragments, [1] tiles, [2..3] unused, [4 .. 4 + blocks] the exclusive
// prefix of the blocks' record counts (blocks + 1 words), then, from the next multiple of 4 words,
// one 16-byte descriptor per tile (at most 8 tiles per block's worth of records).
#ifdef __CUDACC__
__host__ __device__
#endif
inline int64_t kShadeTileDescWord(int64_t blocks) { return (5 + blocks + 3) / 4 * 4; }
inline int64_t kShadeIndexWords(int64_t blocks) { return kShadeTileDescWord(blocks) + 4 * 8 * blocks; }
// counters word counting the resolve blocks that finished (deferred shading)
constexpr int kResolveTicket = 5;
// shade_stats: [0] tiles shaded by the MLP, [1] tiles sent to the exact shader, [2] fragments
// checked, [3] largest checked error (float bits of the channel error in 1/255 units).
constexpr int kShadeStats = 4;

struct DrawParams {
    Mat4 camera, normal;
    uint32_t width, height;
    uint32_t flags;
    uint32_t small_max;     // bounding boxes up to this many pixels take the per-triangle path
    uint32_t tile;          // tile edge: 8, 16, 32
    uint32_t row_chunk;     // pixels per work item of the per-triangle path: 4, 8 or 32 (whole rows)
    uint32_t tile_threads = 0;  // threads per tile of the tile raster: 64, 128, 256, 512 (tile 32 only);
                                // 0 or a value the tile edge does not take: min(tile^2, 256)
    bool chained = true;    // launch the frame's kernels after the first as programmatic dependents
                            // (off for batches, whose lanes fill the SMs with each other's work)
    cudaEvent_t before_resolve = nullptr;  // when set, the resolve pass waits for it (the colour
                                           // input of a host draw, copied beside the first passes)
    bool keep_outputs_on_overflow = false;  // the resolve pass writes nothing after a bin-pool
                                            // overflow, so a redraw starts from the same buffers
    uint32_t tiles_x, tiles_y;
    int32_t n_sm;           // streaming multiprocessors of the device
    int32_t nl;
    const float* lights;    // device, nl * 7
    uint8_t* rgb;           // device planar RGB8
    float* depth;           // device
    uint32_t* tri_id;       // device, nullable
    int32_t shader = 0;     // 0 exact in the resolve pass, 1 exact deferred, 2 learned deferred
    const void* mlp = nullptr;  // shader 2: the device image of the weights (MlpNet)
    int32_t mlp_net = 0;        // shader 2: its network (kMlpNetCompact or kMlpNetWide)
    int32_t mlp_samples = 2;    // shader 2: fragments per tile checked against the exact shader
    float mlp_bound = 0.5f;     // shader 2: largest checked channel error (1/255 units) a tile may have
    bool mlp_stall_test = false;  // shader 2, test only: the first MMA wait gives up (RAST_OPT_TEST_SHADE_STALL)
};

// The depth view (rast_view.cu): min / max of n depths into mm[0..1] (order keys), then the bytes.
// Returns the number of launches, or -1.
int launch_depth_view(const float* depth, int64_t n, uint32_t* mm, uint8_t* out, int n_sm, cudaStream_t stream);

// The deferred shading pass over the resolve's fragment records (rast_shade.cu): the exact or
// learned shading kernel over the tiles the resolve listed. Returns the number of launches, or -1.
int launch_shade(const FrameScratch& s, const DrawParams& p, int64_t blocks, cudaStream_t stream);

// Launches every kernel of one draw on `stream`. Returns the number of kernel launches made
// (memsets excluded) or -1 with cudaGetLastError() set.
// With `events` (9 events, nullable) it records events[0] before the first kernel and
// events[1..8] after key arming, vertex, setup, scan, scatter, tile raster, resolve and the
// deferred shading pass.
int launch_draw(const DeviceMesh& mesh, const FrameScratch& s, const DrawParams& p, cudaStream_t stream,
                cudaEvent_t* events = nullptr);

// Fills keys[0, n) with the key of a pixel no fragment has reached: for clear mode the key that
// only fragments nearer than 1.0 beat, else a key above every fragment's. The resolve pass re-arms
// every key it reads for its own mode, so this is needed only for fresh keys or a change of mode.
int launch_arm_keys(unsigned long long* keys, int64_t n, bool clear, cudaStream_t stream);

// Sets the text rast_last_error(NULL) returns on this thread.
void set_thread_error(const std::string& msg);

// Splits the reference's Triangle records (10 int32 each) into tri_v and tri_nm on the device.
int launch_split_triangles(const int32_t* tris10, int64_t ntri, int32_t* tri_v, int4* tri_nm, cudaStream_t stream);

}  // namespace rast
