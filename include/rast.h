/* librast: C ABI of the GB300 (sm_103a) rasteriser hot path.
 *
 * It replaces canmom/rasteriser's per-frame path, draw_frame (drawing.cpp:205-258, declared at
 * headers/drawing.h:16-18), and the geometry.h / shading.h calls it makes. Plain pointers and
 * sizes only; the C++ drop-in (rasteriser_gb300/cpp) and the Python binding
 * (rasteriser_gb300/abi.py) sit on top.
 *
 * Results match the reference exactly: coverage, depth and the index of the triangle that wins
 * each pixel are bit for bit those of the reference's sequential loop (nearest first, then lowest
 * triangle index), and the RGB8 frame is computed with the reference's shading arithmetic.
 *
 * Threading: a context is used by one host thread at a time. Device work of a context runs in
 * order on its stream.
 */
#ifndef RAST_H
#define RAST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAST_ABI_VERSION 1

typedef enum rast_status {
    RAST_OK = 0,
    RAST_ERR_INVALID_ARG = 1,   /* null pointer, zero or oversized frame, negative count */
    RAST_ERR_BAD_INDEX = 2,     /* a triangle refers to a vertex, normal, uv or material that does not exist */
    RAST_ERR_NO_MESH = 3,       /* draw before rast_upload_mesh */
    RAST_ERR_CUDA = 4,          /* a CUDA runtime call failed; rast_last_error has the text */
    RAST_ERR_OUT_OF_MEMORY = 5,
    RAST_ERR_BIN_OVERFLOW = 6,  /* a device draw overflowed the tile-bin pool; the pool has been
                                   grown, draw the frame again */
    RAST_ERR_TIMEOUT = 7,       /* a bounded device-side wait gave up */
    RAST_ERR_NO_DEVICE = 8,
    RAST_ERR_INTERNAL = 9       /* a device-side consistency check failed; the access was skipped
                                   and the frame is not trustworthy (rast_get_device_status) */
} rast_status;

typedef struct rast_ctx rast_ctx;

/* Frame flags. */
#define RAST_WIND_CLOCKWISE 1u /* Args::wind_clockwise (arguments.h:13): front faces have
                                  signed_area_2d <= 0 and shading normals are negated */
#define RAST_CLEAR 2u          /* treat the frame as cleared to 0 and the depth buffer to 1.0
                                  before drawing, as the reference's spin loop does
                                  (renderer.cpp:107-108); the incoming buffers are not read */
#define RAST_FLAT 4u           /* Args::flat (arguments.h:12, readme.md:46): flat shading with
                                  face normals computed in the path. Each triangle's three vertex
                                  normals are replaced by cross(p1 - p0, p2 - p0) of its model-space
                                  positions, which then go through the normal matrix, perspective
                                  interpolation, normalisation and the clockwise flip as vertex
                                  normals do. The mesh's normals are still uploaded and checked but
                                  not read. (The reference parses the flag and never reads it.) */

/* ------------------------------------------------------------------------------------------ */
/* host-side geometry (no device work)                                                         */
/* ------------------------------------------------------------------------------------------ */

/* The per-frame matrices of draw_frame (drawing.cpp:221-229; geometry.cpp:22-33):
 *   model     = transformation_matrix(scale, disp, angles)  = T * Ry * Rx * Rz * S
 *   view      = transformation_matrix(1, (0,0,-3), 0)
 *   modelview = view * model
 *   camera    = perspective(radians(fovy_deg), width/height, z_near, z_far) * modelview
 *   normal    = transpose(inverse(modelview))                (geometry.cpp:101)
 * Each output (nullable) receives 16 floats, column major. disp and angles are xyz; angles are
 * the YXZ Tait-Bryan angles (rx, ry, rz) in radians. The reference fixes fovy / near / far to
 * 45 / 0.1 / 6 (geometry.cpp:30); pass those for an identical camera. */
rast_status rast_frame_matrices(uint32_t width, uint32_t height, float scale, const float disp[3],
                                const float angles[3], float fovy_deg, float z_near, float z_far,
                                float model[16], float view[16], float modelview[16], float camera[16],
                                float normal[16]);

/* Light::transform (geometry.cpp:124-133): trans_dir = normalize(xyz(view * (direction, 0))).
 * lights_in: n records of 7 floats (direction xyz, intensity, colour rgb; light.h:7-14).
 * lights_out: n records of 7 floats with trans_dir in place of direction (may alias lights_in). */
rast_status rast_transform_lights(const float view[16], const float* lights_in, int32_t n, float* lights_out);

/* ------------------------------------------------------------------------------------------ */
/* context                                                                                     */
/* ------------------------------------------------------------------------------------------ */

/* Creates a context on CUDA device `device` with its own non-blocking stream. */
rast_status rast_create(rast_ctx** out, int device);
void rast_destroy(rast_ctx* ctx);

/* Text of the last error on this context (or of the last failed rast_create when ctx is NULL). */
const char* rast_last_error(const rast_ctx* ctx);
const char* rast_status_string(rast_status s);
int rast_abi_version(void);

/* Makes the context launch on `stream` (a created cudaStream_t). NULL restores the context's own
 * stream; the legacy default stream cannot be selected. */
rast_status rast_set_stream(rast_ctx* ctx, void* stream);
void* rast_get_stream(const rast_ctx* ctx);

/* ------------------------------------------------------------------------------------------ */
/* scene data (device resident until replaced)                                                 */
/* ------------------------------------------------------------------------------------------ */

/* Uploads a mesh in the reference's host layouts (the vectors draw_frame receives):
 *   pos: nv * 3 floats (vector<vec3> model_vertices)
 *   nrm: nn * 3 floats (vector<vec3> model_vertnormals)
 *   uv:  nuv * 2 floats (vector<vec2> vertuvs; may be NULL when nuv == 0; read by textures)
 *   tris: ntri * 10 int32, the Triangle layout of face.h:6-13 (vertices[3], normals[3], uvs[3],
 *         material); vector<Triangle>::data() can be passed as is
 *   kd:  nmat * 3 floats, each material's constant albedo (Material::diffuse_colour,
 *        material.h:13; the value Material::sample returns without a texture, material.cpp:24)
 * Every index is checked on the host first. The reference reads out of bounds on a bad index
 * (drawing.cpp:165-173); here such a mesh is refused with RAST_ERR_BAD_INDEX. A uv index < 0
 * means "no uv", as in the reference (drawing.cpp:168). Synchronous. */
rast_status rast_upload_mesh(rast_ctx* ctx, const float* pos, int64_t nv, const float* nrm, int64_t nn,
                             const float* uv, int64_t nuv, const int32_t* tris, int64_t ntri,
                             const float* kd, int32_t nmat);

/* Per-vertex albedo for the uploaded mesh (no counterpart in the reference, whose materials are
 * constant): nv * 3 floats, interpolated perspective-correctly like the normals
 * (drawing.cpp:64-75) and used in place of the material's Kd (Material::sample). nv must equal
 * the mesh's vertex count; rgb3 = NULL with nv = 0 returns to the materials' Kd. A new
 * rast_upload_mesh drops it. Synchronous. */
rast_status rast_upload_vertex_albedo(rast_ctx* ctx, const float* rgb3, int64_t nv);

/* A texture for material `material` of the uploaded mesh (Material(dc, file), material.h:17-22):
 * texels as CImg loads an image, planar (x + y*w + c*w*h, rows top first, e.g. rast_image_load),
 * channels 3 or 4 (the first three are sampled). They are normalised as the reference's Material
 * does (CImg normalize(0, 1) over every channel), and fragments of the material take the texture's
 * colour at their perspective-correct uv (drawing.cpp:135, Material::sample: bilinear, coordinates
 * clamped to the image, v flipped) in place of Kd. A uv index < 0 reads uv (0, 0), as in the
 * reference. texels = NULL removes the texture. Per-vertex albedo, where set, takes precedence.
 * A new rast_upload_mesh drops the textures. Synchronous. */
rast_status rast_upload_texture(rast_ctx* ctx, int32_t material, const float* texels, uint32_t width,
                                uint32_t height, uint32_t channels);

/* Sets the frame's lights: n records of 7 floats (trans_dir xyz, intensity, colour rgb), i.e.
 * already transformed (rast_transform_lights). Shading sums them in this order
 * (shading.cpp:24-34). 0 <= n <= 4096. */
rast_status rast_set_lights(rast_ctx* ctx, const float* lights7, int32_t n);

/* ------------------------------------------------------------------------------------------ */
/* drawing                                                                                     */
/* ------------------------------------------------------------------------------------------ */

/* One frame of draw_frame with HOST buffers (the reference's calling convention); returns when
 * done. Buffers the device reaches are used in place (RAST_OPT_HOST_IN_PLACE, default on):
 * page-locked memory that the device maps (cudaHostAlloc, cudaHostRegister), each buffer within
 * one allocation, and ordinary pageable memory on devices that translate host addresses through
 * the host's page tables (Grace), whose pages are first made present and writable on the host.
 * The kernels then read the incoming depth where a fragment landed and write the pixels they
 * draw over the link. Other buffers are copied in (unless RAST_CLEAR), rendered on the device
 * and copied back. rast_get_stats word 7 says which path the last draw took.
 *   camera, normal: the frame's camera and normal matrices (rast_frame_matrices)
 *   rgb_planar: width*height*3 bytes, planar (x + y*width + c*width*height) as CImg stores
 *               CImg<unsigned char>(W,H,1,3) (renderer.cpp:85); read and written
 *   depth: width*height floats (CImg<float>(W,H,1,1), renderer.cpp:86); read and written; the
 *          incoming value is the depth every fragment must beat (drawing.cpp:119)
 *   tri_id (nullable): width*height uint32, the index of the triangle that wrote each pixel in
 *          this call, or 0xFFFFFFFF
 * Pixels no fragment wins keep their colour and depth. 1 <= width, height <= 32768. Copied inputs
 * are uploaded while the first passes run, and the results and the device status are read back in
 * one wait. A bin overflow is redrawn from the same inputs (kept copies, or in place buffers the
 * overflowed pass left untouched); after any other error the buffers' contents are unspecified. */
rast_status rast_draw(rast_ctx* ctx, const float camera[16], const float normal[16], uint32_t width,
                      uint32_t height, uint32_t flags, uint8_t* rgb_planar, float* depth, uint32_t* tri_id);

/* The same with DEVICE buffers, enqueued on the context's stream and not waited for. */
rast_status rast_draw_device(rast_ctx* ctx, const float camera[16], const float normal[16], uint32_t width,
                             uint32_t height, uint32_t flags, uint8_t* d_rgb_planar, float* d_depth,
                             uint32_t* d_tri_id);

/* Waits for the context's stream; reports device-side conditions of earlier draws
 * (RAST_ERR_BIN_OVERFLOW). */
rast_status rast_sync(rast_ctx* ctx);

/* Counters of the last completed draw (call after rast_sync):
 *   [0] front-facing triangles      [1] bounding-box pixels tested
 *   [2] inside fragments            [3] pixels written
 *   [4] triangles on the binned path [5] tile-bin entries
 *   [6] kernel launches of the draw  [7] 1 when it was a rast_draw that used its host buffers in
 *                                        place (RAST_OPT_HOST_IN_PLACE), else 0 */
rast_status rast_get_stats(rast_ctx* ctx, uint64_t out[8]);

/* Tuning knobs (see rast_set_option keys). Values outside the supported set are refused. */
#define RAST_OPT_SMALL_MAX_PIXELS 1   /* bounding boxes up to this many pixels (default 4096) and
                                         at most 32 pixels wide are rasterised by the per-triangle
                                         path; the others are binned into tiles (1..65536) */
#define RAST_OPT_TILE_SIZE 2          /* tile edge for binning: 8, 16 or 32 */
#define RAST_OPT_BIN_CAPACITY 3       /* initial tile-bin pool, entries */
#define RAST_OPT_STAGE_TIMING 4       /* 1: record CUDA events between the kernels of each draw */
#define RAST_OPT_ROW_CHUNK 5          /* pixels of a bounding-box row per work item of the
                                         per-triangle path: 4 or 8, each pixel's edges evaluated,
                                         or 32 (default): whole rows, the ends of the passing
                                         interval found from the edges' crossings */
#define RAST_OPT_SHADER 6             /* RAST_SHADER_* (default RAST_SHADER_EXACT) */
#define RAST_OPT_MLP_SAMPLES 7        /* learned shader: fragments of each 128-fragment tile whose
                                         learned colour is checked against the per-light sum, 0..4
                                         (default 2) */
#define RAST_OPT_MLP_BOUND_MILLI 8    /* learned shader: a tile whose checked fragments differ from
                                         the exact shader by more than this many thousandths of
                                         1/255 in a channel is shaded exactly (default 500) */
#define RAST_OPT_TILE_THREADS 10      /* threads per tile of the tile raster (binned triangles):
                                         64, 128, 256 or, with tile 32, 512; 0 (default):
                                         min(tile * tile, 256) */
#define RAST_OPT_HOST_IN_PLACE 11     /* rast_draw's host buffers. 1 (default): used in place by the
                                         kernels when the device reaches them (page-locked memory
                                         it maps; ordinary pageable memory when it translates host
                                         addresses through the host's page tables, as on Grace);
                                         0: always copied through device memory */
#define RAST_OPT_MLP_NETWORK 12      /* learned shader: the network rast_mlp_train builds. 0 (default):
                                         3 Fourier frequencies per normal component, hidden layers of
                                         32; 1: 16 frequencies, hidden layers of 64 (the 16-frequency
                                         64 -> 64 -> 3 network). Weights already trained or loaded
                                         keep their own network; rast_mlp_load takes it from the blob */
#define RAST_OPT_TEST_SHADE_STALL 9   /* test only (default 0). 1: the learned shader's first wait
                                         for a tensor-core MMA polls an mbarrier nothing arrives
                                         on, 1024 times, so it gives up as a lost MMA would: the
                                         kernel waits for the MMA in flight with the full bound,
                                         frees its tensor memory and returns, and the draw
                                         reports RAST_ERR_TIMEOUT */
/* Shading (RAST_OPT_SHADER). Coverage, depth and triangle ids are the same in every mode.
 *   EXACT: shading.cpp's per-light sum inside the resolve pass (the reference's colour, bit for bit)
 *   EXACT_DEFERRED: the resolve pass stores the winning fragments (normal, albedo, pixel); a
 *     separate pass shades them with the same per-light sum (same colour as EXACT)
 *   LEARNED: the stored fragments are shaded by the context's MLP (rast_mlp_train / rast_mlp_load)
 *     on the tensor cores; for RAST_OPT_MLP_SAMPLES fragments per 128-fragment tile the learned
 *     colour is compared with the per-light sum (summed in a different order, as an estimate), and
 *     a tile whose sampled error exceeds RAST_OPT_MLP_BOUND_MILLI is shaded exactly, in the
 *     reference's order, in full. Needs weights trained or loaded for the current lights (RAST_ERR_INVALID_ARG
 *     otherwise). Single draws only: batches always use EXACT. */
#define RAST_SHADER_EXACT 0
#define RAST_SHADER_EXACT_DEFERRED 1
#define RAST_SHADER_LEARNED 2
rast_status rast_set_option(rast_ctx* ctx, int option, int64_t value);
rast_status rast_get_option(rast_ctx* ctx, int option, int64_t* value);

/* ------------------------------------------------------------------------------------------ */
/* batches: many frames of different meshes, sizes, transforms and light rigs                   */
/* ------------------------------------------------------------------------------------------ */

/* One frame of a batch. Everything a single rast_draw_device takes, per frame. */
typedef struct rast_frame_desc {
    int32_t mesh;            /* 0: the mesh of rast_upload_mesh; otherwise an id from rast_add_mesh */
    uint32_t width, height;  /* 1..32768 */
    uint32_t flags;          /* RAST_WIND_CLOCKWISE, RAST_CLEAR */
    float camera[16];        /* as rast_draw */
    float normal[16];
    const float* d_lights7;  /* device: nl records as rast_set_lights takes them */
    int32_t nl;
    int32_t reserved;
    uint8_t* d_rgb_planar;   /* device outputs, as rast_draw_device */
    float* d_depth;
    uint32_t* d_tri_id;      /* nullable */
} rast_frame_desc;

/* Uploads another mesh (same layouts and checks as rast_upload_mesh) for use by batches;
 * *mesh_id receives its id (1, 2, ...). Synchronous. */
rast_status rast_add_mesh(rast_ctx* ctx, const float* pos, int64_t nv, const float* nrm, int64_t nn,
                          const float* uv, int64_t nuv, const int32_t* tris, int64_t ntri, const float* kd,
                          int32_t nmat, int32_t* mesh_id);

#define RAST_BATCH_GRAPH 1u /* record the batch as one CUDA graph and launch that; while the frames'
                               descriptors, the options and the stream stay the same, later calls
                               launch the recorded graph again without recording */

/* Draws n frames, frame i on stream i % lanes (1..64 lanes, each with its own scratch), forked from
 * and joined back into the context's stream; asynchronous. Each frame's result equals that of
 * rast_draw_device with the same arguments. Call rast_sync to wait and to collect device status
 * (RAST_ERR_BIN_OVERFLOW: a lane's bin pool was grown, draw the batch again). */
rast_status rast_draw_batch(rast_ctx* ctx, const rast_frame_desc* frames, int32_t n, int32_t lanes,
                            uint32_t batch_flags);

/* Per-frame counters of the last batch (waits for the stream): out[8*i + k] as rast_get_stats. */
rast_status rast_get_batch_stats(rast_ctx* ctx, uint64_t* out);

/* Autotuner: draws the batch (as a CUDA graph) `repeats` times for each tile size (8, 16, 32),
 * per-triangle-path limit (256, 1024, 4096 pixels) and row chunk (4, 8, 32); then, for the fastest
 * of those, for each number of threads per tile of the tile raster (64, 128, 256, and 512 with
 * tile 32). It keeps the fastest as the context's options and sizes the bin pools to what the
 * batch needed. out: tile, small_max, row_chunk, bin capacity (entries), threads per tile. */
rast_status rast_autotune(rast_ctx* ctx, const rast_frame_desc* frames, int32_t n, int32_t lanes,
                          int32_t repeats, int64_t out[5]);

/* Device status words of the last draw (waits for the stream): [0] triangles on the binned path,
 * [1] status bits (1 bin-pool overflow, 2 binned-list overflow, 4 failed consistency check,
 * 8 the learned shader timed out waiting for the tensor cores),
 * [2] code of the first failed check (0 none), [3] its detail. Kernels built with RAST_CHECKED
 * bounds-check every derived index; the default build checks the ones that index other arrays. */
rast_status rast_get_device_status(rast_ctx* ctx, uint32_t out[4]);

/* Device time of each stage of the last draw in milliseconds, from CUDA events recorded on the
 * context's stream between its kernels (needs RAST_OPT_STAGE_TIMING = 1; waits for the stream):
 *   [0] key arming   [1] vertex        [2] setup + per-triangle raster   [3] bin scan
 *   [4] bin scatter  [5] tile raster   [6] resolve (+ shade in EXACT mode)
 *   [7] deferred shading (fragment scan + shading kernel; 0 in EXACT mode)   [8] whole draw */
rast_status rast_get_stage_times(rast_ctx* ctx, float out_ms[9]);

/* ------------------------------------------------------------------------------------------ */
/* learned many-light shading (no counterpart in the reference)                                 */
/* ------------------------------------------------------------------------------------------ */

/* Training of the context's MLP for its current lights (rast_set_lights). Samples are normals
 * uniform on the sphere and albedos uniform in [0,1]^3, labelled on the GPU with the exact
 * per-light shader's float radiance; training is Adam on the mean squared error with the
 * forward pass rounded as the tensor-core kernel rounds it (BF16 weights and activations). */
typedef struct rast_mlp_train_desc {
    int64_t samples;   /* training samples (default 4194304) */
    int64_t holdout;   /* held-out samples for the error report (default 65536) */
    int32_t epochs;    /* passes over the samples (default 24) */
    int32_t ctas;      /* CTAs per step, 64 samples each (default: the SM count) */
    float lr;          /* peak learning rate (default 0.003), cosine decay to lr/100 */
    uint64_t seed;     /* samples and initial weights (default 1) */
} rast_mlp_train_desc;

/* Trains (desc NULL: defaults; zero fields take their default). out (nullable): [0] mean squared
 * error of the last epoch (1/255 units squared), [1] mean and [2] largest absolute channel error
 * of the tensor-core kernel on the held-out samples (1/255 units, before clamping), [3] seconds.
 * Synchronous. */
rast_status rast_mlp_train(rast_ctx* ctx, const rast_mlp_train_desc* desc, float out[4]);

/* The weights as a versioned blob ("RMLP", see rasteriser_gb300/csrc/rast_mlp.h: header with the
 * light rig's hash and the output scale, then the BF16 weights; the biases are weights of constant
 * inputs). *size receives the blob size;
 * buf may be NULL to query it. RAST_ERR_INVALID_ARG if cap is too small or nothing is trained. */
rast_status rast_mlp_save(rast_ctx* ctx, void* buf, size_t cap, size_t* size);

/* Loads a blob from rast_mlp_save. It is used only while the context's lights hash to the rig it
 * was trained for. */
rast_status rast_mlp_load(rast_ctx* ctx, const void* buf, size_t size);

/* Evaluates n (normal, albedo) pairs (host buffers, 3 floats each) through the tensor-core kernel
 * (exact = 0) or the exact shader (exact = 1); out: n * 3 radiance floats before clamping and
 * truncation (1/255 units). Synchronous. */
rast_status rast_mlp_eval(rast_ctx* ctx, const float* normals3, const float* albedo3, int64_t n, int32_t exact,
                          float* out3);

/* Benchmark helper (no counterpart in the reference): runs the deferred shading pass of the
 * context's last draw (made with RAST_SHADER_EXACT_DEFERRED or RAST_SHADER_LEARNED) `repeats` more
 * times, back to back on the context's stream, over the same fragment records and tiles, and
 * returns the mean time of one pass in microseconds (CUDA events around all of them; each pass is
 * launched as in a draw, while its predecessor finishes). The passes rewrite the same colours into
 * that draw's frame buffer, which must still exist (use it after rast_draw_device); the learned
 * shader's counters (rast_get_shade_stats) then hold the sums over the passes. Waits for the
 * stream. RAST_ERR_INVALID_ARG when the last draw did not shade in a separate pass. */
rast_status rast_time_shading(rast_ctx* ctx, int32_t repeats, float* us_per_pass);

/* Learned-shader counters of the last draw (waits for the stream): [0] tiles, [1] tiles shaded
 * exactly after their check failed, [2] fragments checked, [3] largest checked channel error in
 * millionths of 1/255. */
rast_status rast_get_shade_stats(rast_ctx* ctx, uint64_t out[4]);

/* ------------------------------------------------------------------------------------------ */
/* drawing without device allocation (no counterpart in the reference)                         */
/* ------------------------------------------------------------------------------------------ */

/* One frame like rast_draw_device, for callers that must not allocate device memory: a host
 * application that gives all device memory to its own pool and allows no allocation it does not
 * own, or a frame loop that cannot take the device-wide synchronisation of cudaMalloc / cudaFree.
 * No context is needed and nothing is allocated: the mesh (in the layouts of rast_upload_mesh),
 * the lights (as for rast_set_lights) and the outputs are the caller's device buffers, and every
 * intermediate buffer lives in one fixed 64 MiB array inside the library, which each GPU that
 * loads the library holds until the process exits. A frame whose buffers do not fit is refused
 * with RAST_ERR_INVALID_ARG: 92 bytes per triangle, 16 per vertex, 8 per pixel and 256 KiB of
 * tile-bin entries must fit, e.g. a closed mesh of about 640 k triangles at 640x480 or 500 k at
 * 1920x1080. The tile-bin entries (one per large triangle and 16x16 tile it covers) take the rest
 * of the array; a frame that needs more returns RAST_ERR_BIN_OVERFLOW and leaves the frame, depth
 * and id buffers as they were. Indices are checked on the device (RAST_ERR_BAD_INDEX); uv indices
 * are not read. The draw uses the context's default options (tile 16, whole-row items). The
 * first call on a device looks up the array's device address (with that device current); make
 * that first call before any stream capture. All calls share the array and it keeps the last
 * call's contents; each call clears what it needs. Calls that overlap on the GPU race on the
 * array: serialise them. Runs on `stream` (a cudaStream_t, NULL for the legacy default stream)
 * and returns when the frame is complete. Errors: rast_last_error(NULL). */
rast_status rast_draw_noalloc(const float* d_pos, int64_t nv, const float* d_nrm, int64_t nn,
                              const int32_t* d_tris, int64_t ntri, const float* d_kd, int32_t nmat,
                              const float* d_lights7, int32_t nl, const float camera[16],
                              const float normal[16], uint32_t width, uint32_t height, uint32_t flags,
                              uint8_t* d_rgb_planar, float* d_depth, uint32_t* d_tri_id, void* stream);

/* ------------------------------------------------------------------------------------------ */
/* inputs from files (fileloader.cpp, material.h) and outputs (renderer.cpp)                    */
/* ------------------------------------------------------------------------------------------ */

/* A Wavefront OBJ model loaded as the reference's load_obj loads it (fileloader.cpp:81-118, with
 * the vendored tinyobjloader): vertex positions, normals and uvs in file order, the triangles of
 * every kept shape in order (polygons as fans), in the Triangle layout of rast_upload_mesh, and the
 * MTL materials in file order. Missing uv / normal indices are -1; a face without `usemtl` gets
 * material -1 (rast_upload_mesh refuses both normals and materials < 0, where the reference's
 * draw_frame reads out of bounds). textures[i] is mats_dir + map_Kd of material i, or "". */
typedef struct rast_obj rast_obj;
typedef struct rast_obj_data {
    const float* pos;     int64_t nv;
    const float* nrm;     int64_t nn;
    const float* uv;      int64_t nuv;
    const int32_t* tris;  int64_t ntri;
    const float* kd;      int32_t nmat;
    const char* const* textures;
} rast_obj_data;

/* Loads obj_path; MTL files named by `mtllib` are read from mats_dir + name (the reference's
 * --mats-dir, concatenated as given). Errors: rast_last_error(NULL). */
rast_status rast_obj_load(const char* obj_path, const char* mats_dir, rast_obj** out);
void rast_obj_free(rast_obj* obj);
/* Pointers into the loaded model, valid until rast_obj_free. */
rast_status rast_obj_view(const rast_obj* obj, rast_obj_data* out);

/* The lights CSV (fileloader.cpp:121-132): one light per non-blank line, 7 comma-separated numbers
 * (direction xyz, intensity, colour rgb) as rast_set_lights takes them once transformed
 * (rast_transform_lights). Writes min(n, cap) records; *n receives the count. */
rast_status rast_lights_load(const char* path, float* lights7, int32_t cap, int32_t* n);

/* A raw image for a texture: binary or ASCII PGM / PPM (maxval up to 65535) or PFM, as floats in
 * CImg's planar layout (x + y*w + c*w*h, rows top first), values as stored (0..maxval). With
 * out = NULL only w, h and channels (1 or 3) are reported; otherwise cap >= w*h*channels floats. */
rast_status rast_image_load(const char* path, uint32_t* w, uint32_t* h, uint32_t* channels, float* out,
                            size_t cap);

/* renderer.cpp:93 `depth_buffer.normalize(0,255)` for a device depth buffer: the smallest and
 * largest depth m, M of the w*h values, each value v written as (uint8)((v - m) / (M - m) * 255)
 * (0 everywhere when m == M), on the context's stream (asynchronous). */
rast_status rast_depth_to_u8(rast_ctx* ctx, const float* d_depth, uint32_t width, uint32_t height,
                             uint8_t* d_out);

/* The same for host buffers (synchronous). */
rast_status rast_depth_to_u8_host(rast_ctx* ctx, const float* depth, uint32_t width, uint32_t height,
                                  uint8_t* out);

/* The spin loop of renderer.cpp:94-125 without a window: `frames` frames drawn one after another
 * on the device into buffers the context owns (each cleared first, as the loop fills the frame
 * with 0 and the depth with 1), the model's ry advancing by `step` radians per frame (the
 * reference advances it by each frame's wall-clock time). The lights are the world-space records
 * of the lights CSV; they are transformed with the frames' view matrix (it does not depend on the
 * rotation). The mesh is the context's. last_rgb / last_depth (nullable, host, planar RGB8 and
 * floats) receive the last frame; *seconds (nullable) the wall-clock time of the loop, frames
 * enqueued without waiting in between. */
typedef struct rast_spin_desc {
    uint32_t width, height;   /* 1..32768 */
    uint32_t flags;           /* RAST_WIND_CLOCKWISE, RAST_FLAT */
    int32_t frames;           /* >= 1 */
    float scale, disp[3], angles[3];
    float step;               /* ry increment per frame, radians */
    float fovy_deg, z_near, z_far;
    const float* lights7;     /* nl records: direction xyz, intensity, colour rgb */
    int32_t nl;
} rast_spin_desc;
rast_status rast_spin(rast_ctx* ctx, const rast_spin_desc* desc, uint8_t* last_rgb, float* last_depth,
                      double* seconds);

#ifdef __cplusplus
}
#endif

#endif /* RAST_H */
