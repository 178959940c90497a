/* Oracle test infrastructure: a plain-C restatement of canmom/rasteriser's per-frame path
 * (draw_frame, drawing.cpp:205-258), used only by tests, the smoke check and the CPU-baseline leg
 * of bench.py as the checker. Parity status: pinned bit for bit (depth and RGB) against the
 * reference's own drawing.cpp / geometry.cpp / shading.cpp compiled from source (oracle/_ref) on
 * the scenes in tests/golden. It adds what the reference computes but does not expose: the
 * index of the triangle that wrote each pixel, and fragment counts. */
#ifndef RAST_ORACLE_H
#define RAST_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_frame {
    /* mesh, in the reference's layouts */
    const float* pos;      /* nv * 3 */
    int64_t nv;
    const int32_t* tris;   /* ntri * 10: vertices[3], normals[3], uvs[3], material (face.h:6-13) */
    int64_t ntri;
    const float* nrm;      /* nn * 3 */
    int64_t nn;
    const float* uv;       /* nuv * 2 */
    int64_t nuv;
    const float* kd;       /* nmat * 3, constant albedo per material */
    int32_t nmat;
    /* per frame */
    const float* camera;        /* 16, column major: projection * view * model */
    const float* normal_matrix; /* 16, column major: transpose(inverse(view * model)) */
    const float* lights;        /* nl * 7: trans_dir xyz (already transformed), intensity, colour rgb */
    int32_t nl;
    uint32_t width, height;
    int32_t wind_clockwise;
    /* Per-vertex albedo (nv * 3, nullable). The reference's materials are constant per material;
     * the many-light workload adds a colour per vertex, interpolated perspective-correctly exactly
     * as the normals are (drawing.cpp:64-75, 131), in place of Material::sample. */
    const float* vcol;
    /* Textures (nullable; ignored where vcol is given): for material m with tex_off[m] >= 0, its
     * texels normalised to 0..1 as material.h:20-22 does (CImg normalize over all channels), three
     * planes of tex_wh[2m] * tex_wh[2m+1] floats from tex + tex_off[m] (x + y*w + c*w*h), sampled at
     * the perspective-correct uv as Material::sample does (material.cpp:11-26, CImg linear_atXY). */
    const float* tex;
    const int64_t* tex_off;
    const int32_t* tex_wh;
    /* Flat shading (Args::flat, readme.md:46; the reference parses it but never reads it): each
     * triangle's three normals are its face normal cross(p1 - p0, p2 - p0) in model space, which
     * then goes through the path as vertex normals do. */
    int32_t flat;
} oracle_frame;

/* stats (nullable) receives: [0] front-facing triangles, [1] bounding-box pixels tested,
 * [2] inside fragments, [3] depth-test passes. Returns 0, or -1 on a bad argument. */
int oracle_draw_frame(const oracle_frame* f, uint8_t* frame_planar, float* depth, uint32_t* tri_id,
                      uint64_t* stats);

/* Per-vertex stage only: raster x, y, NDC z and 1/w_clip per vertex (out4: nv * 4). */
void oracle_raster_vertices(const float* camera, const float* pos, int64_t nv, uint32_t width,
                            uint32_t height, float* out4);

/* One fragment of shading.cpp:24-34. */
void oracle_shade(const float* normal3, const float* albedo3, const float* lights7, int32_t nl,
                  uint32_t* out3);

/* The per-frame matrices of draw_frame (drawing.cpp:221-229; geometry.cpp:22-33, 101): model,
 * view, modelview, camera = perspective(fovy_deg, width/height, z_near, z_far) * modelview, and the
 * normal matrix transpose(inverse(modelview)); each 16 floats, column major. Returns 0 or -1. */
int oracle_frame_matrices(uint32_t width, uint32_t height, float scale, const float* disp, const float* angles,
                          float fovy_deg, float z_near, float z_far, float* model, float* view,
                          float* modelview, float* camera, float* normal);

/* Light::transform over n (direction xyz, intensity, rgb) records (geometry.cpp:124-133):
 * trans_dir = normalize(xyz(view * (direction, 0))). Returns 0 or -1. */
int oracle_transform_lights(const float* view, const float* lights_in, int32_t n, float* lights_out);

#ifdef __cplusplus
}
#endif

#endif
