// Oracle test infrastructure. A C-ABI harness around canmom/rasteriser's own, unmodified
// geometry.cpp, drawing.cpp, shading.cpp, material.cpp, fileloader.cpp and arguments.cpp (with the
// vendored CImg and tinyobjloader), compiled from the reference tree by oracle/Makefile into
// oracle/_ref/libref.so. Tests and the golden-fixture script
// load it with ctypes; nothing in the product links it.
//
// The reference hard-codes its projection to 45 deg / 0.1 / 6 (geometry.cpp:27-33). geometry.cpp is
// compiled with -Dcamera_matrix=ref_camera_matrix_45 so that the harness supplies camera_matrix,
// built the same way (perspective * modelview) but with a configurable fovy / near / far.
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>

#include "CImg.h"
#include "arguments.h"
#include "drawing.h"
#include "face.h"
#include "fileloader.h"
#include "geometry.h"
#include "light.h"
#include "material.h"
#include "shading.h"

glm::mat4 ref_camera_matrix_45(const glm::mat4& modelview, float aspect_ratio);

namespace {
float g_fovy_deg = 45.0f;
float g_near = 0.1f;
float g_far = 6.0f;

void put_mat(const glm::mat4& m, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = m[c][r];
}

Args make_args(uint32_t w, uint32_t h, int cw, float scale, const float* disp, const float* angles) {
    char a0[] = "oracle", a1[] = "-l", a2[] = "unused.csv";
    char* argv[] = {a0, a1, a2, nullptr};
    Args args(3, argv);
    args.image_width = w;
    args.image_height = h;
    // Same expression as arguments.cpp:39.
    args.aspect_ratio = (float)args.image_width / (float)args.image_height;
    args.wind_clockwise = cw != 0;
    args.scale = scale;
    args.displacement = glm::vec3(disp[0], disp[1], disp[2]);
    args.tait_bryan_angles = glm::vec3(angles[0], angles[1], angles[2]);
    return args;
}
}  // namespace

// Replaces the reference's camera_matrix (geometry.cpp:27-33) with the same formula and a
// projection chosen by the caller.
glm::mat4 camera_matrix(const glm::mat4& modelview, float aspect_ratio) {
    glm::mat4 perspective = glm::perspective(glm::radians(g_fovy_deg), aspect_ratio, g_near, g_far);
    return perspective * modelview;
}

extern "C" {

void ref_set_projection(float fovy_deg, float z_near, float z_far) {
    g_fovy_deg = fovy_deg;
    g_near = z_near;
    g_far = z_far;
}

// out: model, view, modelview, camera, normal matrix (transpose(inverse(modelview))) and the
// unmodified 45-degree camera matrix, each 16 floats column major (96 floats).
void ref_matrices(uint32_t w, uint32_t h, float scale, const float* disp, const float* angles, float* out) {
    const float aspect = (float)w / (float)h;
    glm::mat4 model = transformation_matrix(scale, glm::vec3(disp[0], disp[1], disp[2]),
                                            glm::vec3(angles[0], angles[1], angles[2]));
    glm::mat4 view = transformation_matrix(1.f, glm::vec3(0.f, 0.f, -3.f), glm::vec3(0.f));
    glm::mat4 modelview = view * model;
    glm::mat4 camera = camera_matrix(modelview, aspect);
    glm::mat4 normal = glm::transpose(glm::inverse(modelview));
    glm::mat4 camera45 = ref_camera_matrix_45(modelview, aspect);
    put_mat(model, out + 0);
    put_mat(view, out + 16);
    put_mat(modelview, out + 32);
    put_mat(camera, out + 48);
    put_mat(normal, out + 64);
    put_mat(camera45, out + 80);
}

// The reference's per-vertex stage (geometry.cpp:85-95, 110-116, 135-142) for the given camera
// matrix: raster (x, y, ndc z, 1/w) per vertex, 4 floats each.
void ref_raster_vertices(const float* camera16, const float* verts, int64_t nv, uint32_t w, uint32_t h,
                         float* out4) {
    glm::mat4 cam;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) cam[c][r] = camera16[c * 4 + r];
    std::vector<glm::vec3> v((size_t)nv);
    for (int64_t i = 0; i < nv; ++i) v[i] = glm::vec3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    std::vector<glm::vec4> clip, ndc, raster;
    transform_vertices(cam, v, clip);
    z_divide_all(clip, ndc);
    ndc_to_raster_all((int)w, (int)h, ndc, raster);
    for (int64_t i = 0; i < nv; ++i) {
        out4[4 * i + 0] = raster[i].x;
        out4[4 * i + 1] = raster[i].y;
        out4[4 * i + 2] = raster[i].z;
        out4[4 * i + 3] = raster[i].w;
    }
}

float ref_signed_area_2d(const float* v12) {
    std::array<glm::vec4, 3> v;
    for (int k = 0; k < 3; ++k) v[k] = glm::vec4(v12[4 * k], v12[4 * k + 1], v12[4 * k + 2], v12[4 * k + 3]);
    return signed_area_2d(v);
}

// shading.cpp:24-34 for one fragment. lights7: trans_dir xyz, intensity, colour rgb.
void ref_shade(const float* normal3, const float* albedo3, const float* lights7, int nl, uint32_t* out3) {
    std::vector<Light> lights;
    for (int i = 0; i < nl; ++i) {
        const float* L = lights7 + 7 * i;
        lights.push_back(Light(glm::vec3(0.f), L[3], glm::vec3(L[4], L[5], L[6])));
        lights.back().trans_dir = glm::vec3(L[0], L[1], L[2]);
    }
    glm::uvec3 px = shade(glm::vec3(normal3[0], normal3[1], normal3[2]),
                          glm::vec3(albedo3[0], albedo3[1], albedo3[2]), lights);
    out3[0] = px.x;
    out3[1] = px.y;
    out3[2] = px.z;
}

// Runs the reference's draw_frame (drawing.cpp:205-258) once.
//   verts: nv*3; tris: ntri*10 int32 in the Triangle layout (vertices[3], normals[3], uvs[3],
//   material); normals: nn*3; uvs: nuv*2; lights7: direction xyz, intensity, colour rgb per light;
//   kd: nmat*3 (constant-albedo materials). frame: planar RGB8 (W*H*3), depth: W*H floats; both
//   are read and written. trans_dirs (nullable): the lights' trans_dir after the call, nl*3.
// Returns 0 on success, 1 on a C++ exception.
// ref_draw_frame with textured materials: textures[i] (nullable, or "") is the image file material
// i loads through the reference's Material (CImg, normalised to 0..1, material.h:20-22).
int ref_draw_frame_tex(const float* verts, int64_t nv, const int32_t* tris, int64_t ntri, const float* normals,
                       int64_t nn, const float* uvs, int64_t nuv, const float* lights7, int nl, const float* kd,
                       int nmat, const char* const* textures, uint32_t w, uint32_t h, int cw, float scale,
                       const float* disp, const float* angles, uint8_t* frame, float* depth, float* trans_dirs);

int ref_draw_frame(const float* verts, int64_t nv, const int32_t* tris, int64_t ntri, const float* normals,
                   int64_t nn, const float* uvs, int64_t nuv, const float* lights7, int nl, const float* kd,
                   int nmat, uint32_t w, uint32_t h, int cw, float scale, const float* disp, const float* angles,
                   uint8_t* frame, float* depth, float* trans_dirs) {
    return ref_draw_frame_tex(verts, nv, tris, ntri, normals, nn, uvs, nuv, lights7, nl, kd, nmat, nullptr, w, h, cw,
                              scale, disp, angles, frame, depth, trans_dirs);
}

int ref_draw_frame_tex(const float* verts, int64_t nv, const int32_t* tris, int64_t ntri, const float* normals,
                       int64_t nn, const float* uvs, int64_t nuv, const float* lights7, int nl, const float* kd,
                       int nmat, const char* const* textures, uint32_t w, uint32_t h, int cw, float scale,
                       const float* disp, const float* angles, uint8_t* frame, float* depth, float* trans_dirs) {
    try {
        Args args = make_args(w, h, cw, scale, disp, angles);
        std::vector<glm::vec3> mv((size_t)nv), mn((size_t)nn);
        std::vector<glm::vec2> mu((size_t)nuv);
        for (int64_t i = 0; i < nv; ++i) mv[i] = glm::vec3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
        for (int64_t i = 0; i < nn; ++i) mn[i] = glm::vec3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
        for (int64_t i = 0; i < nuv; ++i) mu[i] = glm::vec2(uvs[2 * i], uvs[2 * i + 1]);
        std::vector<Triangle> faces;
        faces.reserve((size_t)ntri);
        for (int64_t i = 0; i < ntri; ++i) {
            const int32_t* t = tris + 10 * i;
            faces.push_back(Triangle({t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]}, t[9]));
        }
        std::vector<Material> mats;
        for (int i = 0; i < nmat; ++i) {
            const glm::vec3 dc(kd[3 * i], kd[3 * i + 1], kd[3 * i + 2]);
            if (textures && textures[i] && textures[i][0]) mats.push_back(Material(dc, textures[i]));
            else mats.push_back(Material(dc));
        }
        std::vector<Light> lights;
        for (int i = 0; i < nl; ++i) {
            const float* L = lights7 + 7 * i;
            lights.push_back(Light(glm::vec3(L[0], L[1], L[2]), L[3], glm::vec3(L[4], L[5], L[6])));
        }
        cimg_library::CImg<unsigned char> fb(w, h, 1, 3, 0);
        cimg_library::CImg<float> db(w, h, 1, 1, 1.f);
        std::memcpy(fb.data(), frame, (size_t)w * h * 3);
        std::memcpy(db.data(), depth, (size_t)w * h * sizeof(float));
        draw_frame(mv, faces, mn, mu, lights, mats, args, &fb, &db);
        std::memcpy(frame, fb.data(), (size_t)w * h * 3);
        std::memcpy(depth, db.data(), (size_t)w * h * sizeof(float));
        if (trans_dirs)
            for (int i = 0; i < nl; ++i) {
                trans_dirs[3 * i] = lights[i].trans_dir.x;
                trans_dirs[3 * i + 1] = lights[i].trans_dir.y;
                trans_dirs[3 * i + 2] = lights[i].trans_dir.z;
            }
        return 0;
    } catch (...) {
        return 1;
    }
}

// The reference's load_obj (fileloader.cpp:81-118) on obj_path with --mats-dir mats_dir. The
// arrays are kept until the next call: ref_obj_counts gives nv, nn, nuv, ntri, nmat and ref_obj_copy
// copies them (positions, normals, uvs, Triangle records, and each material's Material::sample at
// uv (0, 0): its Kd without a texture). Returns 0, or 1 on a C++ exception.
namespace {
std::vector<glm::vec3> g_v, g_n;
std::vector<glm::vec2> g_uv;
std::vector<Triangle> g_tris;
std::vector<Material> g_mats;
}  // namespace

int ref_load_obj(const char* obj_path, const char* mats_dir) {
    try {
        std::string o(obj_path), d(mats_dir ? mats_dir : "");
        char a0[] = "oracle", a1[] = "-l", a2[] = "unused.csv", a3[] = "-o", a5[] = "--mats-dir";
        std::vector<char> a4(o.begin(), o.end()), a6(d.begin(), d.end());
        a4.push_back('\0');
        a6.push_back('\0');
        char* argv[] = {a0, a1, a2, a3, a4.data(), a5, a6.data(), nullptr};
        Args args(7, argv);
        g_v.clear(); g_n.clear(); g_uv.clear(); g_tris.clear(); g_mats.clear();
        load_obj(args, g_v, g_tris, g_n, g_uv, g_mats);
        return 0;
    } catch (...) {
        return 1;
    }
}

void ref_obj_counts(int64_t* out5) {
    out5[0] = (int64_t)g_v.size();
    out5[1] = (int64_t)g_n.size();
    out5[2] = (int64_t)g_uv.size();
    out5[3] = (int64_t)g_tris.size();
    out5[4] = (int64_t)g_mats.size();
}

void ref_obj_copy(float* pos, float* nrm, float* uv, int32_t* tris, float* kd) {
    for (size_t i = 0; i < g_v.size(); ++i)
        for (int k = 0; k < 3; ++k) pos[3 * i + k] = g_v[i][k];
    for (size_t i = 0; i < g_n.size(); ++i)
        for (int k = 0; k < 3; ++k) nrm[3 * i + k] = g_n[i][k];
    for (size_t i = 0; i < g_uv.size(); ++i)
        for (int k = 0; k < 2; ++k) uv[2 * i + k] = g_uv[i][k];
    for (size_t i = 0; i < g_tris.size(); ++i) {
        const Triangle& t = g_tris[i];
        for (int k = 0; k < 3; ++k) {
            tris[10 * i + k] = t.vertices[k];
            tris[10 * i + 3 + k] = t.normals[k];
            tris[10 * i + 6 + k] = t.uvs[k];
        }
        tris[10 * i + 9] = t.material;
    }
    for (size_t i = 0; i < g_mats.size(); ++i) {
        const glm::vec3 c = g_mats[i].sample(glm::vec2(0.f, 0.f));
        for (int k = 0; k < 3; ++k) kd[3 * i + k] = c[k];
    }
}

// The reference's load_lights (fileloader.cpp:121-132): up to cap records of 7 floats; returns the
// number it read.
int ref_load_lights(const char* path, float* out7, int cap) {
    std::vector<Light> lights;
    load_lights(path, lights);
    int n = 0;
    for (const Light& L : lights) {
        if (n < cap) {
            float* o = out7 + 7 * n;
            o[0] = L.direction.x; o[1] = L.direction.y; o[2] = L.direction.z;
            o[3] = L.intensity;
            o[4] = L.colour.r; o[5] = L.colour.g; o[6] = L.colour.b;
        }
        ++n;
    }
    return n;
}

}  // extern "C"
