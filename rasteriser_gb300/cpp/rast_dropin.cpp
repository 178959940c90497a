// Drop-in implementation of canmom/rasteriser's geometry.h, drawing.h and shading.h entry points
// over librast (include/rast.h). Compiled against the reference's own headers (and its glm and
// CImg); see rast_dropin.h for what it replaces.
//
// draw_frame keeps the reference's contract (drawing.cpp:205-258): the caller owns every vector
// and both CImg buffers, the buffers are read and written (the incoming depth is the value each
// fragment must beat; pixels nothing beats keep their colour and depth), lights[i].trans_dir is
// updated, and the call returns when the frame is complete. It differs in one way: where the
// reference has undefined behaviour on an out-of-range index, this throws std::runtime_error.
#include <array>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <glm/glm.hpp>
#include <glm/gtc/constants.hpp>
#include <glm/gtc/matrix_transform.hpp>

#include "CImg.h"
#include "arguments.h"
#include "drawing.h"
#include "face.h"
#include "geometry.h"
#include "light.h"
#include "material.h"
#include "shading.h"

#include "rast.h"
#include "rast_dropin.h"

using glm::mat4;
using glm::uvec3;
using glm::vec2;
using glm::vec3;
using glm::vec4;
using std::vector;

static_assert(sizeof(Triangle) == 10 * sizeof(int), "Triangle must be 10 packed ints (face.h:6-13)");

// Material keeps its texture private (material.h:11-16) and offers only sample(uv). The drop-in
// uploads the texture itself, so it reads those two members through an explicit instantiation,
// which may name private members (C++11 [temp.explicit] p12), without editing the reference's
// header: member_of(Tag) returns the member pointer the instantiation was given.
template <class Tag, typename Tag::type Member>
struct PrivateMember {
    friend typename Tag::type member_of(Tag) { return Member; }
};
struct MaterialHasTexture {
    typedef bool Material::*type;
    friend type member_of(MaterialHasTexture);
};
struct MaterialTexture {
    typedef cimg_library::CImg<float> Material::*type;
    friend type member_of(MaterialTexture);
};
template struct PrivateMember<MaterialHasTexture, &Material::has_texture>;
template struct PrivateMember<MaterialTexture, &Material::diffuse_texture>;

namespace {

struct State {
    std::mutex mu;
    rast_ctx* ctx = nullptr;
    int device = -1;
    float fovy = 45.0f, z_near = 0.1f, z_far = 6.0f;
    bool static_mesh = false;
    const void* key[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t sizes[4] = {0, 0, 0, 0};
    size_t nmat = 0;
};

State& state() {
    static State s;
    return s;
}

void check(rast_status st, rast_ctx* ctx, const char* what) {
    if (st != RAST_OK)
        throw std::runtime_error(std::string(what) + ": " + rast_status_string(st) + ": " + rast_last_error(ctx));
}

rast_ctx* context(State& s) {
    if (!s.ctx) {
        int dev = s.device;
        if (dev < 0) {
            const char* e = std::getenv("RAST_DEVICE");
            dev = e ? std::atoi(e) : 0;
        }
        check(rast_create(&s.ctx, dev), nullptr, "rast_create");
    }
    return s.ctx;
}

void to_floats(const mat4& m, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = m[c][r];
}

}  // namespace

namespace rast_dropin {

void set_projection(float fovy_degrees, float z_near, float z_far) {
    State& s = state();
    std::lock_guard<std::mutex> g(s.mu);
    s.fovy = fovy_degrees;
    s.z_near = z_near;
    s.z_far = z_far;
}

void set_device(int device) {
    State& s = state();
    std::lock_guard<std::mutex> g(s.mu);
    s.device = device;
}

void set_static_mesh(bool is_static) {
    State& s = state();
    std::lock_guard<std::mutex> g(s.mu);
    s.static_mesh = is_static;
    for (auto& k : s.key) k = nullptr;
}

void shutdown() {
    State& s = state();
    std::lock_guard<std::mutex> g(s.mu);
    if (s.ctx) rast_destroy(s.ctx);
    s.ctx = nullptr;
    for (auto& k : s.key) k = nullptr;
}

}  // namespace rast_dropin

// ------------------------------------------------------------------------------------------------
// geometry.h (geometry.cpp:22-142): host functions with the reference's arithmetic
// ------------------------------------------------------------------------------------------------
mat4 transformation_matrix(float factor, const vec3& displacement, const vec3& tait_bryan) {
    // T * Ry * Rx * Rz * S, multiplied left to right (geometry.cpp:24)
    return glm::translate(mat4(1.f), displacement) * glm::rotate(mat4(1.f), tait_bryan.y, vec3(0.f, 1.f, 0.f)) *
           glm::rotate(mat4(1.f), tait_bryan.x, vec3(1.f, 0.f, 0.f)) *
           glm::rotate(mat4(1.f), tait_bryan.z, vec3(0.f, 0.f, 1.f)) * glm::scale(mat4(1.f), vec3(factor));
}

mat4 camera_matrix(const mat4& modelview, float aspect_ratio) {
    State& s = state();
    float fovy, zn, zf;
    {
        std::lock_guard<std::mutex> g(s.mu);
        fovy = s.fovy;
        zn = s.z_near;
        zf = s.z_far;
    }
    return glm::perspective(glm::radians(fovy), aspect_ratio, zn, zf) * modelview;
}

vec3 transform_direction(const mat4& transformation, const vec3& point) {
    const vec4 t = transformation * vec4(point.x, point.y, point.z, 0.f);
    return vec3(t.x, t.y, t.z);
}

vec4 transform_point(const mat4& transformation, const vec3& point) {
    return transformation * vec4(point.x, point.y, point.z, 1.f);
}

vec4 z_divide(const vec4& c) { return vec4(c.x / c.w, c.y / c.w, c.z / c.w, 1.f / c.w); }

float remap_ndc(float value, float high) { return 0.5f * (value + 1.0f) * high; }

vec4 ndc_to_raster(int width, int height, const vec4& n) {
    return vec4(remap_ndc(n.x, width), remap_ndc(-n.y, height), n.z, n.w);
}

float signed_area_2d(const std::array<vec4, 3>& v) {
    return -0.5f * (v[0].x * v[1].y - v[1].x * v[0].y + v[1].x * v[2].y - v[2].x * v[1].y + v[2].x * v[0].y -
                    v[0].x * v[2].y);
}

void transform_vertices(const mat4& transformation, const vector<vec3>& vertices, vector<vec4>& result) {
    result.resize(vertices.size());
    for (size_t i = 0; i < vertices.size(); ++i) result[i] = transform_point(transformation, vertices[i]);
}

void transform_normals(const mat4& transformation, const vector<vec3>& vertices, vector<vec3>& result) {
    result.resize(vertices.size());
    const mat4 n = glm::transpose(glm::inverse(transformation));
    for (size_t i = 0; i < vertices.size(); ++i) result[i] = transform_direction(n, vertices[i]);
}

void z_divide_all(const vector<vec4>& clip_vertices, vector<vec4>& ndc_vertices) {
    ndc_vertices.resize(clip_vertices.size());
    for (size_t i = 0; i < clip_vertices.size(); ++i) ndc_vertices[i] = z_divide(clip_vertices[i]);
}

void xyz_all(const vector<vec4>& homo, vector<vec3>& cart) {
    cart.resize(homo.size());
    for (size_t i = 0; i < homo.size(); ++i) cart[i] = vec3(homo[i].x, homo[i].y, homo[i].z);
}

void Light::transform(const mat4& transformation) {
    trans_dir = glm::normalize(transform_direction(transformation, direction));
}

void transform_lights(const mat4& transformation, vector<Light>& lights) {
    for (auto& l : lights) l.transform(transformation);
}

void ndc_to_raster_all(int width, int height, const vector<vec4>& ndc, vector<vec4>& raster) {
    raster.resize(ndc.size());
    for (size_t i = 0; i < ndc.size(); ++i) raster[i] = ndc_to_raster(width, height, ndc[i]);
}

// ------------------------------------------------------------------------------------------------
// shading.h (shading.cpp:20-34)
// ------------------------------------------------------------------------------------------------
vec3 light_contribution(const vec3& normal, const vec3& albedo, const Light& light) {
    return light.intensity * light.colour * albedo * glm::max(0.f, glm::dot(normal, -light.trans_dir)) *
           glm::one_over_pi<float>();
}

uvec3 shade(const vec3& normal, const vec3& albedo, const vector<Light> lights) {
    vec3 sum(0.f);
    for (const Light& l : lights) sum = sum + light_contribution(normal, albedo, l);
    return (uvec3)glm::min(sum, vec3(255.f));
}

// ------------------------------------------------------------------------------------------------
// drawing.h: the frame on the GPU
// ------------------------------------------------------------------------------------------------
void draw_frame(const vector<vec3>& model_vertices, const vector<Triangle>& faces, const vector<vec3>& model_vertnormals,
                const vector<vec2>& vertuvs, vector<Light>& lights, const vector<Material>& materials,
                const Args& arguments, cimg_library::CImg<unsigned char>* frame_buffer,
                cimg_library::CImg<float>* depth_buffer) {
    if (!frame_buffer || !depth_buffer) throw std::runtime_error("draw_frame: null frame or depth buffer");
    const uint32_t W = arguments.image_width, H = arguments.image_height;
    if ((uint32_t)frame_buffer->width() != W || (uint32_t)frame_buffer->height() != H ||
        frame_buffer->spectrum() != 3 || (uint32_t)depth_buffer->width() != W ||
        (uint32_t)depth_buffer->height() != H)
        throw std::runtime_error("draw_frame: buffer size differs from Args image size");

    // drawing.cpp:221-238
    const mat4 model = transformation_matrix(arguments.scale, arguments.displacement, arguments.tait_bryan_angles);
    const mat4 view = transformation_matrix(1.f, vec3(0.f, 0.f, -3.f), vec3(0.f));
    const mat4 modelview = view * model;
    const mat4 camera = camera_matrix(modelview, arguments.aspect_ratio);
    const mat4 normal = glm::transpose(glm::inverse(modelview));
    transform_lights(view, lights);

    State& s = state();
    std::lock_guard<std::mutex> g(s.mu);
    rast_ctx* ctx = context(s);

    const void* key[4] = {model_vertices.data(), faces.data(), model_vertnormals.data(), vertuvs.data()};
    const size_t sizes[4] = {model_vertices.size(), faces.size(), model_vertnormals.size(), vertuvs.size()};
    bool same = s.static_mesh && s.nmat == materials.size();
    for (int i = 0; i < 4; ++i) same = same && key[i] == s.key[i] && sizes[i] == s.sizes[i];
    if (!same) {
        // Material::sample returns the constant albedo for an untextured material (material.cpp:24);
        // a textured one samples its texture (material.cpp:12-22), which librast does per fragment.
        vector<float> kd(3 * materials.size(), 0.f);
        for (size_t i = 0; i < materials.size(); ++i) {
            if (materials[i].*member_of(MaterialHasTexture())) continue;
            const vec3 c = materials[i].sample(vec2(0.f));
            kd[3 * i] = c.x;
            kd[3 * i + 1] = c.y;
            kd[3 * i + 2] = c.z;
        }
        check(rast_upload_mesh(ctx, reinterpret_cast<const float*>(model_vertices.data()), (int64_t)model_vertices.size(),
                               reinterpret_cast<const float*>(model_vertnormals.data()),
                               (int64_t)model_vertnormals.size(), reinterpret_cast<const float*>(vertuvs.data()),
                               (int64_t)vertuvs.size(), reinterpret_cast<const int32_t*>(faces.data()),
                               (int64_t)faces.size(), kd.data(), (int32_t)materials.size()),
              ctx, "rast_upload_mesh");
        // the textures, already normalised to 0..1 by Material's constructor (material.h:21);
        // librast's own normalisation leaves such an image as it is
        for (size_t i = 0; i < materials.size(); ++i) {
            if (!(materials[i].*member_of(MaterialHasTexture()))) continue;
            const cimg_library::CImg<float>& tex = materials[i].*member_of(MaterialTexture());
            check(rast_upload_texture(ctx, (int32_t)i, tex.data(), (uint32_t)tex.width(), (uint32_t)tex.height(),
                                      (uint32_t)tex.spectrum()),
                  ctx, "rast_upload_texture");
        }
        for (int i = 0; i < 4; ++i) {
            s.key[i] = key[i];
            s.sizes[i] = sizes[i];
        }
        s.nmat = materials.size();
    }

    vector<float> l7(7 * lights.size());
    for (size_t i = 0; i < lights.size(); ++i) {
        const Light& l = lights[i];
        const float rec[7] = {l.trans_dir.x, l.trans_dir.y, l.trans_dir.z, l.intensity, l.colour.x, l.colour.y, l.colour.z};
        for (int k = 0; k < 7; ++k) l7[7 * i + k] = rec[k];
    }
    check(rast_set_lights(ctx, l7.data(), (int32_t)lights.size()), ctx, "rast_set_lights");

    float cam16[16], nrm16[16];
    to_floats(camera, cam16);
    to_floats(normal, nrm16);
    const uint32_t flags = (arguments.wind_clockwise ? RAST_WIND_CLOCKWISE : 0u) | (arguments.flat ? RAST_FLAT : 0u);
    check(rast_draw(ctx, cam16, nrm16, W, H, flags, frame_buffer->data(), depth_buffer->data(), nullptr), ctx,
          "rast_draw");
}
