// Host-side geometry of the C ABI: the per-frame matrices and the light transform of draw_frame
// (drawing.cpp:221-238; geometry.cpp:22-33, 97-108, 124-133). Written against the glm API and
// compiled with -ffp-contract=off, so the matrices are the ones the reference's own geometry.cpp
// builds with the same glm.
#include <cstring>

#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>

#include "rast.h"

namespace {

// geometry.cpp:22-25: T * Ry * Rx * Rz * S, multiplied left to right.
glm::mat4 transformation(float factor, const glm::vec3& d, const glm::vec3& tb) {
    return glm::translate(glm::mat4(1.f), d) * glm::rotate(glm::mat4(1.f), tb.y, glm::vec3(0.f, 1.f, 0.f)) *
           glm::rotate(glm::mat4(1.f), tb.x, glm::vec3(1.f, 0.f, 0.f)) *
           glm::rotate(glm::mat4(1.f), tb.z, glm::vec3(0.f, 0.f, 1.f)) * glm::scale(glm::mat4(1.f), glm::vec3(factor));
}

void put(const glm::mat4& m, float* out) {
    if (!out) return;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = m[c][r];
}

glm::mat4 get(const float* in) {
    glm::mat4 m(0.f);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) m[c][r] = in[c * 4 + r];
    return m;
}

}  // namespace

extern "C" rast_status rast_frame_matrices(uint32_t width, uint32_t height, float scale, const float disp[3],
                                           const float angles[3], float fovy_deg, float z_near, float z_far,
                                           float model_out[16], float view_out[16], float modelview_out[16],
                                           float camera_out[16], float normal_out[16]) {
    if (width == 0 || height == 0 || !disp || !angles) return RAST_ERR_INVALID_ARG;
    // arguments.cpp:39
    const float aspect = (float)width / (float)height;
    const glm::mat4 model = transformation(scale, glm::vec3(disp[0], disp[1], disp[2]),
                                           glm::vec3(angles[0], angles[1], angles[2]));
    const glm::mat4 view = transformation(1.f, glm::vec3(0.f, 0.f, -3.f), glm::vec3(0.f));
    const glm::mat4 modelview = view * model;
    // geometry.cpp:27-33 with the caller's projection.
    const glm::mat4 camera = glm::perspective(glm::radians(fovy_deg), aspect, z_near, z_far) * modelview;
    const glm::mat4 normal = glm::transpose(glm::inverse(modelview));
    put(model, model_out);
    put(view, view_out);
    put(modelview, modelview_out);
    put(camera, camera_out);
    put(normal, normal_out);
    return RAST_OK;
}

extern "C" rast_status rast_transform_lights(const float view[16], const float* lights_in, int32_t n,
                                             float* lights_out) {
    if (n < 0 || (n > 0 && (!view || !lights_in || !lights_out))) return RAST_ERR_INVALID_ARG;
    const glm::mat4 v = n > 0 ? get(view) : glm::mat4(1.f);
    for (int32_t i = 0; i < n; ++i) {
        const float* L = lights_in + 7 * i;
        float rec[7];
        std::memcpy(rec, L, sizeof rec);
        // geometry.cpp:35-42 transform_direction, then normalize (geometry.cpp:124-127).
        const glm::vec4 t = v * glm::vec4(rec[0], rec[1], rec[2], 0.f);
        const glm::vec3 d = glm::normalize(glm::vec3(t.x, t.y, t.z));
        rec[0] = d.x;
        rec[1] = d.y;
        rec[2] = d.z;
        std::memcpy(lights_out + 7 * i, rec, sizeof rec);
    }
    return RAST_OK;
}
