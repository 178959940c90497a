// Test stand-in for canmom/rasteriser's headers/material.h: the same private members, a
// constructor for untextured materials, and one that takes the texture as loaded instead of a file
// name (this stand-in has no image loader). Like the reference's, it normalises the texture to
// 0..1 (CImg normalize(0, 1): smallest and largest value over all channels; 0 everywhere when they
// are equal). sample() is the untextured case only; the drop-in does not call it for textures.
#ifndef RASTERISER_MATERIAL_H
#define RASTERISER_MATERIAL_H
#include <glm/vec2.hpp>
#include <glm/vec3.hpp>
#include "CImg.h"
class Material {
private:
    glm::vec3 diffuse_colour;
    bool has_texture;
    cimg_library::CImg<float> diffuse_texture;

public:
    explicit Material(const glm::vec3& dc) : diffuse_colour(dc), has_texture(false) {}
    Material(const glm::vec3& dc, const cimg_library::CImg<float>& texture)
        : diffuse_colour(dc), has_texture(true), diffuse_texture(texture) {
        float* v = diffuse_texture.data();
        const size_t n = (size_t)diffuse_texture.width() * diffuse_texture.height() * diffuse_texture.depth() *
                         diffuse_texture.spectrum();
        float m = v[0], M = v[0];
        for (size_t i = 1; i < n; ++i) {
            if (v[i] < m) m = v[i];
            if (v[i] > M) M = v[i];
        }
        for (size_t i = 0; i < n; ++i) v[i] = m == M ? 0.f : (m == 0.f && M == 1.f) ? v[i] : (v[i] - m) / (M - m) * 1.f + 0.f;
    }
    glm::vec3 sample(const glm::vec2&) const { return diffuse_colour; }
};
#endif
