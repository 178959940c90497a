// Test stand-in for canmom/rasteriser's headers/material.h, untextured materials only: sample()
// returns the constant albedo.
#ifndef RASTERISER_MATERIAL_H
#define RASTERISER_MATERIAL_H
#include <glm/vec2.hpp>
#include <glm/vec3.hpp>
class Material {
    glm::vec3 diffuse_colour;
public:
    explicit Material(const glm::vec3& dc) : diffuse_colour(dc) {}
    glm::vec3 sample(const glm::vec2&) const { return diffuse_colour; }
};
#endif
