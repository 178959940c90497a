// Test stand-in for canmom/rasteriser's headers/arguments.h: the fields draw_frame reads. The
// harness fills them directly instead of parsing a command line.
#ifndef RASTERISER_ARGUMENTS_H
#define RASTERISER_ARGUMENTS_H
#include <string>
#include <glm/vec3.hpp>
struct Args {
    unsigned int image_width = 0;
    unsigned int image_height = 0;
    float aspect_ratio = 1.f;
    bool spin = false;
    bool flat = false;
    bool wind_clockwise = false;
    float scale = 1.f;
    glm::vec3 displacement;
    glm::vec3 tait_bryan_angles;
    std::string obj_file, lights_file, materials_directory;
};
#endif
