// Test stand-in for canmom/rasteriser's headers/face.h: the Triangle record the drop-in receives
// (10 ints: vertex, normal and uv indices of the three corners, then the material).
#ifndef RASTERISER_FACE_H
#define RASTERISER_FACE_H
#include <array>
struct Triangle {
    std::array<int, 3> vertices;
    std::array<int, 3> normals;
    std::array<int, 3> uvs;
    int material;
    Triangle(std::array<int, 3> v, std::array<int, 3> n, std::array<int, 3> uv, int m)
        : vertices(v), normals(n), uvs(uv), material(m) {}
};
#endif
