// Test driver for the C++ drop-in (rasteriser_gb300/cpp/rast_dropin.cpp): reads a scene written by
// tests/test_gpu_dropin.py, calls draw_frame exactly as renderer.cpp does, and writes the frame,
// depth and transformed light directions back out. Built against tests/cpp/stand_in headers.
//   dropin_driver <in.bin> <out.bin> [repeat]
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "CImg.h"
#include "arguments.h"
#include "drawing.h"
#include "face.h"
#include "light.h"
#include "material.h"
#include "rast_dropin.h"

namespace {
template <typename T> bool get(FILE* f, T* p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const int repeat = argc > 3 ? std::atoi(argv[3]) : 1;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    char magic[4];
    uint32_t hdr[4];
    float view[10];
    int64_t counts[6];
    if (!get(f, magic, 4) || std::memcmp(magic, "RSCN", 4) || !get(f, hdr, 4) || !get(f, view, 10) ||
        !get(f, counts, 6))
        return 4;
    const uint32_t W = hdr[0], H = hdr[1];
    const int64_t nv = counts[0], nn = counts[1], nuv = counts[2], ntri = counts[3], nmat = counts[4], nl = counts[5];
    std::vector<float> pos(3 * nv), nrm(3 * nn), uv(2 * nuv), kd(3 * nmat), li(7 * nl);
    std::vector<int32_t> tris(10 * ntri);
    std::vector<uint8_t> frame_in((size_t)3 * W * H);
    std::vector<float> depth_in((size_t)W * H);
    if (!get(f, pos.data(), pos.size()) || !get(f, nrm.data(), nrm.size()) || !get(f, uv.data(), uv.size()) ||
        !get(f, tris.data(), tris.size()) || !get(f, kd.data(), kd.size()) || !get(f, li.data(), li.size()) ||
        !get(f, frame_in.data(), frame_in.size()) || !get(f, depth_in.data(), depth_in.size()))
        return 5;
    // optional: textures (int64 count; per texture int32 material, uint32 width, height, channels,
    // then width*height*channels floats, planar)
    std::vector<int32_t> tex_mat;
    std::vector<cimg_library::CImg<float> > tex_img;
    int64_t ntex = 0;
    if (get(f, &ntex, 1)) {
        for (int64_t i = 0; i < ntex; ++i) {
            int32_t m;
            uint32_t whc[3];
            if (!get(f, &m, 1) || !get(f, whc, 3)) return 5;
            cimg_library::CImg<float> img(whc[0], whc[1], 1, whc[2], 0.f);
            if (!get(f, img.data(), (size_t)whc[0] * whc[1] * whc[2])) return 5;
            tex_mat.push_back(m);
            tex_img.push_back(img);
        }
    }
    std::fclose(f);

    std::vector<glm::vec3> mv, mn;
    std::vector<glm::vec2> mu;
    for (int64_t i = 0; i < nv; ++i) mv.push_back(glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    for (int64_t i = 0; i < nn; ++i) mn.push_back(glm::vec3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
    for (int64_t i = 0; i < nuv; ++i) mu.push_back(glm::vec2(uv[2 * i], uv[2 * i + 1]));
    std::vector<Triangle> faces;
    for (int64_t i = 0; i < ntri; ++i) {
        const int32_t* t = &tris[10 * i];
        faces.push_back(Triangle({t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]}, t[9]));
    }
    std::vector<Material> mats;
    for (int64_t i = 0; i < nmat; ++i) {
        const glm::vec3 dc(kd[3 * i], kd[3 * i + 1], kd[3 * i + 2]);
        size_t k = 0;
        while (k < tex_mat.size() && tex_mat[k] != (int32_t)i) ++k;
        mats.push_back(k < tex_mat.size() ? Material(dc, tex_img[k]) : Material(dc));
    }
    std::vector<Light> lights;
    for (int64_t i = 0; i < nl; ++i) {
        const float* L = &li[7 * i];
        lights.push_back(Light(glm::vec3(L[0], L[1], L[2]), L[3], glm::vec3(L[4], L[5], L[6])));
    }
    Args args;
    args.image_width = W;
    args.image_height = H;
    args.aspect_ratio = (float)args.image_width / (float)args.image_height;
    args.wind_clockwise = hdr[2] != 0;
    args.scale = view[0];
    args.displacement = glm::vec3(view[1], view[2], view[3]);
    args.tait_bryan_angles = glm::vec3(view[4], view[5], view[6]);
    rast_dropin::set_projection(view[7], view[8], view[9]);
    rast_dropin::set_static_mesh(hdr[3] != 0);

    cimg_library::CImg<unsigned char> fb(W, H, 1, 3, 0);
    cimg_library::CImg<float> db(W, H, 1, 1, 1.f);
    for (int r = 0; r < repeat; ++r) {
        std::memcpy(fb.data(), frame_in.data(), frame_in.size());
        std::memcpy(db.data(), depth_in.data(), depth_in.size() * sizeof(float));
        try {
            draw_frame(mv, faces, mn, mu, lights, mats, args, &fb, &db);
        } catch (const std::exception& e) {
            std::fprintf(stderr, "draw_frame: %s\n", e.what());
            return 6;
        }
    }
    rast_dropin::shutdown();

    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 7;
    std::fwrite(fb.data(), 1, frame_in.size(), o);
    std::fwrite(db.data(), sizeof(float), depth_in.size(), o);
    for (const Light& l : lights) {
        const float d[3] = {l.trans_dir.x, l.trans_dir.y, l.trans_dir.z};
        std::fwrite(d, sizeof(float), 3, o);
    }
    std::fclose(o);
    return 0;
}
