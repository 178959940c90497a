// rast_render: the reference's renderer (renderer.cpp) as a headless command-line program over the
// C ABI. Same options as arguments.cpp (-o/--obj, -l/--lights, --mats-dir, -x/--width,
// -y/--height, -s/--spin, -f/--flat, --wind-clockwise, --rx/--ry/--rz, --scale, --dx/--dy/--dz),
// the same defaults (540 x 304, the add_square model when no --obj, the 45 deg / 0.1 / 6 projection)
// and the same two modes:
//   - one frame: draws and writes the frame and the depth view (renderer.cpp:88-93) as
//     frame.ppm and depth.pgm (binary PPM / PGM instead of PNG), plus depth.pfm (the raw depths)
//   - --spin: the rotating model (renderer.cpp:94-125) without a window: --frames frames drawn on
//     the device one after another (clear, draw), ry advancing by --step radians per frame (the
//     reference advances it by each frame's wall-clock duration); prints the frame rate and, with
//     --dump, writes frame_NNNN.ppm for every frame.
// -f/--flat shades with face normals computed in the path (readme.md:46; the reference parses the
// flag but never reads it). Extra options: --frames N (60), --step S (1/60), --out DIR (.), --dump,
// --device D, --deferred (per-light shading in a separate pass), and the projection and light units
// the reference hard-codes: --fovy DEG (45), --near Z (0.1), --far Z (6) (geometry.cpp:30) and
// --light-scale K (1: every light's intensity is multiplied by K as it is loaded).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rast.h"

namespace {

struct Options {
    std::string obj, lights, mats_dir, out = ".";
    unsigned width = 540, height = 304;
    bool spin = false, flat = false, wind_clockwise = false, dump = false, deferred = false;
    float rx = 0.f, ry = 0.f, rz = 0.f, scale = 1.f, dx = 0.f, dy = 0.f, dz = 0.f;
    int frames = 60, device = 0;
    float step = 1.f / 60.f;
    float fovy = 45.f, z_near = 0.1f, z_far = 6.f, light_scale = 1.f;
};

[[noreturn]] void usage(const char* msg) {
    std::fprintf(stderr,
                 "Error: %s\nusage: rast_render -l lights.csv [-o model.obj] [--mats-dir dir/] [-x width] "
                 "[-y height]\n  [-s] [-f] [--wind-clockwise] [--rx a] [--ry a] [--rz a] [--scale s] [--dx d] [--dy d] "
                 "[--dz d]\n  [--frames n] [--step rad] [--out dir] [--dump] [--device d] [--deferred]\n"
                 "  [--fovy deg] [--near z] [--far z] [--light-scale k]\n",
                 msg);
    std::exit(1);
}

Options parse(int argc, char** argv) {
    Options o;
    bool have_lights = false;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto value = [&]() -> const char* {
            if (i + 1 >= argc) usage(("missing value for " + a).c_str());
            return argv[++i];
        };
        auto num = [&]() -> float {
            const char* v = value();
            char* end = nullptr;
            const float f = std::strtof(v, &end);
            if (end == v || *end) usage(("not a number for " + a + ": " + v).c_str());
            return f;
        };
        auto uint = [&]() -> unsigned {
            const char* v = value();
            char* end = nullptr;
            const unsigned long u = std::strtoul(v, &end, 10);
            if (end == v || *end || u == 0 || u > 32768) usage(("bad value for " + a + ": " + v).c_str());
            return (unsigned)u;
        };
        if (a == "-o" || a == "--obj") o.obj = value();
        else if (a == "-l" || a == "--lights") { o.lights = value(); have_lights = true; }
        else if (a == "--mats-dir") o.mats_dir = value();
        else if (a == "-x" || a == "--width") o.width = uint();
        else if (a == "-y" || a == "--height") o.height = uint();
        else if (a == "-s" || a == "--spin") o.spin = true;
        else if (a == "-f" || a == "--flat") o.flat = true;
        else if (a == "--wind-clockwise") o.wind_clockwise = true;
        else if (a == "--rx") o.rx = num();
        else if (a == "--ry") o.ry = num();
        else if (a == "--rz") o.rz = num();
        else if (a == "--scale") o.scale = num();
        else if (a == "--dx") o.dx = num();
        else if (a == "--dy") o.dy = num();
        else if (a == "--dz") o.dz = num();
        else if (a == "--frames") o.frames = (int)uint();
        else if (a == "--step") o.step = num();
        else if (a == "--out") o.out = value();
        else if (a == "--dump") o.dump = true;
        else if (a == "--device") o.device = (int)num();
        else if (a == "--deferred") o.deferred = true;
        else if (a == "--fovy") o.fovy = num();
        else if (a == "--near") o.z_near = num();
        else if (a == "--far") o.z_far = num();
        else if (a == "--light-scale") o.light_scale = num();
        else usage(("unknown option " + a).c_str());
    }
    if (!have_lights) usage("-l/--lights is required");
    if (!(o.fovy > 0.f && o.fovy < 180.f)) usage("--fovy must be in (0, 180) degrees");
    if (!(o.z_near > 0.f && o.z_far > o.z_near)) usage("--near must be > 0 and --far > --near");
    return o;
}

void check(rast_status st, rast_ctx* ctx, const char* what) {
    if (st == RAST_OK) return;
    std::fprintf(stderr, "%s failed: %s: %s\n", what, rast_status_string(st), rast_last_error(ctx));
    std::exit(2);
}

bool write_ppm(const std::string& path, const std::vector<uint8_t>& planar, unsigned w, unsigned h) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "P6\n%u %u\n255\n", w, h);
    std::vector<uint8_t> row(3 * (size_t)w);
    const size_t npx = (size_t)w * h;
    for (unsigned y = 0; y < h; ++y) {
        for (unsigned x = 0; x < w; ++x)
            for (int c = 0; c < 3; ++c) row[3 * x + c] = planar[c * npx + (size_t)y * w + x];
        std::fwrite(row.data(), 1, row.size(), f);
    }
    return std::fclose(f) == 0;
}

bool write_pgm(const std::string& path, const std::vector<uint8_t>& v, unsigned w, unsigned h) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "P5\n%u %u\n255\n", w, h);
    std::fwrite(v.data(), 1, v.size(), f);
    return std::fclose(f) == 0;
}

bool write_pfm(const std::string& path, const std::vector<float>& v, unsigned w, unsigned h) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "Pf\n%u %u\n-1.0\n", w, h);  // little endian, rows bottom first
    for (unsigned y = h; y-- > 0;) std::fwrite(v.data() + (size_t)y * w, sizeof(float), w, f);
    return std::fclose(f) == 0;
}

}  // namespace

int main(int argc, char** argv) {
    const Options o = parse(argc, argv);

    // lights
    int32_t nl = 0;
    check(rast_lights_load(o.lights.c_str(), nullptr, 0, &nl), nullptr, "lights");
    std::vector<float> lights(7 * (size_t)(nl > 0 ? nl : 1));
    check(rast_lights_load(o.lights.c_str(), lights.data(), nl, &nl), nullptr, "lights");
    if (o.light_scale != 1.f)
        for (int32_t i = 0; i < nl; ++i) lights[7 * (size_t)i + 3] *= o.light_scale;

    // model: the OBJ, or renderer.cpp's add_square
    std::vector<float> pos, nrm, uv, kd;
    std::vector<int32_t> tris;
    std::vector<std::string> textures;
    if (!o.obj.empty()) {
        rast_obj* obj = nullptr;
        check(rast_obj_load(o.obj.c_str(), o.mats_dir.c_str(), &obj), nullptr, "obj");
        rast_obj_data d;
        rast_obj_view(obj, &d);
        pos.assign(d.pos, d.pos + 3 * d.nv);
        nrm.assign(d.nrm, d.nrm + 3 * d.nn);
        uv.assign(d.uv, d.uv + 2 * d.nuv);
        tris.assign(d.tris, d.tris + 10 * d.ntri);
        kd.assign(d.kd, d.kd + 3 * d.nmat);
        for (int32_t i = 0; i < d.nmat; ++i) textures.push_back(d.textures[i]);
        rast_obj_free(obj);
        std::printf("Loaded model %s: %zu triangles.\n", o.obj.c_str(), tris.size() / 10);
    } else {
        pos = {-0.5f, -0.5f, 0.f, 0.5f, -0.5f, 0.f, -0.5f, 0.5f, 0.f, 0.5f, 0.5f, 0.f};
        nrm = {0.f, 0.f, 1.f};
        uv = {0.f, 0.f, 1.f, 0.f, 0.f, 1.f, 1.f, 1.f};
        tris = {0, 1, 2, 0, 0, 0, 0, 1, 2, 0, 2, 1, 3, 0, 0, 0, 2, 1, 3, 0};
        kd = {1.f, 1.f, 1.f};
    }

    rast_ctx* ctx = nullptr;
    check(rast_create(&ctx, o.device), nullptr, "create");
    check(rast_upload_mesh(ctx, pos.data(), (int64_t)pos.size() / 3, nrm.data(), (int64_t)nrm.size() / 3,
                           uv.empty() ? nullptr : uv.data(), (int64_t)uv.size() / 2, tris.data(),
                           (int64_t)tris.size() / 10, kd.data(), (int32_t)kd.size() / 3),
          ctx, "upload");
    // textures: raw images (PPM / PGM / PFM); other formats are drawn with the material's Kd
    for (size_t i = 0; i < textures.size(); ++i) {
        if (textures[i].empty()) continue;
        uint32_t tw = 0, th = 0, tc = 0;
        if (rast_image_load(textures[i].c_str(), &tw, &th, &tc, nullptr, 0) != RAST_OK || tc < 3) {
            std::fprintf(stderr, "note: texture %s is not a 3-channel PPM / PFM; material %zu uses its Kd\n",
                         textures[i].c_str(), i);
            continue;
        }
        std::vector<float> texels((size_t)tw * th * tc);
        check(rast_image_load(textures[i].c_str(), &tw, &th, &tc, texels.data(), texels.size()), nullptr, "texture");
        check(rast_upload_texture(ctx, (int32_t)i, texels.data(), tw, th, tc), ctx, "texture");
    }
    if (o.deferred) check(rast_set_option(ctx, RAST_OPT_SHADER, RAST_SHADER_EXACT_DEFERRED), ctx, "option");

    const unsigned W = o.width, H = o.height;
    const size_t npx = (size_t)W * H;
    const float disp[3] = {o.dx, o.dy, o.dz};
    const uint32_t shading = (o.wind_clockwise ? RAST_WIND_CLOCKWISE : 0u) | (o.flat ? RAST_FLAT : 0u);
    const uint32_t flags = shading | RAST_CLEAR;
    float model[16], view[16], mv[16], cam[16], nm[16];
    std::vector<float> lt(lights.size());
    auto frame_inputs = [&](float ry) {
        const float angles[3] = {o.rx, ry, o.rz};
        check(rast_frame_matrices(W, H, o.scale, disp, angles, o.fovy, o.z_near, o.z_far, model, view, mv, cam, nm),
              ctx, "matrices");
        check(rast_transform_lights(view, lights.data(), nl, lt.data()), ctx, "lights");
        check(rast_set_lights(ctx, lt.data(), nl), ctx, "lights");
    };

    std::vector<uint8_t> frame(3 * npx);
    std::vector<float> depth(npx, 1.f);
    if (!o.spin) {
        frame_inputs(o.ry);
        check(rast_draw(ctx, cam, nm, W, H, flags, frame.data(), depth.data(), nullptr), ctx, "draw");
        std::vector<uint8_t> view8(npx);
        check(rast_depth_to_u8_host(ctx, depth.data(), W, H, view8.data()), ctx, "depth view");
        const std::string base = o.out + "/";
        if (!write_ppm(base + "frame.ppm", frame, W, H) || !write_pgm(base + "depth.pgm", view8, W, H) ||
            !write_pfm(base + "depth.pfm", depth, W, H)) {
            std::fprintf(stderr, "cannot write to %s\n", o.out.c_str());
            return 3;
        }
        std::printf("Wrote %sframe.ppm, %sdepth.pgm and %sdepth.pfm (%ux%u).\n", base.c_str(), base.c_str(),
                    base.c_str(), W, H);
    } else {
        rast_spin_desc sd = {};
        sd.width = W;
        sd.height = H;
        sd.flags = shading;
        sd.scale = o.scale;
        sd.disp[0] = o.dx; sd.disp[1] = o.dy; sd.disp[2] = o.dz;
        sd.angles[0] = o.rx; sd.angles[1] = o.ry; sd.angles[2] = o.rz;
        sd.step = o.step;
        sd.fovy_deg = o.fovy;
        sd.z_near = o.z_near;
        sd.z_far = o.z_far;
        sd.lights7 = lights.data();
        sd.nl = nl;
        double seconds = 0.0;
        if (o.dump) {  // frame by frame, each copied back and written
            for (int k = 0; k < o.frames; ++k) {
                sd.frames = 1;
                sd.angles[1] = o.ry + (float)k * o.step;
                double s1 = 0.0;
                check(rast_spin(ctx, &sd, frame.data(), nullptr, &s1), ctx, "spin");
                seconds += s1;
                char name[64];
                std::snprintf(name, sizeof name, "/frame_%04d.ppm", k);
                if (!write_ppm(o.out + name, frame, W, H)) {
                    std::fprintf(stderr, "cannot write to %s\n", o.out.c_str());
                    return 3;
                }
            }
        } else {
            sd.frames = o.frames;
            check(rast_spin(ctx, &sd, frame.data(), depth.data(), &seconds), ctx, "spin");
            if (!write_ppm(o.out + "/frame.ppm", frame, W, H)) {
                std::fprintf(stderr, "cannot write to %s\n", o.out.c_str());
                return 3;
            }
        }
        std::printf("%d frames of %ux%u in %.4f s: %.1f frames/s\n", o.frames, W, H, seconds, o.frames / seconds);
    }
    rast_destroy(ctx);
    return 0;
}
