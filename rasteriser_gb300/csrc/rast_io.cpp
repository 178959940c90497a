// File ingest for the renderer's inputs: Wavefront OBJ + MTL (the reference loads them with
// tinyobjloader, fileloader.cpp:81-118), the lights CSV (fileloader.cpp:121-132) and raw PPM / PFM
// images for textures (the reference's Material loads textures through CImg, material.h:20-22).
//
// OBJ parsing follows the behaviour of the tinyobjloader version the reference vendors, so a file
// gives the same arrays, in the same order, as the reference's load_obj:
//   - numbers: a digit-by-digit decimal parser (integer digits accumulate as m = 10 m + d, the
//     fraction adds d * 10^-k, an exponent e gives ldexp(m * 5^e, e)), the double rounded to float;
//     a missing number is 0
//   - face indices: 1-based, 0 stays 0, negative ones count back from the elements read so far;
//     a missing uv or normal index is -1
//   - polygons become fans (v0, v[k-1], v[k])
//   - faces are grouped until `usemtl` changes the material or `g` / `o` starts a group; a group's
//     faces are appended to the current shape and a shape is kept only when its last group had
//     faces (tinyobjloader drops a shape whose faces were all flushed by `usemtl` before a `g`/`o`)
//   - MTL: `newmtl` starts a material (Kd and map_Kd are read), the last one is kept at the end of
//     the file even without a name; a name maps to its first material
// Parsing is parallel: worker threads split the file at line starts, count and parse the element
// lines of their chunk, and one pass over the chunks' face and state lines replays the grouping.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cctype>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "rast.h"
#include "rast_context.h"

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t'; }
inline bool is_digit(char c) { return (unsigned)(c - '0') < 10u; }
inline bool is_eol(char c) { return c == '\r' || c == '\n' || c == '\0'; }

// The decimal parser described above, on [s, e). False when no number starts at s.
//
// Attribution: this function follows the steps of tinyobjloader's tryParseDouble
// (tiny_obj_loader.h 1.0.5, which canmom/rasteriser vendors), because those steps decide the
// float bits of every vertex an OBJ file loads to. tinyobjloader is under the MIT License:
//   Copyright (c) 2012-2016 Syoyo Fujita and many contributors.
//   Permission is hereby granted, free of charge, to any person obtaining a copy of this software
//   and associated documentation files (the "Software"), to deal in the Software without
//   restriction, including without limitation the rights to use, copy, modify, merge, publish,
//   distribute, sublicense, and/or sell copies of the Software, and to permit persons to whom the
//   Software is furnished to do so, subject to the following conditions: The above copyright
//   notice and this permission notice shall be included in all copies or substantial portions of
//   the Software. THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS OR
//   IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF MERCHANTABILITY, FITNESS FOR A
//   PARTICULAR PURPOSE AND NONINFRINGEMENT. IN NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE
//   LIABLE FOR ANY CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT, TORT OR
//   OTHERWISE, ARISING FROM, OUT OF OR IN CONNECTION WITH THE SOFTWARE OR THE USE OR OTHER
//   DEALINGS IN THE SOFTWARE.
bool parse_real(const char* s, const char* e, double* out) {
    if (s >= e) return false;
    double mantissa = 0.0;
    int exponent = 0;
    char sign = '+', exp_sign = '+';
    const char* c = s;
    int read = 0;
    if (*c == '+' || *c == '-') {
        sign = *c;
        ++c;
    } else if (!is_digit(*c)) {
        return false;
    }
    while (c != e && is_digit(*c)) {
        mantissa *= 10;
        mantissa += (int)(*c - '0');
        ++c;
        ++read;
    }
    if (read == 0) return false;
    if (c != e) {
        bool exp_next = false;
        if (*c == '.') {
            ++c;
            read = 1;
            static const double tenth[] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
            while (c != e && is_digit(*c)) {
                mantissa += (int)(*c - '0') * (read < 8 ? tenth[read] : std::pow(10.0, -read));
                ++read;
                ++c;
            }
            exp_next = c != e;
        } else if (*c == 'e' || *c == 'E') {
            exp_next = true;
        }
        if (exp_next && (*c == 'e' || *c == 'E')) {
            ++c;
            if (c != e && (*c == '+' || *c == '-')) {
                exp_sign = *c;
                ++c;
            } else if (!is_digit(*c)) {
                return false;
            }
            read = 0;
            while (c != e && is_digit(*c)) {
                exponent *= 10;
                exponent += (int)(*c - '0');
                ++c;
                ++read;
            }
            exponent *= exp_sign == '+' ? 1 : -1;
            if (read == 0) return false;
        }
    }
    *out = (sign == '+' ? 1 : -1) * (exponent ? std::ldexp(mantissa * std::pow(5.0, exponent), exponent) : mantissa);
    return true;
}

// One whitespace-separated number at *p (0 when absent), advancing past it; it ends at the line's
// end as well.
float next_float(const char** p) {
    *p += std::strspn(*p, " \t");
    const char* end = *p + std::strcspn(*p, " \t\r\n");
    double v = 0.0;
    parse_real(*p, end, &v);
    *p = end;
    return (float)v;
}

int fix_index(int idx, int n) {
    if (idx > 0) return idx - 1;
    if (idx == 0) return 0;
    return n + idx;
}

struct Corner {
    int v = -1, vt = -1, vn = -1;
};

// i, i/j, i//k, i/j/k at *p, indices fixed against the counts so far.
Corner parse_corner(const char** p, int nv, int nvn, int nvt) {
    Corner c;
    c.v = fix_index(std::atoi(*p), nv);
    *p += std::strcspn(*p, "/ \t\r\n");
    if ((*p)[0] != '/') return c;
    ++*p;
    if ((*p)[0] == '/') {
        ++*p;
        c.vn = fix_index(std::atoi(*p), nvn);
        *p += std::strcspn(*p, "/ \t\r\n");
        return c;
    }
    c.vt = fix_index(std::atoi(*p), nvt);
    *p += std::strcspn(*p, "/ \t\r\n");
    if ((*p)[0] != '/') return c;
    ++*p;
    c.vn = fix_index(std::atoi(*p), nvn);
    *p += std::strcspn(*p, "/ \t\r\n");
    return c;
}

// First word after a keyword (what sscanf("%s") reads).
std::string first_word(const char* p) {
    p += std::strspn(p, " \t");
    return std::string(p, std::strcspn(p, " \t\r\n"));
}

// The file's lines: [start, end) offsets with the line terminators (\n, \r\n, \r) removed.
struct Line {
    size_t b, e;
};

std::vector<Line> split_lines(const std::string& s, size_t b, size_t e) {
    std::vector<Line> out;
    size_t i = b;
    while (i < e) {
        size_t j = i;
        while (j < e && s[j] != '\n' && s[j] != '\r') ++j;
        out.push_back({i, j});
        if (j < e && s[j] == '\r' && j + 1 < e && s[j + 1] == '\n') j += 2;
        else if (j < e) j += 1;
        i = j;
    }
    return out;
}

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

struct Material {
    std::string name;
    float kd[3] = {0.f, 0.f, 0.f};
    std::string map_kd;
};

// map_Kd's texture name: the first token that is not a texture option or an option's value.
std::string texture_name(const char* p) {
    static const struct { const char* opt; int args; } opts[] = {
        {"-blendu", 1}, {"-blendv", 1}, {"-clamp", 1}, {"-boost", 1}, {"-bm", 1}, {"-imfchan", 1},
        {"-type", 1}, {"-texres", 1}, {"-mm", 2}, {"-o", 3}, {"-s", 3}, {"-t", 3}};
    std::vector<std::string> tok;
    std::istringstream ss(p);
    std::string w;
    while (ss >> w) tok.push_back(w);
    for (size_t i = 0; i < tok.size(); ++i) {
        int skip = -1;
        for (const auto& o : opts)
            if (tok[i] == o.opt) skip = o.args;
        if (skip < 0) return tok[i];
        // -o / -s / -t take one to three numbers
        size_t k = i + 1, taken = 0;
        while (k < tok.size() && (int)taken < skip) {
            double v;
            const bool number = parse_real(tok[k].c_str(), tok[k].c_str() + tok[k].size(), &v);
            if (skip == 3 && taken >= 1 && !number) break;
            ++k;
            ++taken;
        }
        i = k - 1;
    }
    return std::string();
}

void load_mtl(const std::string& text, std::vector<Material>& mats, std::map<std::string, int>& names) {
    Material m;
    for (const Line& ln : split_lines(text, 0, text.size())) {
        std::string line = text.substr(ln.b, ln.e - ln.b);
        line = line.substr(0, line.find_last_not_of(" \t") + 1);
        if (line.empty()) continue;
        const char* t = line.c_str();
        t += std::strspn(t, " \t");
        if (t[0] == '\0' || t[0] == '#') continue;
        if (std::strncmp(t, "newmtl", 6) == 0 && is_space(t[6])) {
            if (!m.name.empty()) {
                names.insert({m.name, (int)mats.size()});
                mats.push_back(m);
            }
            m = Material();
            m.name = first_word(t + 7);
            continue;
        }
        if (t[0] == 'K' && t[1] == 'd' && is_space(t[2])) {
            const char* p = t + 2;
            m.kd[0] = next_float(&p);
            m.kd[1] = next_float(&p);
            m.kd[2] = next_float(&p);
            continue;
        }
        if (std::strncmp(t, "map_Kd", 6) == 0 && is_space(t[6])) {
            m.map_kd = texture_name(t + 7);
            continue;
        }
    }
    names.insert({m.name, (int)mats.size()});
    mats.push_back(m);
}

enum LineKind : unsigned char { L_OTHER, L_V, L_VN, L_VT, L_F, L_USEMTL, L_MTLLIB, L_G, L_O };

LineKind classify(const char* t) {
    if (t[0] == 'v' && is_space(t[1])) return L_V;
    if (t[0] == 'v' && t[1] == 'n' && is_space(t[2])) return L_VN;
    if (t[0] == 'v' && t[1] == 't' && is_space(t[2])) return L_VT;
    if (t[0] == 'f' && is_space(t[1])) return L_F;
    if (std::strncmp(t, "usemtl", 6) == 0 && is_space(t[6])) return L_USEMTL;
    if (std::strncmp(t, "mtllib", 6) == 0 && is_space(t[6])) return L_MTLLIB;
    if (t[0] == 'g' && is_space(t[1])) return L_G;
    if (t[0] == 'o' && is_space(t[1])) return L_O;
    return L_OTHER;
}

struct Chunk {
    std::vector<std::pair<LineKind, size_t>> lines;  // kind and the offset of its first token
    int nv = 0, nvn = 0, nvt = 0;                    // element lines in the chunk
    int v0 = 0, vn0 = 0, vt0 = 0;                    // elements before the chunk
    std::vector<std::vector<Corner>> faces;          // the chunk's face lines, parsed
};

}  // namespace

struct rast_obj {
    std::vector<float> pos, nrm, uv, kd;
    std::vector<int32_t> tris;
    std::vector<std::string> tex;
    std::vector<const char*> tex_c;
    std::string err;
};

extern "C" {

rast_status rast_obj_load(const char* obj_path, const char* mats_dir, rast_obj** out) {
    if (!obj_path || !out) return RAST_ERR_INVALID_ARG;
    *out = nullptr;
    std::string text;
    if (!read_file(obj_path, text)) {
        rast::set_thread_error(std::string("cannot read ") + obj_path);
        return RAST_ERR_INVALID_ARG;
    }
    const std::string dir = mats_dir ? mats_dir : "";
    text.push_back('\0');
    const size_t n = text.size() - 1;
    const char* base = text.c_str();

    // chunks at line starts
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t want = n < ((size_t)1 << 20) ? 1 : hw;
    std::vector<size_t> cut = {0};
    for (size_t k = 1; k < want; ++k) {
        size_t p = std::max(cut.back(), n * k / want);
        while (p < n && text[p] != '\n' && text[p] != '\r') ++p;
        while (p < n && (text[p] == '\n' || text[p] == '\r')) ++p;
        cut.push_back(p);
    }
    cut.push_back(n);
    std::vector<Chunk> chunks(cut.size() - 1);
    auto run = [&](auto&& fn) {
        std::vector<std::thread> th;
        for (size_t k = 1; k < chunks.size(); ++k) th.emplace_back(fn, k);
        fn(0);
        for (auto& t : th) t.join();
    };
    // pass 1: classify and count
    run([&](size_t k) {
        Chunk& c = chunks[k];
        for (const Line& ln : split_lines(text, cut[k], cut[k + 1])) {
            size_t t = ln.b + std::strspn(base + ln.b, " \t");
            if (t >= ln.e) continue;
            const char* p = base + t;
            if (p[0] == '#') continue;
            const LineKind kind = classify(p);
            if (kind == L_OTHER) continue;
            c.lines.push_back({kind, t});
            c.nv += kind == L_V;
            c.nvn += kind == L_VN;
            c.nvt += kind == L_VT;
        }
    });
    rast_obj* o = new rast_obj();
    int tv = 0, tvn = 0, tvt = 0;
    for (Chunk& c : chunks) {
        c.v0 = tv; c.vn0 = tvn; c.vt0 = tvt;
        tv += c.nv; tvn += c.nvn; tvt += c.nvt;
    }
    o->pos.resize(3 * (size_t)tv);
    o->nrm.resize(3 * (size_t)tvn);
    o->uv.resize(2 * (size_t)tvt);
    // pass 2: element lines into place, face lines parsed against the running counts
    run([&](size_t k) {
        Chunk& c = chunks[k];
        int iv = c.v0, ivn = c.vn0, ivt = c.vt0;
        for (const auto& kl : c.lines) {
            const char* p = base + kl.second;
            // the line ends at its terminator (replaced by the parse stopping at \r, \n)
            switch (kl.first) {
                case L_V: {
                    p += 2;
                    float* d = &o->pos[3 * (size_t)iv++];
                    d[0] = next_float(&p); d[1] = next_float(&p); d[2] = next_float(&p);
                    break;
                }
                case L_VN: {
                    p += 3;
                    float* d = &o->nrm[3 * (size_t)ivn++];
                    d[0] = next_float(&p); d[1] = next_float(&p); d[2] = next_float(&p);
                    break;
                }
                case L_VT: {
                    p += 3;
                    float* d = &o->uv[2 * (size_t)ivt++];
                    d[0] = next_float(&p); d[1] = next_float(&p);
                    break;
                }
                case L_F: {
                    p += 2;
                    p += std::strspn(p, " \t");
                    std::vector<Corner> face;
                    while (!is_eol(p[0])) {
                        face.push_back(parse_corner(&p, iv, ivn, ivt));
                        p += std::strspn(p, " \t\r");
                    }
                    c.faces.push_back(std::move(face));
                    break;
                }
                default:
                    break;
            }
        }
    });
    // the grouping, in file order
    std::vector<Material> mats;
    std::map<std::string, int> names;
    int material = -1;
    std::vector<const std::vector<Corner>*> group;
    std::vector<int32_t> shape;  // triangles of the current shape (10 ints each)
    auto export_group = [&]() -> bool {
        if (group.empty()) return false;
        for (const auto* f : group) {
            const std::vector<Corner>& face = *f;
            if (face.size() < 2) continue;
            Corner c0 = face[0], c1, c2 = face[1];
            for (size_t k = 2; k < face.size(); ++k) {
                c1 = c2;
                c2 = face[k];
                const int32_t t[10] = {c0.v, c1.v, c2.v, c0.vn, c1.vn, c2.vn, c0.vt, c1.vt, c2.vt, material};
                shape.insert(shape.end(), t, t + 10);
            }
        }
        return true;
    };
    auto keep_shape = [&]() {
        o->tris.insert(o->tris.end(), shape.begin(), shape.end());
        shape.clear();
    };
    for (const Chunk& c : chunks) {
        size_t fi = 0;
        for (const auto& kl : c.lines) {
            const char* p = base + kl.second;
            switch (kl.first) {
                case L_F:
                    group.push_back(&c.faces[fi++]);
                    break;
                case L_USEMTL: {
                    const std::string nm = first_word(p + 7);
                    const auto it = names.find(nm);
                    const int id = it == names.end() ? -1 : it->second;
                    if (id != material) {
                        export_group();
                        group.clear();
                        material = id;
                    }
                    break;
                }
                case L_MTLLIB: {
                    std::vector<std::string> files;
                    std::string rest(p + 7, std::strcspn(p + 7, "\r\n"));
                    std::istringstream ss(rest);
                    std::string item;
                    while (std::getline(ss, item, ' ')) files.push_back(item);
                    for (const std::string& f : files) {
                        std::string mtl;
                        if (read_file(dir + f, mtl)) {
                            load_mtl(mtl, mats, names);
                            break;
                        }
                    }
                    break;
                }
                case L_G:
                case L_O:
                    if (export_group()) keep_shape();
                    else shape.clear();
                    group.clear();
                    break;
                default:
                    break;
            }
        }
    }
    if (export_group()) keep_shape();
    for (const Material& m : mats) {
        o->kd.insert(o->kd.end(), m.kd, m.kd + 3);
        o->tex.push_back(m.map_kd.empty() ? std::string() : dir + m.map_kd);
    }
    for (const std::string& t : o->tex) o->tex_c.push_back(t.c_str());
    *out = o;
    return RAST_OK;
}

void rast_obj_free(rast_obj* o) { delete o; }

rast_status rast_obj_view(const rast_obj* o, rast_obj_data* v) {
    if (!o || !v) return RAST_ERR_INVALID_ARG;
    v->pos = o->pos.data();
    v->nv = (int64_t)o->pos.size() / 3;
    v->nrm = o->nrm.data();
    v->nn = (int64_t)o->nrm.size() / 3;
    v->uv = o->uv.data();
    v->nuv = (int64_t)o->uv.size() / 2;
    v->tris = o->tris.data();
    v->ntri = (int64_t)o->tris.size() / 10;
    v->kd = o->kd.data();
    v->nmat = (int32_t)o->kd.size() / 3;
    v->textures = o->tex_c.data();
    return RAST_OK;
}

rast_status rast_lights_load(const char* path, float* lights7, int32_t cap, int32_t* n) {
    if (!path || !n || cap < 0 || (cap > 0 && !lights7)) return RAST_ERR_INVALID_ARG;
    std::string text;
    if (!read_file(path, text)) {
        rast::set_thread_error(std::string("cannot read ") + path);
        return RAST_ERR_INVALID_ARG;
    }
    int32_t count = 0;
    for (const Line& ln : split_lines(text, 0, text.size())) {
        std::string line = text.substr(ln.b, ln.e - ln.b);
        if (line.find_first_not_of(" \t") == std::string::npos) continue;
        float f[7];
        const char* p = line.c_str();
        for (int k = 0; k < 7; ++k) {
            char* end = nullptr;
            f[k] = std::strtof(p, &end);
            if (end == p) {
                rast::set_thread_error("lights line " + std::to_string(count + 1) + ": 7 numbers expected");
                return RAST_ERR_INVALID_ARG;
            }
            p = end;
            p += std::strspn(p, " \t");
            if (k < 6) {
                if (*p != ',') {
                    rast::set_thread_error("lights line " + std::to_string(count + 1) + ": 7 numbers expected");
                    return RAST_ERR_INVALID_ARG;
                }
                ++p;
            }
        }
        if (count < cap)
            for (int k = 0; k < 7; ++k) lights7[7 * (size_t)count + k] = f[k];
        ++count;
    }
    *n = count;
    return RAST_OK;
}

// Netpbm (P2, P3, P5, P6; maxval up to 65535) and PFM (PF, Pf) images as floats, planar
// (x + y*W + c*W*H), rows top to bottom, the values as stored (0..maxval; PFM as written, rows
// flipped to top-first). Two calls: with out NULL it reports w, h, channels.
rast_status rast_image_load(const char* path, uint32_t* w, uint32_t* h, uint32_t* channels, float* out, size_t cap) {
    if (!path || !w || !h || !channels) return RAST_ERR_INVALID_ARG;
    std::string s;
    if (!read_file(path, s) || s.size() < 2 || s[0] != 'P') {
        rast::set_thread_error(std::string("not a PPM/PGM/PFM image: ") + path);
        return RAST_ERR_INVALID_ARG;
    }
    const char kind = s[1];
    size_t i = 2;
    auto next_token = [&](std::string& tok) -> bool {
        for (;;) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
            if (i < s.size() && s[i] == '#') {
                while (i < s.size() && s[i] != '\n') ++i;
                continue;
            }
            break;
        }
        const size_t b = i;
        while (i < s.size() && !std::isspace((unsigned char)s[i])) ++i;
        tok = s.substr(b, i - b);
        return !tok.empty();
    };
    std::string tw, th, tm;
    const bool pfm = kind == 'F' || kind == 'f';
    const int ch = (kind == '3' || kind == '6' || kind == 'F') ? 3 : 1;
    if (!(kind == '2' || kind == '3' || kind == '5' || kind == '6' || pfm) || !next_token(tw) || !next_token(th) ||
        !next_token(tm)) {
        rast::set_thread_error(std::string("unsupported image header: ") + path);
        return RAST_ERR_INVALID_ARG;
    }
    const long W = std::atol(tw.c_str()), H = std::atol(th.c_str());
    const double maxval = std::atof(tm.c_str());
    if (W <= 0 || H <= 0 || W > 65536 || H > 65536 || (!pfm && (maxval < 1 || maxval > 65535))) {
        rast::set_thread_error(std::string("bad image size or range: ") + path);
        return RAST_ERR_INVALID_ARG;
    }
    *w = (uint32_t)W;
    *h = (uint32_t)H;
    *channels = (uint32_t)ch;
    const size_t npx = (size_t)W * H;
    if (!out) return RAST_OK;
    if (cap < npx * ch) return RAST_ERR_INVALID_ARG;
    if (kind == '2' || kind == '3') {
        std::string tok;
        for (size_t k = 0; k < npx * ch; ++k) {
            if (!next_token(tok)) {
                rast::set_thread_error(std::string("truncated image: ") + path);
                return RAST_ERR_INVALID_ARG;
            }
            out[(k % ch) * npx + k / ch] = (float)std::atof(tok.c_str());
        }
        return RAST_OK;
    }
    ++i;  // the single whitespace after the header
    if (pfm) {
        const bool little = maxval < 0;
        if (s.size() < i + 4 * npx * ch) {
            rast::set_thread_error(std::string("truncated image: ") + path);
            return RAST_ERR_INVALID_ARG;
        }
        for (long y = 0; y < H; ++y)
            for (long x = 0; x < W; ++x)
                for (int c = 0; c < ch; ++c) {
                    const unsigned char* b = (const unsigned char*)s.data() + i + 4 * (((size_t)y * W + x) * ch + c);
                    const uint32_t u = little ? (b[0] | b[1] << 8 | b[2] << 16 | (uint32_t)b[3] << 24)
                                              : (b[3] | b[2] << 8 | b[1] << 16 | (uint32_t)b[0] << 24);
                    float f;
                    std::memcpy(&f, &u, 4);
                    out[(size_t)c * npx + (size_t)(H - 1 - y) * W + x] = f;
                }
        return RAST_OK;
    }
    const int bytes = maxval > 255 ? 2 : 1;
    if (s.size() < i + bytes * npx * ch) {
        rast::set_thread_error(std::string("truncated image: ") + path);
        return RAST_ERR_INVALID_ARG;
    }
    for (size_t k = 0; k < npx * ch; ++k) {
        const unsigned char* b = (const unsigned char*)s.data() + i + bytes * k;
        out[(k % ch) * npx + k / ch] = (float)(bytes == 2 ? (b[0] << 8 | b[1]) : b[0]);
    }
    return RAST_OK;
}

}  // extern "C"
