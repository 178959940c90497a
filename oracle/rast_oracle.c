/* Oracle test infrastructure: plain-C restatement of canmom/rasteriser's draw_frame. Only tests,
 * the smoke check and bench.py's CPU-baseline leg use it, and only as the checker.
 *
 * Every floating-point expression keeps the reference's operation order; the file is compiled
 * with -ffp-contract=off so that no multiply-add is fused. glm arithmetic follows the order fixed
 * by the project's glm subset (rasteriser_gb300/compat/glm/detail/subset_core.hpp). */
#include "rast_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z, w; } v4;
typedef struct { float x, y, z; } v3;

/* glm::min / glm::max for scalars (x < y ? x : y, x > y ? x : y). */
static inline float gmin(float x, float y) { return x < y ? x : y; }
static inline float gmax(float x, float y) { return x > y ? x : y; }

/* mat4 * vec4 as (c0*x + c1*y) + (c2*z + c3*w), column-major m. Row r of the result. */
static inline float mrow(const float* m, int r, float x, float y, float z, float w) {
    float lo = m[0 + r] * x + m[4 + r] * y;
    float hi = m[8 + r] * z + m[12 + r] * w;
    return lo + hi;
}

/* geometry.cpp:44-50 (transform_point), 52-60 (z_divide), 62-74 (remap_ndc, ndc_to_raster). */
static inline v4 raster_vertex(const float* cam, const float* p, float wf, float hf) {
    float cx = mrow(cam, 0, p[0], p[1], p[2], 1.f);
    float cy = mrow(cam, 1, p[0], p[1], p[2], 1.f);
    float cz = mrow(cam, 2, p[0], p[1], p[2], 1.f);
    float cw = mrow(cam, 3, p[0], p[1], p[2], 1.f);
    float nx = cx / cw, ny = cy / cw, nz = cz / cw, iw = 1.f / cw;
    v4 r;
    r.x = 0.5f * (nx + 1.0f) * wf;
    r.y = 0.5f * (-ny + 1.0f) * hf;
    r.z = nz;
    r.w = iw;
    return r;
}

/* geometry.cpp:35-42 (transform_direction) with the normal matrix. */
static inline v3 camera_normal(const float* nm, const float* n) {
    v3 r;
    r.x = mrow(nm, 0, n[0], n[1], n[2], 0.f);
    r.y = mrow(nm, 1, n[0], n[1], n[2], 0.f);
    r.z = mrow(nm, 2, n[0], n[1], n[2], 0.f);
    return r;
}

void oracle_raster_vertices(const float* camera, const float* pos, int64_t nv, uint32_t width,
                            uint32_t height, float* out4) {
    const float wf = (float)(int)width, hf = (float)(int)height;
    for (int64_t i = 0; i < nv; ++i) {
        v4 r = raster_vertex(camera, pos + 3 * i, wf, hf);
        out4[4 * i + 0] = r.x;
        out4[4 * i + 1] = r.y;
        out4[4 * i + 2] = r.z;
        out4[4 * i + 3] = r.w;
    }
}

/* shading.cpp:20-34. lights7: trans_dir xyz, intensity, colour rgb. */
static inline void shade(v3 n, v3 albedo, const float* lights7, int32_t nl, uint32_t* out3) {
    const float one_over_pi = 0.318309886183790671537767526745028724f;
    float ax = 0.f, ay = 0.f, az = 0.f; /* std::accumulate from vec3(0) */
    for (int32_t l = 0; l < nl; ++l) {
        const float* L = lights7 + 7 * l;
        float I = L[3];
        float cx = I * L[4], cy = I * L[5], cz = I * L[6];
        cx = cx * albedo.x;
        cy = cy * albedo.y;
        cz = cz * albedo.z;
        float d = (n.x * -L[0] + n.y * -L[1]) + n.z * -L[2];
        float m = gmax(0.f, d);
        cx = cx * m;
        cy = cy * m;
        cz = cz * m;
        cx = cx * one_over_pi;
        cy = cy * one_over_pi;
        cz = cz * one_over_pi;
        ax = ax + cx;
        ay = ay + cy;
        az = az + cz;
    }
    out3[0] = (uint32_t)gmin(ax, 255.f);
    out3[1] = (uint32_t)gmin(ay, 255.f);
    out3[2] = (uint32_t)gmin(az, 255.f);
}

void oracle_shade(const float* normal3, const float* albedo3, const float* lights7, int32_t nl,
                  uint32_t* out3) {
    v3 n = {normal3[0], normal3[1], normal3[2]};
    v3 a = {albedo3[0], albedo3[1], albedo3[2]};
    shade(n, a, lights7, nl, out3);
}

/* ---- per-frame matrices and lights (drawing.cpp:221-238) -------------------------------------
 * 4x4 matrices are 16 floats, column major (m[4*c + r] is row r of column c), in the operation
 * order of the project's glm subset: mat4*mat4 sums each column left to right, translate and
 * rotate post-multiply, normalize is v * (1 / sqrt(dot(v, v))). */
static void m4_identity(float* m, float d) {
    for (int i = 0; i < 16; ++i) m[i] = 0.f;
    m[0] = m[5] = m[10] = m[15] = d;
}

static void m4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k)
            r[4 * c + k] = ((a[k] * b[4 * c] + a[4 + k] * b[4 * c + 1]) + a[8 + k] * b[4 * c + 2]) +
                           a[12 + k] * b[4 * c + 3];
    memcpy(out, r, sizeof r);
}

/* glm::rotate(mat4(1), angle, axis): Rodrigues' rotation, columns R[j]. */
static void m4_rotation(float angle, float ax, float ay, float az, float* out) {
    const float c = cosf(angle), s = sinf(angle);
    const float inv = 1.0f / sqrtf((ax * ax + ay * ay) + az * az);
    const float kx = ax * inv, ky = ay * inv, kz = az * inv;
    const float omc = 1.0f - c;
    const float tx = omc * kx, ty = omc * ky, tz = omc * kz;
    const float R[3][3] = {{c + tx * kx, tx * ky + s * kz, tx * kz - s * ky},
                           {ty * kx - s * kz, c + ty * ky, ty * kz + s * kx},
                           {tz * kx + s * ky, tz * ky - s * kx, c + tz * kz}};
    /* identity columns times R: (m0*R.x + m1*R.y) + m2*R.z with m = I */
    float id[16];
    m4_identity(id, 1.f);
    for (int j = 0; j < 3; ++j)
        for (int r = 0; r < 4; ++r)
            out[4 * j + r] = (id[r] * R[j][0] + id[4 + r] * R[j][1]) + id[8 + r] * R[j][2];
    for (int r = 0; r < 4; ++r) out[12 + r] = id[12 + r];
}

/* geometry.cpp:22-25: translate(I, d) * rotate(ry) * rotate(rx) * rotate(rz) * scale(f). */
static void transformation_matrix(float factor, const float* d, const float* tb, float* out) {
    float T[16], Ry[16], Rx[16], Rz[16], S[16], acc[16];
    m4_identity(T, 1.f);
    for (int r = 0; r < 4; ++r) /* glm::translate: ((m0*dx + m1*dy) + m2*dz) + m3 */
        T[12 + r] = ((T[r] * d[0] + T[4 + r] * d[1]) + T[8 + r] * d[2]) + T[12 + r];
    m4_rotation(tb[1], 0.f, 1.f, 0.f, Ry);
    m4_rotation(tb[0], 1.f, 0.f, 0.f, Rx);
    m4_rotation(tb[2], 0.f, 0.f, 1.f, Rz);
    m4_identity(S, 1.f);
    for (int r = 0; r < 4; ++r) { S[r] = S[r] * factor; S[4 + r] = S[4 + r] * factor; S[8 + r] = S[8 + r] * factor; }
    m4_mul(T, Ry, acc);
    m4_mul(acc, Rx, acc);
    m4_mul(acc, Rz, acc);
    m4_mul(acc, S, out);
}

/* glm::inverse through the adjugate (the 2x2 minors of the top and bottom row pairs). */
static void m4_inverse(const float* m, float* out) {
#define A(r, c) m[4 * (c) + (r)]
    const float a00 = A(0, 0), a01 = A(0, 1), a02 = A(0, 2), a03 = A(0, 3);
    const float a10 = A(1, 0), a11 = A(1, 1), a12 = A(1, 2), a13 = A(1, 3);
    const float a20 = A(2, 0), a21 = A(2, 1), a22 = A(2, 2), a23 = A(2, 3);
    const float a30 = A(3, 0), a31 = A(3, 1), a32 = A(3, 2), a33 = A(3, 3);
#undef A
    const float s0 = a00 * a11 - a10 * a01, s1 = a00 * a12 - a10 * a02, s2 = a00 * a13 - a10 * a03;
    const float s3 = a01 * a12 - a11 * a02, s4 = a01 * a13 - a11 * a03, s5 = a02 * a13 - a12 * a03;
    const float c5 = a22 * a33 - a32 * a23, c4 = a21 * a33 - a31 * a23, c3 = a21 * a32 - a31 * a22;
    const float c2 = a20 * a33 - a30 * a23, c1 = a20 * a32 - a30 * a22, c0 = a20 * a31 - a30 * a21;
    const float det = (s0 * c5 - s1 * c4 + s2 * c3) + (s3 * c2 - s4 * c1 + s5 * c0);
    const float inv = 1.0f / det;
#define B(r, c) out[4 * (c) + (r)]
    B(0, 0) = ( a11 * c5 - a12 * c4 + a13 * c3) * inv;
    B(0, 1) = (-a01 * c5 + a02 * c4 - a03 * c3) * inv;
    B(0, 2) = ( a31 * s5 - a32 * s4 + a33 * s3) * inv;
    B(0, 3) = (-a21 * s5 + a22 * s4 - a23 * s3) * inv;
    B(1, 0) = (-a10 * c5 + a12 * c2 - a13 * c1) * inv;
    B(1, 1) = ( a00 * c5 - a02 * c2 + a03 * c1) * inv;
    B(1, 2) = (-a30 * s5 + a32 * s2 - a33 * s1) * inv;
    B(1, 3) = ( a20 * s5 - a22 * s2 + a23 * s1) * inv;
    B(2, 0) = ( a10 * c4 - a11 * c2 + a13 * c0) * inv;
    B(2, 1) = (-a00 * c4 + a01 * c2 - a03 * c0) * inv;
    B(2, 2) = ( a30 * s4 - a31 * s2 + a33 * s0) * inv;
    B(2, 3) = (-a20 * s4 + a21 * s2 - a23 * s0) * inv;
    B(3, 0) = (-a10 * c3 + a11 * c1 - a12 * c0) * inv;
    B(3, 1) = ( a00 * c3 - a01 * c1 + a02 * c0) * inv;
    B(3, 2) = (-a30 * s3 + a31 * s1 - a32 * s0) * inv;
    B(3, 3) = ( a20 * s3 - a21 * s1 + a22 * s0) * inv;
#undef B
}

int oracle_frame_matrices(uint32_t width, uint32_t height, float scale, const float* disp, const float* angles,
                          float fovy_deg, float z_near, float z_far, float* model, float* view,
                          float* modelview, float* camera, float* normal) {
    if (width == 0 || height == 0 || !disp || !angles || !model || !view || !modelview || !camera || !normal)
        return -1;
    /* arguments.cpp:39 */
    const float aspect = (float)width / (float)height;
    const float zero[3] = {0.f, 0.f, 0.f}, eye[3] = {0.f, 0.f, -3.f};
    transformation_matrix(scale, disp, angles, model);   /* drawing.cpp:222 */
    transformation_matrix(1.f, eye, zero, view);          /* drawing.cpp:224 */
    m4_mul(view, model, modelview);                       /* drawing.cpp:226 */
    /* geometry.cpp:27-33 with the caller's projection: glm::perspective(radians(fovy), ...) */
    const float fovy = fovy_deg * (float)0.01745329251994329576923690768489;
    const float th = tanf(fovy / 2.0f);
    float P[16];
    m4_identity(P, 0.f);
    P[0] = 1.0f / (aspect * th);
    P[5] = 1.0f / th;
    P[10] = -(z_far + z_near) / (z_far - z_near);
    P[11] = -1.0f;
    P[14] = -(2.0f * z_far * z_near) / (z_far - z_near);
    m4_mul(P, modelview, camera);
    /* geometry.cpp:101: transpose(inverse(modelview)) */
    float inv[16];
    m4_inverse(modelview, inv);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) normal[4 * c + r] = inv[4 * r + c];
    return 0;
}

int oracle_transform_lights(const float* view, const float* lights_in, int32_t n, float* lights_out) {
    if (n < 0 || (n > 0 && (!view || !lights_in || !lights_out))) return -1;
    for (int32_t i = 0; i < n; ++i) {
        const float* L = lights_in + 7 * i;
        float rec[7];
        memcpy(rec, L, sizeof rec);
        /* geometry.cpp:35-42 transform_direction (w = 0), then normalize (geometry.cpp:124-127) */
        const float tx = mrow(view, 0, rec[0], rec[1], rec[2], 0.f);
        const float ty = mrow(view, 1, rec[0], rec[1], rec[2], 0.f);
        const float tz = mrow(view, 2, rec[0], rec[1], rec[2], 0.f);
        const float inv = 1.0f / sqrtf((tx * tx + ty * ty) + tz * tz);
        rec[0] = tx * inv;
        rec[1] = ty * inv;
        rec[2] = tz * inv;
        memcpy(lights_out + 7 * i, rec, sizeof rec);
    }
    return 0;
}

/* CImg's linear_atXY(fx, fy, 0, c) with Neumann boundaries: the coordinates clamped to the image
 * (cimg::cut), the integer corner, and the bilinear blend in CImg's order of operations. */
static float cimg_linear_xy(const float* img, int w, int h, int c, float fx, float fy) {
    const float wm = (float)(w - 1), hm = (float)(h - 1);
    const float nfx = fx < 0.f ? 0.f : (fx > wm ? wm : fx);
    const float nfy = fy < 0.f ? 0.f : (fy > hm ? hm : fy);
    const unsigned x = (unsigned)nfx, y = (unsigned)nfy;
    const float dx = nfx - (float)x, dy = nfy - (float)y;
    const unsigned nx = dx > 0 ? x + 1 : x, ny = dy > 0 ? y + 1 : y;
    const size_t plane = (size_t)w * h, co = (size_t)c * plane;
    const float Icc = img[co + x + (size_t)y * w], Inc = img[co + nx + (size_t)y * w];
    const float Icn = img[co + x + (size_t)ny * w], Inn = img[co + nx + (size_t)ny * w];
    return Icc + dx * (Inc - Icc + dy * (Icc + Inn - Icn - Inc)) + dy * (Icn - Icc);
}

int oracle_draw_frame(const oracle_frame* f, uint8_t* frame, float* depth, uint32_t* tri_id,
                      uint64_t* stats) {
    if (!f || !frame || !depth || f->width == 0 || f->height == 0) return -1;
    const uint32_t W = f->width, H = f->height;
    const size_t plane = (size_t)W * H;
    const float wf = (float)(int)W, hf = (float)(int)H;
    /* drawing.cpp:84: vec2 image_bottom_right(image_width - 1, image_height - 1) */
    const float brx_lim = (float)(W - 1u), bry_lim = (float)(H - 1u);
    const int cw = f->wind_clockwise != 0;
    uint64_t n_front = 0, n_tested = 0, n_inside = 0, n_pass = 0;

    /* drawing.cpp:236 and 241-247: normals to camera space, vertices to raster space. */
    v4* rv = (v4*)malloc((size_t)(f->nv > 0 ? f->nv : 1) * sizeof(v4));
    v3* cn = (v3*)malloc((size_t)(f->nn > 0 ? f->nn : 1) * sizeof(v3));
    if (!rv || !cn) { free(rv); free(cn); return -1; }
    for (int64_t i = 0; i < f->nv; ++i) rv[i] = raster_vertex(f->camera, f->pos + 3 * i, wf, hf);
    for (int64_t i = 0; i < f->nn; ++i) cn[i] = camera_normal(f->normal_matrix, f->nrm + 3 * i);

    /* drawing.cpp:250-257: faces in order. */
    for (int64_t t = 0; t < f->ntri; ++t) {
        const int32_t* tri = f->tris + 10 * t;
        /* drawing.cpp:165-173: de-index */
        v4 v0 = rv[tri[0]], v1 = rv[tri[1]], v2 = rv[tri[2]];
        v3 n0, n1, n2;
        if (f->flat) {
            const float* p0 = f->pos + 3 * tri[0];
            const float* p1 = f->pos + 3 * tri[1];
            const float* p2 = f->pos + 3 * tri[2];
            const float a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            const float b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
            /* glm::cross(a, b) */
            const float fn[3] = {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
            n0 = n1 = n2 = camera_normal(f->normal_matrix, fn);
        } else {
            n0 = cn[tri[3]];
            n1 = cn[tri[4]];
            n2 = cn[tri[5]];
        }
        const float* kd = f->kd + 3 * tri[9];
        v3 albedo = {kd[0], kd[1], kd[2]};
        v3 c0 = {0, 0, 0}, c1 = {0, 0, 0}, c2 = {0, 0, 0};
        /* drawing.cpp:166-170: a face's uvs, (0, 0) where the index is < 0 */
        const int textured = !f->vcol && f->tex && f->tex_off && f->tex_off[tri[9]] >= 0;
        float uvx[3] = {0.f, 0.f, 0.f}, uvy[3] = {0.f, 0.f, 0.f};
        if (textured)
            for (int k = 0; k < 3; ++k)
                if (tri[6 + k] >= 0) {
                    uvx[k] = f->uv[2 * tri[6 + k]];
                    uvy[k] = f->uv[2 * tri[6 + k] + 1];
                }
        if (f->vcol) {
            const float* a = f->vcol + 3 * tri[0];
            const float* b = f->vcol + 3 * tri[1];
            const float* c = f->vcol + 3 * tri[2];
            c0 = (v3){a[0], a[1], a[2]};
            c1 = (v3){b[0], b[1], b[2]};
            c2 = (v3){c[0], c[1], c[2]};
        }

        /* geometry.cpp:76-83 signed_area_2d, drawing.cpp:176-178 culling */
        float sa = -0.5f * (v0.x * v1.y - v1.x * v0.y + v1.x * v2.y - v2.x * v1.y + v2.x * v0.y - v0.x * v2.y);
        int front = (sa > 0) != cw;
        if (!front) continue;
        ++n_front;

        /* drawing.cpp:77-93 bounding_box */
        float mnx = gmin(gmin(v0.x, v1.x), v2.x), mny = gmin(gmin(v0.y, v1.y), v2.y);
        float mxx = gmax(gmax(v0.x, v1.x), v2.x), mxy = gmax(gmax(v0.y, v1.y), v2.y);
        uint32_t tlx = (uint32_t)gmin(gmax(mnx, 0.f), brx_lim);
        uint32_t tly = (uint32_t)gmin(gmax(mny, 0.f), bry_lim);
        uint32_t brx = (uint32_t)gmin(gmax(ceilf(mxx), 0.f), brx_lim);
        uint32_t bry = (uint32_t)gmin(gmax(ceilf(mxy), 0.f), bry_lim);

        /* drawing.cpp:191-201 and update_pixel 96-149 */
        for (uint32_t y = tly; y <= bry; ++y) {
            for (uint32_t x = tlx; x <= brx; ++x) {
                ++n_tested;
                const float px = (float)x, py = (float)y;
                /* drawing.cpp:36-49 edge / barycentric */
                float area = (v1.x - v0.x) * (v2.y - v0.y) - (v1.y - v0.y) * (v2.x - v0.x);
                float b0 = ((v2.x - v1.x) * (py - v1.y) - (v2.y - v1.y) * (px - v1.x)) / area;
                float b1 = ((v0.x - v2.x) * (py - v2.y) - (v0.y - v2.y) * (px - v2.x)) / area;
                float b2 = ((v1.x - v0.x) * (py - v0.y) - (v1.y - v0.y) * (px - v0.x)) / area;
                if (!(b0 >= 0.f && b1 >= 0.f && b2 >= 0.f)) continue;
                ++n_inside;
                /* drawing.cpp:115-121 depth test */
                float z = v0.z * b0 + v1.z * b1 + v2.z * b2;
                const size_t p = (size_t)x + (size_t)y * W;
                if (!(z < depth[p])) continue;
                ++n_pass;
                depth[p] = z;
                /* drawing.cpp:125-132 perspective-correct normal */
                float i0 = v0.w * b0, i1 = v1.w * b1, i2 = v2.w * b2;
                float dd = 1.f / (i0 + i1 + i2);
                v3 s;
                s.x = i0 * n0.x + i1 * n1.x + i2 * n2.x;
                s.y = i0 * n0.y + i1 * n1.y + i2 * n2.y;
                s.z = i0 * n0.z + i1 * n1.z + i2 * n2.z;
                s.x = dd * s.x;
                s.y = dd * s.y;
                s.z = dd * s.z;
                float inv = 1.0f / sqrtf((s.x * s.x + s.y * s.y) + s.z * s.z);
                v3 nrm = {s.x * inv, s.y * inv, s.z * inv};
                if (cw) { nrm.x = -nrm.x; nrm.y = -nrm.y; nrm.z = -nrm.z; }
                if (f->vcol) {  /* per-vertex albedo, interpolated as the normal is */
                    v3 u;
                    u.x = i0 * c0.x + i1 * c1.x + i2 * c2.x;
                    u.y = i0 * c0.y + i1 * c1.y + i2 * c2.y;
                    u.z = i0 * c0.z + i1 * c1.z + i2 * c2.z;
                    albedo.x = dd * u.x;
                    albedo.y = dd * u.y;
                    albedo.z = dd * u.z;
                }
                if (textured) {  /* drawing.cpp:135, material.cpp:18-21 */
                    const float ux = dd * (i0 * uvx[0] + i1 * uvx[1] + i2 * uvx[2]);
                    const float uy = dd * (i0 * uvy[0] + i1 * uvy[1] + i2 * uvy[2]);
                    const int tw = f->tex_wh[2 * tri[9]], th = f->tex_wh[2 * tri[9] + 1];
                    const float* img = f->tex + f->tex_off[tri[9]];
                    const float u = ux * (float)tw, v = (1.f - uy) * (float)th;
                    albedo.x = cimg_linear_xy(img, tw, th, 0, u, v);
                    albedo.y = cimg_linear_xy(img, tw, th, 1, u, v);
                    albedo.z = cimg_linear_xy(img, tw, th, 2, u, v);
                }
                /* drawing.cpp:138-146 shade and write planar RGB */
                uint32_t rgb[3];
                shade(nrm, albedo, f->lights, f->nl, rgb);
                frame[p] = (uint8_t)rgb[0];
                frame[p + plane] = (uint8_t)rgb[1];
                frame[p + 2 * plane] = (uint8_t)rgb[2];
                if (tri_id) tri_id[p] = (uint32_t)t;
            }
        }
    }
    free(rv);
    free(cn);
    if (stats) {
        stats[0] = n_front;
        stats[1] = n_tested;
        stats[2] = n_inside;
        stats[3] = n_pass;
    }
    return 0;
}
