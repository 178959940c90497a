// A subset of the OpenGL Mathematics (glm 0.9.7.6) API: exactly the types and functions that the
// rasteriser's geometry, drawing and shading code calls (geometry.cpp, drawing.cpp, shading.cpp,
// material.cpp of canmom/rasteriser). It lets code written against glm build on hosts where glm
// is not installed. Deployments that have glm may use it instead; nothing here depends on being
// this header rather than glm itself.
//
// Floating-point operation order is fixed here and documented per function. The CUDA kernels of
// this project follow the same order, and the host build uses -ffp-contract=off, so a result
// computed here and on the GPU agrees bit for bit. Where glm 0.9.7's own order is known it is the
// one used; glm is not present on this machine, so the agreement with glm itself is a stated
// belief, not a measured fact:
//   - mat4 * vec4 sums the four column products pairwise: (c0*x + c1*y) + (c2*z + c3*w);
//   - mat4 * mat4 sums left to right per column: ((a0*b.x + a1*b.y) + a2*b.z) + a3*b.w;
//   - dot(a, b) sums left to right: (a.x*b.x + a.y*b.y) + a.z*b.z;
//   - normalize(v) = v * (1 / sqrt(dot(v, v)));
//   - min(x, y) = x < y ? x : y and max(x, y) = x > y ? x : y (this decides NaN and -0 cases);
//   - clamp(x, lo, hi) = min(max(x, lo), hi).
#ifndef RAST_GLM_SUBSET_CORE_HPP
#define RAST_GLM_SUBSET_CORE_HPP

#include <cmath>
#include <cstddef>

namespace glm {

// ---------------------------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------------------------
template <typename T>
struct tvec2 {
    union { T x, r, s; };
    union { T y, g, t; };

    tvec2() : x(0), y(0) {}
    explicit tvec2(T v) : x(v), y(v) {}
    template <typename A, typename B>
    tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    template <typename U>
    explicit tvec2(const tvec2<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}

    T& operator[](std::size_t i) { return i == 0 ? x : y; }
    const T& operator[](std::size_t i) const { return i == 0 ? x : y; }
};

template <typename T>
struct tvec3 {
    union { T x, r, s; };
    union { T y, g, t; };
    union { T z, b, p; };

    tvec3() : x(0), y(0), z(0) {}
    explicit tvec3(T v) : x(v), y(v), z(v) {}
    template <typename A, typename B, typename C>
    tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U>
    explicit tvec3(const tvec3<U>& v)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}

    T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T>
struct tvec4 {
    union { T x, r, s; };
    union { T y, g, t; };
    union { T z, b, p; };
    union { T w, a, q; };

    tvec4() : x(0), y(0), z(0), w(0) {}
    explicit tvec4(T v) : x(v), y(v), z(v), w(v) {}
    template <typename A, typename B, typename C, typename D>
    tvec4(A a_, B b_, C c_, D d_)
        : x(static_cast<T>(a_)), y(static_cast<T>(b_)), z(static_cast<T>(c_)), w(static_cast<T>(d_)) {}
    template <typename U>
    explicit tvec4(const tvec4<U>& v)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(v.w)) {}

    T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

typedef tvec2<float> vec2;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;
typedef tvec2<int> ivec2;
typedef tvec3<int> ivec3;
typedef tvec2<unsigned int> uvec2;
typedef tvec3<unsigned int> uvec3;
typedef tvec4<unsigned int> uvec4;
typedef tvec2<bool> bvec2;
typedef tvec3<bool> bvec3;
typedef tvec4<bool> bvec4;

// Component-wise arithmetic. Each component is one IEEE operation; there is no reassociation.
#define RAST_GLM_VEC_BINOP(OP)                                                                    \
    template <typename T> inline tvec2<T> operator OP(const tvec2<T>& a, const tvec2<T>& b) {    \
        return tvec2<T>(a.x OP b.x, a.y OP b.y); }                                                 \
    template <typename T> inline tvec3<T> operator OP(const tvec3<T>& a, const tvec3<T>& b) {    \
        return tvec3<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z); }                                     \
    template <typename T> inline tvec4<T> operator OP(const tvec4<T>& a, const tvec4<T>& b) {    \
        return tvec4<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }                         \
    template <typename T> inline tvec2<T> operator OP(const tvec2<T>& a, T s) {                   \
        return tvec2<T>(a.x OP s, a.y OP s); }                                                     \
    template <typename T> inline tvec3<T> operator OP(const tvec3<T>& a, T s) {                   \
        return tvec3<T>(a.x OP s, a.y OP s, a.z OP s); }                                           \
    template <typename T> inline tvec4<T> operator OP(const tvec4<T>& a, T s) {                   \
        return tvec4<T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }                                 \
    template <typename T> inline tvec2<T> operator OP(T s, const tvec2<T>& a) {                   \
        return tvec2<T>(s OP a.x, s OP a.y); }                                                     \
    template <typename T> inline tvec3<T> operator OP(T s, const tvec3<T>& a) {                   \
        return tvec3<T>(s OP a.x, s OP a.y, s OP a.z); }                                           \
    template <typename T> inline tvec4<T> operator OP(T s, const tvec4<T>& a) {                   \
        return tvec4<T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }

RAST_GLM_VEC_BINOP(+)
RAST_GLM_VEC_BINOP(-)
RAST_GLM_VEC_BINOP(*)
RAST_GLM_VEC_BINOP(/)
#undef RAST_GLM_VEC_BINOP

template <typename T> inline tvec2<T> operator-(const tvec2<T>& a) { return tvec2<T>(-a.x, -a.y); }
template <typename T> inline tvec3<T> operator-(const tvec3<T>& a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <typename T> inline tvec4<T> operator-(const tvec4<T>& a) { return tvec4<T>(-a.x, -a.y, -a.z, -a.w); }

template <typename T> inline tvec2<T>& operator+=(tvec2<T>& a, const tvec2<T>& b) { a = a + b; return a; }
template <typename T> inline tvec3<T>& operator+=(tvec3<T>& a, const tvec3<T>& b) { a = a + b; return a; }
template <typename T> inline tvec4<T>& operator+=(tvec4<T>& a, const tvec4<T>& b) { a = a + b; return a; }

template <typename T> inline bool operator==(const tvec2<T>& a, const tvec2<T>& b) { return a.x == b.x && a.y == b.y; }
template <typename T> inline bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <typename T> inline bool operator==(const tvec4<T>& a, const tvec4<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

// ---------------------------------------------------------------------------------------------
// scalar and component-wise common functions
// ---------------------------------------------------------------------------------------------
template <typename T> inline T min(T x, T y) { return x < y ? x : y; }
template <typename T> inline T max(T x, T y) { return x > y ? x : y; }
template <typename T> inline T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }

template <typename T> inline tvec2<T> min(const tvec2<T>& a, const tvec2<T>& b) {
    return tvec2<T>(min(a.x, b.x), min(a.y, b.y)); }
template <typename T> inline tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) {
    return tvec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <typename T> inline tvec2<T> max(const tvec2<T>& a, const tvec2<T>& b) {
    return tvec2<T>(max(a.x, b.x), max(a.y, b.y)); }
template <typename T> inline tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) {
    return tvec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
template <typename T> inline tvec2<T> clamp(const tvec2<T>& v, const tvec2<T>& lo, const tvec2<T>& hi) {
    return min(max(v, lo), hi); }
template <typename T> inline tvec3<T> clamp(const tvec3<T>& v, const tvec3<T>& lo, const tvec3<T>& hi) {
    return min(max(v, lo), hi); }

inline vec2 ceil(const vec2& v) { return vec2(std::ceil(v.x), std::ceil(v.y)); }
inline vec3 ceil(const vec3& v) { return vec3(std::ceil(v.x), std::ceil(v.y), std::ceil(v.z)); }

template <typename T> inline bvec2 greaterThanEqual(const tvec2<T>& a, const tvec2<T>& b) {
    return bvec2(a.x >= b.x, a.y >= b.y); }
template <typename T> inline bvec3 greaterThanEqual(const tvec3<T>& a, const tvec3<T>& b) {
    return bvec3(a.x >= b.x, a.y >= b.y, a.z >= b.z); }
inline bool all(const bvec2& v) { return v.x && v.y; }
inline bool all(const bvec3& v) { return v.x && v.y && v.z; }
inline bool all(const bvec4& v) { return v.x && v.y && v.z && v.w; }

// ---------------------------------------------------------------------------------------------
// geometric functions
// ---------------------------------------------------------------------------------------------
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline float inversesqrt(float v) { return 1.0f / std::sqrt(v); }
inline vec2 normalize(const vec2& v) { return v * inversesqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
inline vec4 normalize(const vec4& v) { return v * inversesqrt(dot(v, v)); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }

template <typename T> inline T radians(T degrees) {
    return degrees * static_cast<T>(0.01745329251994329576923690768489); }
template <typename T> inline T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }
template <typename T> inline T one_over_pi() { return static_cast<T>(0.318309886183790671537767526745028724); }

// ---------------------------------------------------------------------------------------------
// 4x4 matrix, column major: m[c] is column c and m[c][r] the entry in row r.
// ---------------------------------------------------------------------------------------------
struct mat4 {
    vec4 col[4];

    mat4() { *this = mat4(1.0f); }
    explicit mat4(float d) {
        col[0] = vec4(d, 0.0f, 0.0f, 0.0f);
        col[1] = vec4(0.0f, d, 0.0f, 0.0f);
        col[2] = vec4(0.0f, 0.0f, d, 0.0f);
        col[3] = vec4(0.0f, 0.0f, 0.0f, d);
    }
    mat4(const vec4& c0, const vec4& c1, const vec4& c2, const vec4& c3) {
        col[0] = c0; col[1] = c1; col[2] = c2; col[3] = c3;
    }
    vec4& operator[](std::size_t c) { return col[c]; }
    const vec4& operator[](std::size_t c) const { return col[c]; }
};

typedef mat4 mat4x4;

inline vec4 operator*(const mat4& m, const vec4& v) {
    const vec4 lo = m[0] * v.x + m[1] * v.y;
    const vec4 hi = m[2] * v.z + m[3] * v.w;
    return lo + hi;
}

inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 out(0.0f);
    for (int c = 0; c < 4; ++c)
        out[c] = ((a[0] * b[c].x + a[1] * b[c].y) + a[2] * b[c].z) + a[3] * b[c].w;
    return out;
}

inline mat4 transpose(const mat4& m) {
    mat4 out(0.0f);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c][r] = m[r][c];
    return out;
}

// Inverse through the adjugate. The twelve 2x2 minors of the top two rows (s*) and of the bottom
// two rows (c*) give every 3x3 cofactor; the determinant is the Laplace expansion over them.
inline mat4 inverse(const mat4& m) {
    // a_rc: entry in row r, column c.
    const float a00 = m[0][0], a01 = m[1][0], a02 = m[2][0], a03 = m[3][0];
    const float a10 = m[0][1], a11 = m[1][1], a12 = m[2][1], a13 = m[3][1];
    const float a20 = m[0][2], a21 = m[1][2], a22 = m[2][2], a23 = m[3][2];
    const float a30 = m[0][3], a31 = m[1][3], a32 = m[2][3], a33 = m[3][3];

    const float s0 = a00 * a11 - a10 * a01;
    const float s1 = a00 * a12 - a10 * a02;
    const float s2 = a00 * a13 - a10 * a03;
    const float s3 = a01 * a12 - a11 * a02;
    const float s4 = a01 * a13 - a11 * a03;
    const float s5 = a02 * a13 - a12 * a03;

    const float c5 = a22 * a33 - a32 * a23;
    const float c4 = a21 * a33 - a31 * a23;
    const float c3 = a21 * a32 - a31 * a22;
    const float c2 = a20 * a33 - a30 * a23;
    const float c1 = a20 * a32 - a30 * a22;
    const float c0 = a20 * a31 - a30 * a21;

    const float det = (s0 * c5 - s1 * c4 + s2 * c3) + (s3 * c2 - s4 * c1 + s5 * c0);
    const float inv = 1.0f / det;

    // b_rc of the inverse, written into column c, row r.
    mat4 out(0.0f);
    out[0][0] = ( a11 * c5 - a12 * c4 + a13 * c3) * inv;
    out[1][0] = (-a01 * c5 + a02 * c4 - a03 * c3) * inv;
    out[2][0] = ( a31 * s5 - a32 * s4 + a33 * s3) * inv;
    out[3][0] = (-a21 * s5 + a22 * s4 - a23 * s3) * inv;

    out[0][1] = (-a10 * c5 + a12 * c2 - a13 * c1) * inv;
    out[1][1] = ( a00 * c5 - a02 * c2 + a03 * c1) * inv;
    out[2][1] = (-a30 * s5 + a32 * s2 - a33 * s1) * inv;
    out[3][1] = ( a20 * s5 - a22 * s2 + a23 * s1) * inv;

    out[0][2] = ( a10 * c4 - a11 * c2 + a13 * c0) * inv;
    out[1][2] = (-a00 * c4 + a01 * c2 - a03 * c0) * inv;
    out[2][2] = ( a30 * s4 - a31 * s2 + a33 * s0) * inv;
    out[3][2] = (-a20 * s4 + a21 * s2 - a23 * s0) * inv;

    out[0][3] = (-a10 * c3 + a11 * c1 - a12 * c0) * inv;
    out[1][3] = ( a00 * c3 - a01 * c1 + a02 * c0) * inv;
    out[2][3] = (-a30 * s3 + a31 * s1 - a32 * s0) * inv;
    out[3][3] = ( a20 * s3 - a21 * s1 + a22 * s0) * inv;
    return out;
}

// ---------------------------------------------------------------------------------------------
// transform builders (gtc/matrix_transform)
// ---------------------------------------------------------------------------------------------
inline mat4 translate(const mat4& m, const vec3& d) {
    mat4 out = m;
    out[3] = ((m[0] * d.x + m[1] * d.y) + m[2] * d.z) + m[3];
    return out;
}

inline mat4 scale(const mat4& m, const vec3& f) {
    return mat4(m[0] * f.x, m[1] * f.y, m[2] * f.z, m[3]);
}

// Rotation by `angle` radians about `axis` (Rodrigues' formula), post-multiplied onto m.
inline mat4 rotate(const mat4& m, float angle, const vec3& axis_in) {
    const float c = std::cos(angle);
    const float s = std::sin(angle);
    const vec3 k = normalize(axis_in);
    const vec3 t = (1.0f - c) * k;

    // R[j] is column j of the rotation.
    vec3 R[3];
    R[0] = vec3(c + t.x * k.x, t.x * k.y + s * k.z, t.x * k.z - s * k.y);
    R[1] = vec3(t.y * k.x - s * k.z, c + t.y * k.y, t.y * k.z + s * k.x);
    R[2] = vec3(t.z * k.x + s * k.y, t.z * k.y - s * k.x, c + t.z * k.z);

    mat4 out(0.0f);
    for (int j = 0; j < 3; ++j)
        out[j] = (m[0] * R[j].x + m[1] * R[j].y) + m[2] * R[j].z;
    out[3] = m[3];
    return out;
}

// OpenGL right-handed perspective projection with clip depth in [-1, 1].
inline mat4 perspective(float fovy, float aspect, float z_near, float z_far) {
    const float th = std::tan(fovy / 2.0f);
    mat4 out(0.0f);
    out[0][0] = 1.0f / (aspect * th);
    out[1][1] = 1.0f / th;
    out[2][2] = -(z_far + z_near) / (z_far - z_near);
    out[2][3] = -1.0f;
    out[3][2] = -(2.0f * z_far * z_near) / (z_far - z_near);
    return out;
}

}  // namespace glm

#endif  // RAST_GLM_SUBSET_CORE_HPP
