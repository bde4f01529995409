// GLSL's built-in types and functions in C++, for compiling the reference's
// own shader functions on the host. TEST INFRASTRUCTURE ONLY: the recipe
// oracle/build_glsl_ref.py puts this header in front of shader text taken
// from the reference tree (never copied into this repository) and builds
// oracle/_ref/libglsl_ref.so; tests/test_oracle_glsl_ref.py compares what
// those shader functions compute with the oracle.
//
// GLSL semantics kept here: int -> float and ivec -> vec convert implicitly,
// vec -> ivec only by constructor (truncation); vector operators act per
// component; min / max / clamp accept mixed int and float arguments as GLSL's
// implicit conversions do; `==` on vectors compares all components.
// The built-in functions follow the oracle's conventions (the shaders leave
// their precision to the driver): IEEE binary32 without contraction, sums
// left to right, normalize(x) = x * (1 / length(x)), mat4 * vec4 summed
// column by column, exp / exp2 / log2 / pow / sin / cos from omath.h.
// R8 textures and images hold unsigned normalised bytes: a fetch returns
// v / 255, a store rounds x * 255 to the nearest byte after clamping to [0, 1].
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "omath.h"

namespace glsl {

struct vec3;
struct vec4;
struct ivec3;

struct vec2 {
    float x = 0.0f, y = 0.0f;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(const vec3& v);
    explicit vec2(const vec4& v);
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
    vec2 xy() const { return *this; }
};

struct vec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
    explicit vec3(const vec4& v);
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec2 xy() const { return vec2(x, y); }
    vec3 xyz() const { return *this; }
};

struct vec4 {
    float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    vec2 xy() const { return vec2(x, y); }
    vec3 xyz() const { return vec3(x, y, z); }
    vec4 xyzw() const { return *this; }
};

inline vec2::vec2(const vec3& v) : x(v.x), y(v.y) {}
inline vec2::vec2(const vec4& v) : x(v.x), y(v.y) {}
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct uvec3 {
    unsigned x = 0, y = 0, z = 0;
    uvec3 xyz() const { return *this; }
};

struct ivec3 {
    int x = 0, y = 0, z = 0;
    ivec3() = default;
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
    explicit ivec3(const uvec3& u) : x((int)u.x), y((int)u.y), z((int)u.z) {}
    int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    operator vec3() const { return vec3((float)x, (float)y, (float)z); }   // GLSL's implicit int -> float
    ivec3 xyz() const { return *this; }
};


struct ivec2 {
    int x = 0, y = 0;
    ivec2() = default;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
    explicit ivec2(float f) : x((int)f), y((int)f) {}
    int& operator[](int i) { return i == 0 ? x : y; }
    int operator[](int i) const { return i == 0 ? x : y; }
    operator vec2() const { return vec2((float)x, (float)y); }   // GLSL's implicit int -> float
    ivec2 xy() const { return *this; }
};
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator%(const ivec2& a, const ivec2& b) { return ivec2(a.x % b.x, a.y % b.y); }

// mat3: three columns, m * v summed column by column
struct mat3 {
    vec3 c[3];
    mat3(const vec3& a, const vec3& b, const vec3& d) : c{a, b, d} {}
};
inline vec3 operator*(const mat3& m, const vec3& v) {
    vec3 r;
    for (int i = 0; i < 3; i++) r[i] = (m.c[0][i] * v.x + m.c[1][i] * v.y) + m.c[2][i] * v.z;
    return r;
}

// mat4: four columns; m[c] is column c, m * v sums the columns left to right
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; i++) r[i] = ((m.c[0][i] * v.x + m.c[1][i] * v.y) + m.c[2][i] * v.z) + m.c[3][i] * v.w;
    return r;
}
// a * b: column c of the product is a * (column c of b)
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int c = 0; c < 4; c++) r.c[c] = a * b.c[c];
    return r;
}

// ---- float vector operators (component-wise) ----
#define GLSL_VEC_OPS(V, N)                                                                         \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + b[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - b[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * b[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / b[i]; return r; } \
    inline V operator+(const V& a, float s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + s; return r; }       \
    inline V operator-(const V& a, float s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - s; return r; }       \
    inline V operator*(const V& a, float s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * s; return r; }       \
    inline V operator/(const V& a, float s) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / s; return r; }       \
    inline V operator+(float s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s + a[i]; return r; }       \
    inline V operator-(float s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s - a[i]; return r; }       \
    inline V operator*(float s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s * a[i]; return r; }       \
    inline V operator/(float s, const V& a) { V r; for (int i = 0; i < N; i++) r[i] = s / a[i]; return r; }       \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = -a[i]; return r; }                    \
    inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                                               \
    inline V& operator-=(V& a, const V& b) { a = a - b; return a; }                                               \
    inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                                               \
    inline V& operator*=(V& a, float s) { a = a * s; return a; }                                                  \
    inline V& operator/=(V& a, float s) { a = a / s; return a; }                                                  \
    inline bool operator==(const V& a, const V& b) { for (int i = 0; i < N; i++) if (!(a[i] == b[i])) return false; return true; } \
    inline bool operator!=(const V& a, const V& b) { return !(a == b); }
GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)
#undef GLSL_VEC_OPS

// ---- integer vector operators ----
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline ivec3 operator+(int s, const ivec3& a) { return ivec3(s + a.x, s + a.y, s + a.z); }
inline ivec3 operator+(const ivec3& a, int s) { return ivec3(a.x + s, a.y + s, a.z + s); }
inline ivec3 operator-(int s, const ivec3& a) { return ivec3(s - a.x, s - a.y, s - a.z); }
inline ivec3 operator-(const ivec3& a, int s) { return ivec3(a.x - s, a.y - s, a.z - s); }
inline ivec3 operator>>(const ivec3& a, int s) { return ivec3(a.x >> s, a.y >> s, a.z >> s); }
inline ivec3 operator<<(const ivec3& a, int s) { return ivec3(a.x << s, a.y << s, a.z << s); }
inline ivec3 operator-(const ivec3& a) { return ivec3(-a.x, -a.y, -a.z); }
inline bool operator==(const ivec3& a, const ivec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// ---- scalar built-ins (GLSL names; mixed int / float as GLSL converts them) ----
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float min(int a, float b) { return min((float)a, b); }
inline float min(float a, int b) { return min(a, (float)b); }
inline float max(int a, float b) { return max((float)a, b); }
inline float max(float a, int b) { return max(a, (float)b); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float clamp(int x, float lo, float hi) { return clamp((float)x, lo, hi); }
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float floor(float x) { return std::floor(x); }
inline float fract(float x) { return x - std::floor(x); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float exp(float x) { return vpto::dm_exp(x); }
inline float exp2(float x) { return vpto::dm_exp2(x); }
inline float log2(float x) { return vpto::dm_log2(x); }
inline float pow(float x, float y) { return vpto::dm_pow(x, y); }
inline float sin(float x) { return vpto::dm_sin(x); }
inline float cos(float x) { return vpto::dm_cos(x); }
inline float tan(float x) { return vpto::dm_sin(x) / vpto::dm_cos(x); }
inline float radians(float d) { return d * 0.01745329251994329577f; }
inline float rcp(float x) { return 1.0f / x; }   // accepted by the reference's GLSL compiler; 1 / x
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline float mod(float x, float y) { return x - y * floor(x / y); }

// ---- vector built-ins ----
inline vec3 floor(const vec3& v) { return vec3(floor(v.x), floor(v.y), floor(v.z)); }
inline vec2 floor(const vec2& v) { return vec2(floor(v.x), floor(v.y)); }
inline float round(float x) { return std::nearbyint(x); }
inline vec3 sign(const vec3& v) { return vec3(sign(v.x), sign(v.y), sign(v.z)); }
inline vec3 abs(const vec3& v) { return vec3(abs(v.x), abs(v.y), abs(v.z)); }
inline vec2 fract(const vec2& v) { return vec2(fract(v.x), fract(v.y)); }
inline vec2 clamp(const vec2& v, float lo, float hi) { return vec2(clamp(v.x, lo, hi), clamp(v.y, lo, hi)); }
inline vec3 clamp(const vec3& v, float lo, float hi) {
    return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi));
}
inline vec2 mix(const vec2& a, const vec2& b, float t) { return vec2(mix(a.x, b.x, t), mix(a.y, b.y, t)); }
inline vec4 mix(const vec4& a, const vec4& b, float t) {
    return vec4(mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t), mix(a.w, b.w, t));
}
inline vec4 clamp(const vec4& v, float lo, float hi) {
    return vec4(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi), clamp(v.w, lo, hi));
}
inline vec2 sin(const vec2& v) { return vec2(sin(v.x), sin(v.y)); }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float length(const vec2& a) { return sqrt(dot(a, a)); }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& a) { return sqrt(dot(a, a)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3 normalize(const vec3& a) { return a * (1.0f / length(a)); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// A function's `float[6]` return value (GLSL returns arrays by value).
struct arr_float_6 {
    float v[6];
    arr_float_6(const float* p) { for (int i = 0; i < 6; i++) v[i] = p[i]; }   // NOLINT: GLSL's array copy
    float operator[](int i) const { return v[i]; }
};
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

// ---- textures and images (unsigned normalised bytes, x fastest) ----
struct sampler3D {
    const uint8_t* data = nullptr;
    int X = 0, Y = 0, Z = 0;
};
inline vec4 texelFetch(const sampler3D& s, const ivec3& p, int lod) {
    (void)lod;
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= s.X || p.y >= s.Y || p.z >= s.Z) std::abort();
    const uint8_t v = s.data[((size_t)p.z * s.Y + p.y) * s.X + p.x];
    return vec4((float)v / 255.0f, 0.0f, 0.0f, 1.0f);
}
// Float 2-D texture of C interleaved channels (a G-buffer or filter plane),
// rows from the bottom; a fetch fills (r, g, b, a) from the C channels and
// (0, 0, 0, 1) after them. texture() of a GL_NEAREST texture returns the
// texel the coordinate falls in; otherwise it follows the oracle's sampling
// convention: at a texel centre (the texel-space coordinate within 2^-9 of an
// integer, what the hardware's fixed-point addressing snaps) it returns that
// texel, elsewhere it blends the four texels with fp32 weights, REPEAT wrap.
struct sampler2D {
    const float* data = nullptr;
    int W = 0, H = 0, C = 1;
    bool nearest = false;   // GL_NEAREST (the G-buffer's face and block planes)
    bool snap = true;       // texel centres return the texel (off: always the fp32 blend)
};
inline float texel2d(const sampler2D& s, int i, int j, int c) {
    i %= s.W; if (i < 0) i += s.W;
    j %= s.H; if (j < 0) j += s.H;
    return s.data[((size_t)j * s.W + i) * s.C + c];
}
inline vec4 texel_vec(const sampler2D& s, int i, int j) {
    vec4 r(0.0f, 0.0f, 0.0f, 1.0f);
    for (int c = 0; c < s.C && c < 4; c++) r[c] = texel2d(s, i, j, c);
    return r;
}
inline vec4 texture(const sampler2D& s, const vec2& uv) {
    if (s.nearest) return texel_vec(s, (int)std::floor(uv.x * (float)s.W), (int)std::floor(uv.y * (float)s.H));
    const float x = uv.x * (float)s.W - 0.5f, y = uv.y * (float)s.H - 0.5f;
    const float rx = std::nearbyint(x), ry = std::nearbyint(y);
    if (s.snap && std::fabs(x - rx) < 0.001953125f && std::fabs(y - ry) < 0.001953125f)
        return texel_vec(s, (int)rx, (int)ry);
    const float x0 = std::floor(x), y0 = std::floor(y), ax = x - x0, ay = y - y0;
    const int i0 = (int)x0, j0 = (int)y0;
    vec4 r(0.0f, 0.0f, 0.0f, 1.0f);
    for (int c = 0; c < s.C && c < 4; c++) {
        const float lo = texel2d(s, i0, j0, c) * (1.0f - ax) + texel2d(s, i0 + 1, j0, c) * ax;
        const float hi = texel2d(s, i0, j0 + 1, c) * (1.0f - ax) + texel2d(s, i0 + 1, j0 + 1, c) * ax;
        r[c] = lo * (1.0f - ay) + hi * ay;
    }
    return r;
}
inline vec4 texelFetch(const sampler2D& s, const ivec2& p, int lod) {
    (void)lod;
    if (p.x < 0 || p.y < 0 || p.x >= s.W || p.y >= s.H) std::abort();
    return texel_vec(s, p.x, p.y);
}
inline ivec2 textureSize(const sampler2D& s, int lod) { (void)lod; return ivec2(s.W, s.H); }

struct image3D {
    uint8_t* data = nullptr;
    int X = 0, Y = 0, Z = 0;
};
inline vec4 imageLoad(const image3D& im, const ivec3& p) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.X || p.y >= im.Y || p.z >= im.Z) std::abort();
    const uint8_t v = im.data[((size_t)p.z * im.Y + p.y) * im.X + p.x];
    return vec4((float)v / 255.0f, 0.0f, 0.0f, 1.0f);
}
inline void imageStore(image3D& im, const ivec3& p, const vec4& v) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.X || p.y >= im.Y || p.z >= im.Z) std::abort();
    const float c = clamp(v.x, 0.0f, 1.0f) * 255.0f;
    im.data[((size_t)p.z * im.Y + p.y) * im.X + p.x] = (uint8_t)std::nearbyint(c);
}

}  // namespace glsl
