// Oracle math: vector helpers, deterministic transcendental functions and the
// OpenGL texture-sampling rules the reference shaders rely on.
//
// TEST INFRASTRUCTURE ONLY. This header belongs to the CPU oracle that the
// parity tests, the smoke check and the CPU-baseline leg of bench.py use to
// check the CUDA path. The product never includes or links it.
//
// Every operation here is a single IEEE-754 binary32 operation or a fixed
// sequence of them. The oracle is compiled with -ffp-contract=off and without
// fast-math, so no multiply-add is fused implicitly; the polynomial steps of
// the functions below call fmaf explicitly, which is a single correctly
// rounded operation on every IEEE host (x86-64 and aarch64 alike).
//
// Transcendental functions: GLSL leaves exp/pow/sin/cos precision to the
// driver, so the oracle defines its own. They are written from the textbook
// method, not from any vendor library:
//   * exp / exp2: Cody-Waite argument reduction x = k*ln2 + r (|r| <= ln2/2),
//     Taylor series of e^r to degree 8 in Horner form, then scaling by 2^k in
//     two exact power-of-two multiplies (so a subnormal result is rounded once);
//   * log2: x = 2^e * m with m in [sqrt(1/2), sqrt(2)), ln m = 2*atanh(s),
//     s = (m-1)/(m+1), odd series to s^11;
//   * sin / cos: reduction by pi/2 with a three-part Cody-Waite constant,
//     Taylor series on |r| <= pi/4 (sin to r^9, cos to r^10), quadrant table;
//   * pow(x, y): binary powering for integer y in 1..1024 (what GPU compilers
//     emit for pow(x, 2.0) and the like), else exp2(y * log2(x)), with
//     GLSL's defined cases.
// Worst-case errors are a few ulp; tests/test_oracle_math.py checks them
// against numpy float64.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

using std::fmaf;

namespace vpto {

static inline float f_from_bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline uint32_t bits_from_f(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// float -> int32 with round-toward-zero, NaN -> 0 and saturation. GLSL leaves
// int(NaN) undefined; this is the definition the build uses everywhere.
static inline int32_t f2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x < -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)x;
}

// 2^n for n in [-126, 127] as an exact float.
static inline float pow2i(int n) { return f_from_bits((uint32_t)(n + 127) << 23); }

static inline float scale2(float p, int k) {
    int k1 = k / 2;
    int k2 = k - k1;
    return (p * pow2i(k1)) * pow2i(k2);
}

static inline float dm_exp(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.97208404541016f) return 0.0f;
    float kf = std::floor(x * 1.44269502162933350f + 0.5f);
    int k = (int)kf;
    float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187e-06f;
    float p = 1.0f / 40320.0f;
    p = fmaf(p, r, 1.0f / 5040.0f);
    p = fmaf(p, r, 1.0f / 720.0f);
    p = fmaf(p, r, 1.0f / 120.0f);
    p = fmaf(p, r, 1.0f / 24.0f);
    p = fmaf(p, r, 1.0f / 6.0f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return scale2(p, k);
}

static inline float dm_exp2(float x) {
    if (x != x) return x;
    if (x >= 128.0f) return INFINITY;
    if (x < -150.0f) return 0.0f;
    float kf = std::floor(x + 0.5f);
    int k = (int)kf;
    float r = (x - kf) * 0.693147182464599609f;
    float p = 1.0f / 40320.0f;
    p = fmaf(p, r, 1.0f / 5040.0f);
    p = fmaf(p, r, 1.0f / 720.0f);
    p = fmaf(p, r, 1.0f / 120.0f);
    p = fmaf(p, r, 1.0f / 24.0f);
    p = fmaf(p, r, 1.0f / 6.0f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return scale2(p, k);
}

static inline float dm_log2(float x) {
    if (x != x) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return INFINITY;
    int e = 0;
    uint32_t u = bits_from_f(x);
    if ((u >> 23) == 0) {            // subnormal: scale into the normal range
        x = x * 8388608.0f;          // 2^23, exact
        u = bits_from_f(x);
        e = -23;
    }
    e += (int)((u >> 23) & 0xffu) - 127;
    float m = f_from_bits((u & 0x007fffffu) | 0x3f800000u);   // [1, 2)
    if (m > 1.41421353816986084f) { m = m * 0.5f; e += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = 1.0f / 11.0f;
    p = fmaf(p, s2, 1.0f / 9.0f);
    p = fmaf(p, s2, 1.0f / 7.0f);
    p = fmaf(p, s2, 1.0f / 5.0f);
    p = fmaf(p, s2, 1.0f / 3.0f);
    p = fmaf(p, s2, 1.0f);
    float ln_m = 2.0f * (s * p);
    return (float)e + ln_m * 1.44269502162933350f;
}

// GLSL pow: undefined for x < 0 (NaN here) and for x == 0, y <= 0. Integer
// exponents 1..1024 use binary powering (square-and-multiply from the lowest
// bit), the rest exp2(y * log2(x)).
static inline float dm_pow(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (x == 0.0f) return y > 0.0f ? 0.0f : INFINITY;
    if (x < 0.0f || x != x || y != y) return NAN;
    if (y >= 1.0f && y <= 1024.0f && y == std::floor(y)) {
        int n = (int)y;
        float r = 1.0f, b = x;
        for (;;) {
            if (n & 1) r = r * b;
            n >>= 1;
            if (!n) break;
            b = b * b;
        }
        return r;
    }
    return dm_exp2(y * dm_log2(x));
}

static inline float sin_poly(float r) {
    float r2 = r * r;
    float p = 1.0f / 362880.0f;
    p = fmaf(p, r2, -(1.0f / 5040.0f));
    p = fmaf(p, r2, 1.0f / 120.0f);
    p = fmaf(p, r2, -(1.0f / 6.0f));
    return fmaf(r * r2, p, r);
}

static inline float cos_poly(float r) {
    float r2 = r * r;
    float p = -1.0f / 3628800.0f;
    p = fmaf(p, r2, 1.0f / 40320.0f);
    p = fmaf(p, r2, -(1.0f / 720.0f));
    p = fmaf(p, r2, 1.0f / 24.0f);
    p = fmaf(p, r2, -(0.5f));
    return fmaf(r2, p, 1.0f);
}

static inline float reduce_pio2(float x, int* q) {
    float kf = std::floor(x * 0.636619746685028076f + 0.5f);
    *q = ((int)kf) & 3;
    return ((x - kf * 1.5703125f) - kf * 4.837512969970703e-4f) - kf * 7.549790126404332e-8f;
}

static inline float dm_sin(float x) {
    if (x != x || std::isinf(x)) return NAN;
    int q;
    float r = reduce_pio2(x, &q);
    switch (q) {
        case 0: return sin_poly(r);
        case 1: return cos_poly(r);
        case 2: return -sin_poly(r);
        default: return -cos_poly(r);
    }
}

static inline float dm_cos(float x) {
    if (x != x || std::isinf(x)) return NAN;
    int q;
    float r = reduce_pio2(x, &q);
    switch (q) {
        case 0: return cos_poly(r);
        case 1: return -sin_poly(r);
        case 2: return -cos_poly(r);
        default: return sin_poly(r);
    }
}

// ---------------------------------------------------------------- scalars --
static inline float fmaxg(float a, float b) { return std::fmax(a, b); }
static inline float fming(float a, float b) { return std::fmin(a, b); }
static inline float clampf(float x, float lo, float hi) { return fming(fmaxg(x, lo), hi); }
static inline float fract(float x) { return x - std::floor(x); }
// GLSL mix: x*(1-a) + y*a
static inline float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
static inline int isign(float x) { return x > 0.0f ? 1 : (x < 0.0f ? -1 : 0); }

// ---------------------------------------------------------------- vectors --
struct v2 { float x, y; };
struct v3 { float x, y, z; };
struct v4 { float x, y, z, w; };

static inline v3 mk3(float x, float y, float z) { return v3{x, y, z}; }
static inline v3 add(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline v3 sub(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline v3 mul(v3 a, v3 b) { return v3{a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline v3 muls(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
static inline v3 divs(v3 a, float s) { return v3{a.x / s, a.y / s, a.z / s}; }
static inline v3 neg(v3 a) { return v3{-a.x, -a.y, -a.z}; }
static inline float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float length(v3 a) { return std::sqrt(dot(a, a)); }
// GLSL normalize(x): x scaled by 1/length(x) (one division, as GPU compilers
// emit it), every operation IEEE-rounded.
static inline v3 normalize(v3 a) { return muls(a, 1.0f / length(a)); }
static inline v3 vmax(v3 a, float s) { return v3{fmaxg(a.x, s), fmaxg(a.y, s), fmaxg(a.z, s)}; }
static inline v3 vclamp(v3 a, float lo, float hi) {
    return v3{clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi)};
}
static inline v3 vmix(v3 a, v3 b, float t) {
    return v3{mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)};
}
static inline v3 vmixv(v3 a, v3 b, v3 t) {
    return v3{mixf(a.x, b.x, t.x), mixf(a.y, b.y, t.y), mixf(a.z, b.z, t.z)};
}
static inline float comp(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline void set_comp(v3* a, int i, float v) {
    if (i == 0) a->x = v; else if (i == 1) a->y = v; else a->z = v;
}

// Column-major 4x4 (m[col*4 + row]) times (x, y, z, w); sums left to right.
static inline v4 mat_mul4(const float* m, float x, float y, float z, float w) {
    v4 r;
    r.x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w;
    r.y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w;
    r.z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w;
    r.w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w;
    return r;
}

// ------------------------------------------------------------ half storage --
// binary32 -> binary16 -> binary32 with round-to-nearest-even, as a GPU half
// store would do. Used when the oracle emulates the FP16 storage variant.
static inline float half_round(float f) {
    uint32_t x = bits_from_f(f);
    uint32_t sign = x & 0x80000000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) {                       // inf / NaN
        return ax > 0x7f800000u ? f : f_from_bits(sign | 0x7f800000u);
    }
    if (ax >= 0x477ff000u) return f_from_bits(sign | 0x7f800000u);   // rounds to >= 65520 -> inf
    if (ax < 0x33000000u) return f_from_bits(sign);                    // < 2^-25 -> 0
    int exp = (int)(ax >> 23) - 127;
    uint32_t mant = (ax & 0x007fffffu) | 0x00800000u;
    // number of mantissa bits kept: 10 for normal halves, fewer for subnormals
    int keep = exp >= -14 ? 10 : 10 - (-14 - exp);
    int drop = 23 - keep;
    uint32_t rem = mant & ((1u << drop) - 1u);
    uint32_t half_ulp = 1u << (drop - 1);
    uint32_t q = mant >> drop;
    if (rem > half_ulp || (rem == half_ulp && (q & 1u))) q += 1u;
    // rebuild value = q * 2^(exp - keep)
    float v = (float)q;
    int e2 = exp - keep;
    // e2 in [-24, 5]: exact scaling
    v = e2 >= 0 ? v * (float)(1u << e2) : v / (float)(1u << (-e2));
    return sign ? -v : v;
}

}  // namespace vpto
