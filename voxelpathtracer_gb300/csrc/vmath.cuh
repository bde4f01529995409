// Device math for the VoxelPathTracer kernels.
//
// Every function is a fixed sequence of IEEE-754 binary32 operations. The
// library is compiled with -fmad=false (device) and -ffp-contract=off (host),
// with IEEE division and square root; the only fused multiply-adds are the
// explicit fmaf calls of the polynomial steps below (one correctly rounded
// operation on both sides). So the same inputs give the same bits
// on the GPU and on any host. That is what lets the traversal outputs (hit
// voxel, face, step count) and the radiance planes match the CPU restatement
// of the reference shaders bit for bit.
//
// GLSL leaves exp/pow/sin/cos precision to the driver, so these are defined
// here from the textbook methods (not from CUDA's math library):
//   exp/exp2: Cody-Waite reduction x = k*ln2 + r, |r| <= ln2/2, Taylor series
//             of e^r to degree 8 (Horner), scaling by 2^k in two exact
//             power-of-two multiplies;
//   log2:     x = 2^e * m, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s),
//             s = (m-1)/(m+1), odd series to s^11;
//   sin/cos:  reduction by pi/2 with a three-part constant, Taylor series on
//             |r| <= pi/4, quadrant selection;
//   pow:      binary powering for integer exponents 1..1024, otherwise
//             exp2(y * log2(x)), with GLSL's defined special cases.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#define VPT_HD __host__ __device__ __forceinline__

namespace vpt {

VPT_HD float f_from_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f; __builtin_memcpy(&f, &u, 4); return f;
#endif
}
VPT_HD uint32_t bits_from_f(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u; __builtin_memcpy(&u, &f, 4); return u;
#endif
}

VPT_HD bool is_nan(float x) { return x != x; }
VPT_HD float inf_f() { return f_from_bits(0x7f800000u); }
VPT_HD float nan_f() { return f_from_bits(0x7fc00000u); }

// float -> int32, round toward zero, NaN -> 0, saturating. On the device this
// is exactly the cvt.rzi.s32.f32 conversion (PTX float-to-integer conversions
// saturate and map NaN to 0), on the host it is spelled out.
VPT_HD int32_t f2i(float x) {
#ifdef __CUDA_ARCH__
    return __float2int_rz(x);
#else
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x < -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)x;
#endif
}
// f2i(floor(x)) in one conversion (round toward minus infinity).
VPT_HD int32_t f2i_floor(float x) {
#ifdef __CUDA_ARCH__
    return __float2int_rd(x);
#else
    return f2i(floorf(x));
#endif
}

VPT_HD float pow2i(int n) { return f_from_bits((uint32_t)(n + 127) << 23); }
// p * 2^k in two exact steps, so a subnormal result is rounded once (either
// split of k gives the same bits while p * 2^k1 stays normal)
VPT_HD float scale2(float p, int k) {
    // p is in [0.70, 1.42] (exp_poly of |r| <= ln2 / 2): for -125 <= k <= 127
    // 2^k is a normal float and the product stays normal, so one exact
    // multiply gives the same bits as the two steps
    if (k >= -125 && k <= 127) return p * pow2i(k);
    int k1 = k >> 1;
    int k2 = k - k1;
    return (p * pow2i(k1)) * pow2i(k2);
}

VPT_HD float exp_poly(float r) {
    float p = 1.0f / 40320.0f;
    p = fmaf(p, r, 1.0f / 5040.0f);
    p = fmaf(p, r, 1.0f / 720.0f);
    p = fmaf(p, r, 1.0f / 120.0f);
    p = fmaf(p, r, 1.0f / 24.0f);
    p = fmaf(p, r, 1.0f / 6.0f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return p;
}

VPT_HD float dexp(float x) {
    if (!(x >= -103.97208404541016f && x <= 88.72283935546875f)) {   // NaN, overflow, underflow
        if (x != x) return x;
        return x > 0.0f ? inf_f() : 0.0f;
    }
    float kf = floorf(x * 1.44269502162933350f + 0.5f);
    int k = (int)kf;
    float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187e-06f;
    return scale2(exp_poly(r), k);
}

VPT_HD float dexp2(float x) {
    if (x != x) return x;
    if (x >= 128.0f) return inf_f();
    if (x < -150.0f) return 0.0f;
    float kf = floorf(x + 0.5f);
    int k = (int)kf;
    float r = (x - kf) * 0.693147182464599609f;
    return scale2(exp_poly(r), k);
}

VPT_HD float dlog2(float x) {
    if (x != x) return x;
    if (x < 0.0f) return nan_f();
    if (x == 0.0f) return -inf_f();
    if (x == inf_f()) return x;
    int e = 0;
    uint32_t u = bits_from_f(x);
    if ((u >> 23) == 0) {
        x = x * 8388608.0f;
        u = bits_from_f(x);
        e = -23;
    }
    e += (int)((u >> 23) & 0xffu) - 127;
    float m = f_from_bits((u & 0x007fffffu) | 0x3f800000u);
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

// Integer exponents 1..1024: binary powering from the lowest bit.
VPT_HD float dpow(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (x == 0.0f) return y > 0.0f ? 0.0f : inf_f();
    if (x < 0.0f || x != x || y != y) return nan_f();
    if (y >= 1.0f && y <= 1024.0f && y == floorf(y)) {
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
    return dexp2(y * dlog2(x));
}

VPT_HD float sin_poly(float r) {
    float r2 = r * r;
    float p = 1.0f / 362880.0f;
    p = fmaf(p, r2, -(1.0f / 5040.0f));
    p = fmaf(p, r2, 1.0f / 120.0f);
    p = fmaf(p, r2, -(1.0f / 6.0f));
    return fmaf(r * r2, p, r);
}
VPT_HD float cos_poly(float r) {
    float r2 = r * r;
    float p = -1.0f / 3628800.0f;
    p = fmaf(p, r2, 1.0f / 40320.0f);
    p = fmaf(p, r2, -(1.0f / 720.0f));
    p = fmaf(p, r2, 1.0f / 24.0f);
    p = fmaf(p, r2, -(0.5f));
    return fmaf(r2, p, 1.0f);
}
VPT_HD float reduce_pio2(float x, int* q) {
    float kf = floorf(x * 0.636619746685028076f + 0.5f);
    *q = ((int)kf) & 3;
    return ((x - kf * 1.5703125f) - kf * 4.837512969970703e-4f) - kf * 7.549790126404332e-8f;
}
VPT_HD float dsin(float x) {
    if (x != x || x == inf_f() || x == -inf_f()) return nan_f();
    int q;
    float r = reduce_pio2(x, &q);
    if (q == 0) return sin_poly(r);
    if (q == 1) return cos_poly(r);
    if (q == 2) return -sin_poly(r);
    return -cos_poly(r);
}
VPT_HD float dcos(float x) {
    if (x != x || x == inf_f() || x == -inf_f()) return nan_f();
    int q;
    float r = reduce_pio2(x, &q);
    if (q == 0) return cos_poly(r);
    if (q == 1) return -sin_poly(r);
    if (q == 2) return -cos_poly(r);
    return sin_poly(r);
}
// Both at once (shared reduction), same bits as dsin/dcos.
VPT_HD void dsincos(float x, float* s, float* c) {
    if (x != x || x == inf_f() || x == -inf_f()) { *s = nan_f(); *c = nan_f(); return; }
    int q;
    float r = reduce_pio2(x, &q);
    float sp = sin_poly(r), cp = cos_poly(r);
    if (q == 0) { *s = sp; *c = cp; }
    else if (q == 1) { *s = cp; *c = -sp; }
    else if (q == 2) { *s = -sp; *c = -cp; }
    else { *s = -cp; *c = sp; }
}

VPT_HD float fmaxg(float a, float b) { return fmaxf(a, b); }
VPT_HD float fming(float a, float b) { return fminf(a, b); }
VPT_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
VPT_HD float fract(float x) { return x - floorf(x); }
VPT_HD float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
VPT_HD int isign(float x) { return x > 0.0f ? 1 : (x < 0.0f ? -1 : 0); }

struct v2 { float x, y; };
struct v3 { float x, y, z; };
struct v4 { float x, y, z, w; };

VPT_HD v3 mk3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
VPT_HD v2 mk2(float x, float y) { v2 r; r.x = x; r.y = y; return r; }
VPT_HD v3 add(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
VPT_HD v3 sub(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
VPT_HD v3 mul(v3 a, v3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
VPT_HD v3 muls(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
VPT_HD v3 divs(v3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
VPT_HD v3 neg(v3 a) { return mk3(-a.x, -a.y, -a.z); }
VPT_HD float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
VPT_HD v3 cross(v3 a, v3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
VPT_HD float length(v3 a) { return sqrtf(dot(a, a)); }
// x * (1/length(x)): one IEEE division, as GPU compilers emit normalize()
VPT_HD v3 normalize(v3 a) { return muls(a, 1.0f / length(a)); }
VPT_HD v3 vmax(v3 a, float s) { return mk3(fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)); }
VPT_HD v3 vclamp(v3 a, float lo, float hi) {
    return mk3(clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi));
}
VPT_HD v3 vmix(v3 a, v3 b, float t) { return mk3(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
VPT_HD v3 vmixv(v3 a, v3 b, v3 t) { return mk3(mixf(a.x, b.x, t.x), mixf(a.y, b.y, t.y), mixf(a.z, b.z, t.z)); }

// column-major 4x4 times (x, y, z, w), sums left to right
VPT_HD v4 mat_mul4(const float* m, float x, float y, float z, float w) {
    v4 r;
    r.x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w;
    r.y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w;
    r.z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w;
    r.w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w;
    return r;
}

}  // namespace vpt
