// Device-side building blocks shared by the trace, filter and colour kernels:
// camera rays, plane access with the OpenGL sampling rules the reference
// relies on, material lookup, the BRDF / spherical-harmonic helpers and the
// per-pixel random stream. Each helper cites the shader function it restates.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "vmath.cuh"
#include "vpt.h"

namespace vpt {

constexpr float kPI = 3.14159265359f;   // DiffuseRayTraceFrag.glsl:11, ColorPassFrag.glsl:6
constexpr int kFaceMiss = 10;           // round(1.0 * 10) decoded from a miss (InitialRayTraceFrag.glsl:454)

// ------------------------------------------------------------------ world --
struct WorldView {
    const uint8_t* vox;       // block ids, x fastest
    const uint8_t* df;        // Manhattan distance field: x fastest, or in BxBxB bricks (df_index)
    int X, Y, Z;
    const vpt_block* blocks;  // block table
    int n_blocks;
    int bx, by;               // bricks along x and y (brick layouts only)
};

struct CamView {
    float inv_view[16];
    float inv_proj[16];
    float pos[3];             // u_ViewerPosition
};

__device__ __forceinline__ int vox_index(const WorldView& w, int x, int y, int z) {
    return x + w.X * (y + w.Y * z);
}
// Distance-field address of voxel (x, y, z). B == 0: the x-fastest layout of
// the voxel volume. B == 4 or 8: the volume padded to whole BxBxB bricks,
// bricks in x-fastest order, each brick's B^3 bytes x-fastest, so the
// neighbourhood a ray probes in a few steps shares a few 32-byte sectors
// whichever way the ray goes.
template <int B>
__host__ __device__ __forceinline__ int df_index(const WorldView& w, int x, int y, int z) {
    if constexpr (B == 0) {
        return x + w.X * (y + w.Y * z);
    } else {
        static_assert(B == 4 || B == 8, "brick edge 4 or 8");
        constexpr int L = B == 4 ? 2 : 3;
        const int brick = ((z >> L) * w.by + (y >> L)) * w.bx + (x >> L);
        return (brick << (3 * L)) + ((((z & (B - 1)) << L) + (y & (B - 1))) << L) + (x & (B - 1));
    }
}
__device__ __forceinline__ bool in_volume(const WorldView& w, int x, int y, int z) {
    // IsInVolume (InitialRayTraceFrag.glsl:68-77): 0 <= x <= X-1, ... as unsigned compares
    return (unsigned)x < (unsigned)w.X && (unsigned)y < (unsigned)w.Y && (unsigned)z < (unsigned)w.Z;
}
__device__ __forceinline__ int get_voxel(const WorldView& w, int x, int y, int z) {
    // GetVoxel (InitialRayTraceFrag.glsl:79-87)
    return in_volume(w, x, y, z) ? (int)__ldg(w.vox + vox_index(w, x, y, z)) : 0;
}

// --------------------------------------------------------------- camera --
__device__ __forceinline__ v2 texcoord(int i, int j, int W, int H) {
    return mk2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
}
// GetRayDirectionAt (ShadowRayTraceFrag.glsl:303-308), GetRayStuff (InitialRayTraceFrag.glsl:398-414)
__device__ __forceinline__ v3 ray_dir_at(const CamView& c, v2 uv) {
    float cx = uv.x * 2.0f - 1.0f;
    float cy = uv.y * 2.0f - 1.0f;
    v4 e = mat_mul4(c.inv_proj, cx, cy, -1.0f, 1.0f);
    v4 d = mat_mul4(c.inv_view, e.x, e.y, -1.0f, 0.0f);
    return mk3(d.x, d.y, d.z);
}
__device__ __forceinline__ v3 ray_origin(const CamView& c) {
    return mk3(c.inv_view[12], c.inv_view[13], c.inv_view[14]);
}

// GetNormalFromID (SVGF/TemporalFilter.glsl:108-119); `miss` is the value
// ids above 5 decode to (1.0, or 0.5 in DiffuseRayTraceFrag.glsl:790-801).
__device__ __forceinline__ v3 normal_from_id(int id, float miss) {
    switch (id) {
        case 0: return mk3(0.0f, 0.0f, 1.0f);
        case 1: return mk3(0.0f, 0.0f, -1.0f);
        case 2: return mk3(0.0f, 1.0f, 0.0f);
        case 3: return mk3(0.0f, -1.0f, 0.0f);
        case 4: return mk3(-1.0f, 0.0f, 0.0f);
        case 5: return mk3(1.0f, 0.0f, 0.0f);
        default: return mk3(miss, miss, miss);
    }
}

// max(dot(normal_from_id(a, 1), normal_from_id(b, 1)), 0) as an integer: the
// normals are axis vectors or (1, 1, 1) for a miss, so the clamped dot product
// is exactly 0, 1 or 3 (both misses). Checked against the dot product for all
// 256 x 256 id pairs.
__device__ __forceinline__ int face_cos(int a, int b) {
    const unsigned pos = 0x25u;   // ids whose normal is +z (0), +y (2) or +x (5)
    const bool ma = (unsigned)a > 5u, mb = (unsigned)b > 5u;
    if (ma) return mb ? 3 : (int)((pos >> b) & 1u);
    if (mb) return (int)((pos >> a) & 1u);
    return a == b ? 1 : 0;
}

// ------------------------------------------------------------ storage --
__device__ __forceinline__ float ld(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ld(const __half* p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ void st(float* p, float v) { *p = v; }
__device__ __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }

__device__ __forceinline__ int wrapi(int i, int n) {
    // almost every index is already inside: one compare instead of an integer
    // division (which the GPU has no instruction for)
    if ((unsigned)i < (unsigned)n) return i;
    int r = i % n;
    return r < 0 ? r + n : r;
}

// Vector loads of 4 / 2 interleaved channels (planes are cudaMalloc'd, so a
// pixel's channels are 16 / 8 byte aligned in fp32 and 8 / 4 in fp16).
__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ld4(const __half* p) {
    uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
    __half2 a = *reinterpret_cast<__half2*>(&u.x), b = *reinterpret_cast<__half2*>(&u.y);
    float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ float2 ld2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
__device__ __forceinline__ float2 ld2(const __half* p) {
    unsigned u = __ldg(reinterpret_cast<const unsigned*>(p));
    return __half22float2(*reinterpret_cast<__half2*>(&u));
}
__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void st4(__half* p, float a, float b, float c, float d) {
    __half2 x = __floats2half2_rn(a, b), y = __floats2half2_rn(c, d);
    uint2 u;
    u.x = *reinterpret_cast<unsigned*>(&x);
    u.y = *reinterpret_cast<unsigned*>(&y);
    *reinterpret_cast<uint2*>(p) = u;
}
__device__ __forceinline__ void st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }
__device__ __forceinline__ void st2(__half* p, float a, float b) {
    __half2 x = __floats2half2_rn(a, b);
    *reinterpret_cast<unsigned*>(p) = *reinterpret_cast<unsigned*>(&x);
}

// Bilinear footprint of texture() with GL_LINEAR + GL_REPEAT at uv on a W x H
// plane: texel offsets and fp32 weights, shared by every plane sampled there.
struct Bilin {
    int o00, o10, o01, o11;   // pixel indices
    float ax, ay, bx, by;     // weights: bx = 1 - ax, by = 1 - ay
};
__device__ __forceinline__ Bilin bilin(v2 uv, int W, int H) {
    float x = uv.x * (float)W - 0.5f;
    float y = uv.y * (float)H - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    Bilin b;
    b.ax = x - x0;
    b.ay = y - y0;
    b.bx = 1.0f - b.ax;
    b.by = 1.0f - b.ay;
    int i0 = wrapi(f2i(x0), W), j0 = wrapi(f2i(y0), H);
    int i1 = i0 + 1 == W ? 0 : i0 + 1;
    int j1 = j0 + 1 == H ? 0 : j0 + 1;
    b.o00 = j0 * W + i0;
    b.o10 = j0 * W + i1;
    b.o01 = j1 * W + i0;
    b.o11 = j1 * W + i1;
    return b;
}
// (v00*(1-ax) + v10*ax)*(1-ay) + (v01*(1-ax) + v11*ax)*ay, per channel
__device__ __forceinline__ float blend(const Bilin& b, float v00, float v10, float v01, float v11) {
    float lo = v00 * b.bx + v10 * b.ax;
    float hi = v01 * b.bx + v11 * b.ax;
    return lo * b.by + hi * b.ay;
}

// Packed fp32 pairs: sm_100-family GPUs issue two fp32 adds or multiplies as
// one instruction, each lane the same round-to-nearest operation as the
// scalar code, so the bits are unchanged and the filters, which are bound by
// instruction issue, spend fewer issue slots on their blends and sums.
// A packed product must never feed a packed sum directly: the code generator
// contracts that pair into a packed fused multiply-add (one rounding instead
// of two) even with --fmad=false and explicit .rn, as a device test of these
// helpers showed. So products are packed and the sums that take them are
// scalar (the scalar pair is not contracted); padd only adds values that are
// not packed products.
__device__ __forceinline__ float2 pmul(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 padd(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }
// a + b lane by lane as two scalar adds (for sums of packed products)
__device__ __forceinline__ float2 sadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
// acc + v * w for two channels with one weight (the filters' weighted sums)
__device__ __forceinline__ float2 pacc(float2 acc, float2 v, float w) { return sadd(acc, pmul(v, splat(w))); }

// dexp of two arguments with packed products and polynomial steps: lane by
// lane the operations of dexp (vmath.cuh), so the same bits; arguments
// outside its polynomial range take the scalar function.
__device__ __forceinline__ float2 dexp_pair(float a, float b) {
    const float lo = -103.97208404541016f, hi = 88.72283935546875f;
    if (!(a >= lo && a <= hi && b >= lo && b <= hi)) return make_float2(dexp(a), dexp(b));
    const float2 x = make_float2(a, b);
    const float2 t = sadd(pmul(x, splat(1.44269502162933350f)), splat(0.5f));
    const float2 kf = make_float2(floorf(t.x), floorf(t.y));
    // (x - kf * ln2_hi) - kf * ln2_lo, each subtraction an addition of the negated product
    const float2 r = sadd(sadd(x, pmul(kf, splat(-0.693145751953125f))), pmul(kf, splat(-1.428606765330187e-06f)));
    float2 q = splat(1.0f / 40320.0f);
    q = __ffma2_rn(q, r, splat(1.0f / 5040.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 720.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 120.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 24.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 6.0f));
    q = __ffma2_rn(q, r, splat(0.5f));
    q = __ffma2_rn(q, r, splat(1.0f));
    q = __ffma2_rn(q, r, splat(1.0f));
    const int k0 = (int)kf.x, k1 = (int)kf.y;
    if (k0 >= -125 && k0 <= 127 && k1 >= -125 && k1 <= 127) return pmul(q, make_float2(pow2i(k0), pow2i(k1)));
    return make_float2(scale2(q.x, k0), scale2(q.y, k1));
}

// dexp_pair for arguments that are never positive (the filters' negated
// distances and differences; the caller guarantees a <= 0 and b <= 0 unless
// NaN): the same operations, without the range tests a positive argument
// needs (kf = floor(x log2(e) + 1/2) <= 0 here, so k <= 127 always). NaN and
// arguments below the polynomial's range take the scalar function.
__device__ __forceinline__ float2 dexp_pair_np(float a, float b) {
    const float lo = -103.97208404541016f;
    if (!(a >= lo && b >= lo)) return make_float2(dexp(a), dexp(b));
    const float2 x = make_float2(a, b);
    const float2 t = sadd(pmul(x, splat(1.44269502162933350f)), splat(0.5f));
    const float2 kf = make_float2(floorf(t.x), floorf(t.y));
    const float2 r = sadd(sadd(x, pmul(kf, splat(-0.693145751953125f))), pmul(kf, splat(-1.428606765330187e-06f)));
    float2 q = splat(1.0f / 40320.0f);
    q = __ffma2_rn(q, r, splat(1.0f / 5040.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 720.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 120.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 24.0f));
    q = __ffma2_rn(q, r, splat(1.0f / 6.0f));
    q = __ffma2_rn(q, r, splat(0.5f));
    q = __ffma2_rn(q, r, splat(1.0f));
    q = __ffma2_rn(q, r, splat(1.0f));
    const int k0 = (int)kf.x, k1 = (int)kf.y;
    if (k0 >= -125 && k1 >= -125) return pmul(q, make_float2(pow2i(k0), pow2i(k1)));
    return make_float2(scale2(q.x, k0), scale2(q.y, k1));
}

// x / 5 for finite x in three operations: q = x * RN(1/5), then one
// correction with the exact remainder, q + fma(-q, 5, x) * RN(1/5)
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990). For the divisor 5 this is
// IEEE division's result for every finite x, which the oracle's exhaustive
// check over all 2^31 non-negative finite floats establishes (the form is
// odd in x); the device division instead takes a reciprocal estimate,
// refinement steps and a range check.
__device__ __forceinline__ float div5(float x) {
    const float y = 0.2f;   // RN(1/5)
    const float q = __fmul_rn(x, y);
    return __fmaf_rn(__fmaf_rn(-q, 5.0f, x), y, q);
}

// blend of two channels at once
__device__ __forceinline__ float2 blend2(const Bilin& b, float2 v00, float2 v10, float2 v01, float2 v11) {
    const float2 bx = splat(b.bx), ax = splat(b.ax);
    const float2 lo = sadd(pmul(v00, bx), pmul(v10, ax));
    const float2 hi = sadd(pmul(v01, bx), pmul(v11, ax));
    return sadd(pmul(lo, splat(b.by)), pmul(hi, splat(b.ay)));
}
// blend of one channel, its two rows at once
__device__ __forceinline__ float blend1(const Bilin& b, float v00, float v10, float v01, float v11) {
    const float2 r = sadd(pmul(make_float2(v00, v01), splat(b.bx)), pmul(make_float2(v10, v11), splat(b.ax)));
    const float2 q = pmul(r, make_float2(b.by, b.ay));
    return q.x + q.y;
}
// Scalar blend of one channel: the a-trous iteration's single-channel taps
// (depth, variance), whose packed form needs operand copies its register
// budget cannot spare, measured faster with it.
template <typename S>
__device__ __forceinline__ float bl1s(const S* p, const Bilin& b) {
    return blend(b, ld(p + b.o00), ld(p + b.o10), ld(p + b.o01), ld(p + b.o11));
}
template <typename S>
__device__ __forceinline__ float bl1(const S* p, const Bilin& b) {
    return blend1(b, ld(p + b.o00), ld(p + b.o10), ld(p + b.o01), ld(p + b.o11));
}
template <typename S>
__device__ __forceinline__ float2 bl2(const S* p, const Bilin& b) {
    float2 a = ld2(p + 2 * (size_t)b.o00), c = ld2(p + 2 * (size_t)b.o10);
    float2 d = ld2(p + 2 * (size_t)b.o01), e = ld2(p + 2 * (size_t)b.o11);
    return blend2(b, a, c, d, e);
}
template <typename S>
__device__ __forceinline__ float4 bl4(const S* p, const Bilin& b) {
    float4 a = ld4(p + 4 * (size_t)b.o00), c = ld4(p + 4 * (size_t)b.o10);
    float4 d = ld4(p + 4 * (size_t)b.o01), e = ld4(p + 4 * (size_t)b.o11);
    const float2 xy = blend2(b, make_float2(a.x, a.y), make_float2(c.x, c.y), make_float2(d.x, d.y),
                             make_float2(e.x, e.y));
    const float2 zw = blend2(b, make_float2(a.z, a.w), make_float2(c.z, c.w), make_float2(d.z, d.w),
                             make_float2(e.z, e.w));
    return make_float4(xy.x, xy.y, zw.x, zw.y);
}

// A W x H plane with C interleaved channels of storage type S.
template <typename S, int C>
struct Plane {
    const S* p;
    int W, H;
    __device__ __forceinline__ float at(int i, int j, int c) const {
        return ld(p + ((size_t)wrapi(j, H) * W + wrapi(i, W)) * C + c);
    }
    __device__ __forceinline__ float at_in(int i, int j, int c) const {   // i, j known in range
        return ld(p + ((size_t)j * W + i) * C + c);
    }
    // texture() with GL_LINEAR and GL_REPEAT (Core/GLClasses/Framebuffer.cpp:64-70), fp32 weights
    __device__ __forceinline__ void linear(v2 uv, float* out) const {
        float x = uv.x * (float)W - 0.5f;
        float y = uv.y * (float)H - 0.5f;
        float x0 = floorf(x), y0 = floorf(y);
        float ax = x - x0, ay = y - y0;
        int i0 = wrapi(f2i(x0), W), j0 = wrapi(f2i(y0), H);
        int i1 = i0 + 1 == W ? 0 : i0 + 1;
        int j1 = j0 + 1 == H ? 0 : j0 + 1;
        const S* r0 = p + (size_t)j0 * W * C;
        const S* r1 = p + (size_t)j1 * W * C;
#pragma unroll
        for (int c = 0; c < C; c++) {
            float v00 = ld(r0 + i0 * C + c), v10 = ld(r0 + i1 * C + c);
            float v01 = ld(r1 + i0 * C + c), v11 = ld(r1 + i1 * C + c);
            float b = v00 * (1.0f - ax) + v10 * ax;
            float t = v01 * (1.0f - ax) + v11 * ax;
            out[c] = b * (1.0f - ay) + t * ay;
        }
    }
};

struct Plane8 {
    const uint8_t* p;
    int W, H;
    __device__ __forceinline__ int at(int i, int j) const { return __ldg(p + (size_t)wrapi(j, H) * W + wrapi(i, W)); }
    __device__ __forceinline__ int at_in(int i, int j) const { return __ldg(p + (size_t)j * W + i); }
    // texture() with GL_NEAREST and GL_REPEAT
    __device__ __forceinline__ int nearest(v2 uv) const {
        return at(f2i_floor(uv.x * (float)W), f2i_floor(uv.y * (float)H));
    }
};

// GetPositionAt (SVGF/TemporalFilter.glsl:82-86) at a texel centre or anywhere.
template <typename S>
__device__ __forceinline__ v4 position_fetch(const CamView& c, const Plane<S, 1>& t, int i, int j, v2 txc) {
    float d = t.at_in(i, j, 0);
    v3 p = add(ray_origin(c), muls(normalize(ray_dir_at(c, txc)), d));
    v4 r; r.x = p.x; r.y = p.y; r.z = p.z; r.w = d;
    return r;
}
template <typename S>
__device__ __forceinline__ v4 position_linear(const CamView& c, const Plane<S, 1>& t, v2 txc) {
    float d;
    t.linear(txc, &d);
    v3 p = add(ray_origin(c), muls(normalize(ray_dir_at(c, txc)), d));
    v4 r; r.x = p.x; r.y = p.y; r.z = p.z; r.w = d;
    return r;
}

// ------------------------------------------------------------- shading --
__device__ __forceinline__ float luminance(v3 c) { return dot(c, mk3(0.299f, 0.587f, 0.114f)); }
__device__ __forceinline__ float sh_to_y(const float* sh) { return fmaxf(0.0f, 3.544905f * sh[3]); }

// Analytic horizon-to-zenith sky standing in for the atmosphere cubemap.
__device__ __forceinline__ v3 sky_radiance(v3 d) {
    v3 n = normalize(d);
    float a = clampf(n.y, 0.0f, 1.0f);
    return vmix(mk3(0.62f, 0.74f, 0.92f), mk3(0.20f, 0.38f, 0.85f), a);
}
// GetSkyColorAt (DiffuseRayTraceFrag.glsl:984-988)
__device__ __forceinline__ v3 sky_color_at(v3 rd) {
    rd.y = clampf(rd.y, 0.125f, 1.5f);
    return sky_radiance(rd);
}

// IrridianceToSH (DiffuseRayTraceFrag.glsl:766-784)
__device__ __forceinline__ void irradiance_to_sh(v3 r, v3 d, float* sh, float* cocg) {
    float co = r.x - r.z;
    float t = r.z + co * 0.5f;
    float cg = r.y - t;
    float y = fmaxf(t + cg * 0.5f, 0.0f);
    float l00 = 0.282095f;
    float l1_1 = 0.488603f * d.y;
    float l10 = 0.488603f * d.z;
    float l11 = 0.488603f * d.x;
    sh[0] = fmaxf(l11 * y, -100.0f);
    sh[1] = fmaxf(l1_1 * y, -100.0f);
    sh[2] = fmaxf(l10 * y, -100.0f);
    sh[3] = fmaxf(l00 * y, -100.0f);
    cocg[0] = co;
    cocg[1] = cg;
}

// SHToIrridiance (ColorPassFrag.glsl:357-368)
__device__ __forceinline__ v3 sh_to_irradiance(const float* sh, const float* cocg_in, v3 v) {
    float x = dot(mk3(sh[0], sh[1], sh[2]), v);
    float y = 2.0f * (1.023326f * x + 0.886226f * sh[3]);
    y = fmaxf(y, 0.0f);
    float s = (y * 0.282095f) / (sh[3] + 1e-6f);
    float co = cocg_in[0] * s, cg = cocg_in[1] * s;
    float t = y - cg * 0.5f;
    float g = cg + t;
    float b = t - co * 0.5f;
    float r = b + co;
    return vmax(mk3(r, g, b), 0.0f);
}

// InverseSchlick (DiffuseRayTraceFrag.glsl:1305-1308)
__device__ __forceinline__ float inverse_schlick(float f0, float voh) {
    return 1.0f - clampf(f0 + (1.0f - f0) * dpow(1.0f - voh, 5.0f), 0.0f, 1.0f);
}

// DiffuseHammon (DiffuseRayTraceFrag.glsl:1311-1332), rcp(x) = 1/x
__device__ __forceinline__ float diffuse_hammon(v3 n, v3 v, v3 l, float rough) {
    float ndl = fmaxf(dot(n, l), 0.0f);
    if (ndl <= 0.0f) return 0.0f;
    float ndv = fmaxf(dot(n, v), 0.0f);
    float ldv = fmaxf(dot(l, v), 0.0f);
    v3 h = normalize(add(v, l));
    float ndh = fmaxf(dot(n, h), 0.0f);
    float facing = ldv * 0.5f + 0.5f;
    float single_rough = facing * (0.9f - 0.4f * facing) * ((0.5f + ndh) * (1.0f / fmaxf(ndh, 0.02f)));
    float single_smooth = 1.05f * inverse_schlick(0.0f, ndl) * inverse_schlick(0.0f, fmaxf(ndv, 0.0f));
    float single = clampf(mixf(single_smooth, single_rough, rough) * (1.0f / kPI), 0.0f, 1.0f);
    float multi = 0.1159f * rough;
    return clampf((multi + single) * ndl, 0.0f, 1.0f);
}

// ---------------------------------------------------------------- random --
// PCG-RXS-M-XS 32 (Jarzynski & Olano 2020), seeded per pixel; stands in for
// the reference's fract(sin()) / blue-noise sequences.
__host__ __device__ __forceinline__ uint32_t pcg_step(uint32_t* s) {
    *s = *s * 747796405u + 2891336453u;
    uint32_t w = ((*s >> ((*s >> 28u) + 4u)) ^ *s) * 277803737u;
    return (w >> 22u) ^ w;
}
__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    uint32_t s = v;
    return pcg_step(&s);
}
__device__ __forceinline__ float rand01(uint32_t* s) { return (float)(pcg_step(s) >> 8) * (1.0f / 16777216.0f); }

// cosWeightedRandomHemisphereDirection (DiffuseRayTraceFrag.glsl:945-967)
__device__ __forceinline__ v3 cos_hemisphere(v3 n, uint32_t* rng) {
    float rx_ = rand01(rng);
    float ry_ = rand01(rng);
    float pi2 = 2.0f * kPI;
    v3 uu = normalize(cross(n, mk3(0.0f, 1.0f, 1.0f)));
    v3 vv = cross(uu, n);
    float ra = sqrtf(ry_);
    float sn, cs;
    dsincos(pi2 * rx_, &sn, &cs);
    float rx = ra * cs;
    float ry = ra * sn;
    float rz = sqrtf(1.0f - ry_);
    v3 rr = mk3((rx * uu.x + ry * vv.x) + rz * n.x, (rx * uu.y + ry * vv.y) + rz * n.y,
                (rx * uu.z + ry * vv.z) + rz * n.z);
    return normalize(rr);
}

// ------------------------------------------------------------- materials --
struct Material {
    v3 albedo;
    float rough, metal;
    int emissive;
};
__device__ __forceinline__ Material material(const WorldView& w, int id) {
    if (id < 0 || id >= w.n_blocks) id = 0;
    const uint8_t* b = reinterpret_cast<const uint8_t*>(w.blocks + id);
    Material m;
    m.albedo = mk3((float)__ldg(b + 0) / 255.0f, (float)__ldg(b + 1) / 255.0f, (float)__ldg(b + 2) / 255.0f);
    m.rough = (float)__ldg(b + 3) / 255.0f;
    m.metal = (float)__ldg(b + 4) / 255.0f;
    m.emissive = __ldg(b + 5) ? 1 : 0;
    return m;
}

// The PBR G-buffer's roughness / metalness for flat materials
// (GenerateGBuffer.glsl: nearest filtered, 0 for the sky, :362-363).
__device__ __forceinline__ float pbr_rough(const WorldView& w, int block) {
    return block > 0 ? material(w, min(block, 127)).rough : 0.0f;
}
__device__ __forceinline__ float pbr_metal(const WorldView& w, int block) {
    return block > 0 ? material(w, min(block, 127)).metal : 0.0f;
}

// texture(u_GBufferNormals, uv): the RGB16F normal G-buffer with GL_LINEAR,
// i.e. the face normals ((1, 1, 1) for the sky) blended bilinearly.
__device__ __forceinline__ v3 gnormal_linear(const uint8_t* face, int W, int H, v2 uv) {
    const Bilin b = bilin(uv, W, H);
    const v3 n00 = normal_from_id(__ldg(face + b.o00), 1.0f), n10 = normal_from_id(__ldg(face + b.o10), 1.0f);
    const v3 n01 = normal_from_id(__ldg(face + b.o01), 1.0f), n11 = normal_from_id(__ldg(face + b.o11), 1.0f);
    return mk3(blend(b, n00.x, n10.x, n01.x, n11.x), blend(b, n00.y, n10.y, n01.y, n11.y),
               blend(b, n00.z, n10.z, n01.z, n11.z));
}

// Per-frame constants of DiffuseRayTraceFrag main (:832-839), computed once on the host.
struct GILighting {
    float light_color[3];
    float light_dir[3];
    int moon_stronger;
    float emissivity_multiplier;
    float sun_visibility;          // Core/Pipeline.cpp:1828
    float gi_sky_strength;
    float diffuse_light_intensity;
};

}  // namespace vpt
