// Sampling of the block texture arrays as the CUDA path defines GL's fetches
// (textures.cu has the full statement of the choices): REPEAT wrap, fp32
// bilinear weights, texel = a 256-entry table of the byte (byte / 255, or its
// sRGB decode for the albedo array), and
// LINEAR / LINEAR_MIPMAP_LINEAR selection by level of detail. Shared by the
// textured G-buffer pass and the diffuse trace's bounce hits.
#pragma once
#include "dda.cuh"
#include "kernels.cuh"

namespace vpt {

__device__ __forceinline__ float fract_f(float x) { return x - floorf(x); }

// texel channel value: the byte through the array's table (byte / 255 or the
// sRGB decode, computed once on the host: a table load instead of a division)
__device__ __forceinline__ float texel_value(uint8_t v, const float* lut) { return __ldg(lut + v); }

// texture() at one mip level: bilinear with REPEAT wrap and fp32 weights,
// channels [0, nch)
__device__ inline void bilinear_level(const TexArray& a, int level, int layer, float u, float v, int nch, const float* lut,
                               float* out) {
    const int sl = a.size >> level;
    const float x = u * (float)sl - 0.5f, y = v * (float)sl - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float ax = x - x0, ay = y - y0, bx = 1.0f - ax, by = 1.0f - ay;
    const int i0 = wrapi(f2i(x0), sl), j0 = wrapi(f2i(y0), sl);
    const int i1 = i0 + 1 == sl ? 0 : i0 + 1, j1 = j0 + 1 == sl ? 0 : j0 + 1;
    const uint8_t* base = a.texels + (a.level_off[level] + (long long)layer * sl * sl) * a.channels;
    const uint8_t* p00 = base + ((long long)j0 * sl + i0) * a.channels;
    const uint8_t* p10 = base + ((long long)j0 * sl + i1) * a.channels;
    const uint8_t* p01 = base + ((long long)j1 * sl + i0) * a.channels;
    const uint8_t* p11 = base + ((long long)j1 * sl + i1) * a.channels;
    // a texel's channels in one load (RGBA8 texels are 4-byte aligned)
    uint32_t w00, w10, w01, w11;
    if (a.channels == 4) {
        w00 = __ldg(reinterpret_cast<const uint32_t*>(p00));
        w10 = __ldg(reinterpret_cast<const uint32_t*>(p10));
        w01 = __ldg(reinterpret_cast<const uint32_t*>(p01));
        w11 = __ldg(reinterpret_cast<const uint32_t*>(p11));
    } else {
        w00 = __ldg(p00);
        w10 = __ldg(p10);
        w01 = __ldg(p01);
        w11 = __ldg(p11);
    }
    for (int c = 0; c < nch; c++) {
        const int sh = 8 * c;
        const float v00 = texel_value((uint8_t)(w00 >> sh), lut), v10 = texel_value((uint8_t)(w10 >> sh), lut);
        const float v01 = texel_value((uint8_t)(w01 >> sh), lut), v11 = texel_value((uint8_t)(w11 >> sh), lut);
        const float lo = v00 * bx + v10 * ax;
        const float hi = v01 * bx + v11 * ax;
        out[c] = lo * by + hi * ay;
    }
}

// level of detail of textureGrad(dPdx, dPdy) on a size x size array
__device__ __forceinline__ float lod_of(int size, float dxu, float dxv, float dyu, float dyv) {
    const float s = (float)size;
    const float ax = dxu * s, ay = dxv * s, bx = dyu * s, by = dyv * s;
    const float rx = sqrtf(ax * ax + ay * ay), ry = sqrtf(bx * bx + by * by);
    return dlog2(fmaxf(rx, ry));
}

// LINEAR magnification / LINEAR_MIPMAP_LINEAR minification at level of detail lam
__device__ inline void sample_lod(const TexArray& a, int layer_id, float u, float v, float lam, int nch, const float* lut,
                           float* out) {
    const int layer = min(max(layer_id, 0), a.layers - 1);
    const int q = a.levels - 1;
    if (!(lam > 0.0f)) {
        bilinear_level(a, 0, layer, u, v, nch, lut, out);
        return;
    }
    if (lam >= (float)q) {
        bilinear_level(a, q, layer, u, v, nch, lut, out);
        return;
    }
    const float d1f = floorf(lam);
    const int d1 = (int)d1f;
    const float f = lam - d1f;
    float t1[4], t2[4];
    bilinear_level(a, d1, layer, u, v, nch, lut, t1);
    bilinear_level(a, d1 + 1, layer, u, v, nch, lut, t2);
    for (int c = 0; c < nch; c++) out[c] = (1.0f - f) * t1[c] + f * t2[c];
}

// the two face coordinates CalculateVectors (GenerateGBuffer.glsl:440-509)
// and CalculateUV (DiffuseRayTraceFrag.glsl:1235-1273) take for face id f:
// (x, y) for +-Z, (x, z) for +-Y, (z, y) for +-X
__device__ __forceinline__ v2 face_coords(v3 p, int f) {
    const int axis = f >> 1;
    return axis == 0 ? mk2(p.x, p.y) : (axis == 1 ? mk2(p.x, p.z) : mk2(p.z, p.y));
}

// textureLod at an integer level: the level's bilinear sample (the last
// level from q on)
__device__ __forceinline__ void sample_level(const TexArray& a, int layer_id, float u, float v, int level, int nch,
                                             const float* lut, float* out) {
    const int layer = min(max(layer_id, 0), a.layers - 1);
    bilinear_level(a, min(level, a.levels - 1), layer, u, v, nch, lut, out);
}

// channel c alone of a textureLod at an integer level
__device__ __forceinline__ float sample_channel_level(const TexArray& a, int layer_id, float u, float v, int level,
                                                      int c, const float* lut) {
    float out[4];
    sample_level(a, layer_id, u, v, level, c + 1, lut, out);
    return out[c];
}

// StopRay (InitialRayTraceFrag.glsl:189-202): an opaque block stops the ray;
// a transparent one (BlockTransparentData) only where the albedo alpha,
// sampled at the face UV (CalculateUV, both coordinates flipped) at level
// int(log2(size / ((1 / D) * K))) clamped to 0..8 (D the distance to the
// camera, K = 1 / (2 tan(fov / (2 W))) in pixels per radian; the reference
// writes its 512-texel size as a constant), exceeds 0.975.
// The shadow pass's StopRay (ShadowRayTraceFrag.glsl:105-117) flips only the
// v coordinate and samples two levels finer (flip_x = 0, lod_bias = -2).
struct AlphaStop {
    BlockTexView tv;
    v3 cam;
    float k;
    int flip_x = 1, lod_bias = 0;
    __device__ __forceinline__ bool operator()(v3 p, v3 n, int type) const {
        const int id = min(max(type, 0), 127);
        if (__ldg(tv.ids + 512 + id) == 0) return true;
        const v2 fc = face_coords(p, normal_id(n));
        const float u = flip_x ? 1.0f - fract_f(fc.x) : fract_f(fc.x), v = 1.0f - fract_f(fc.y);
        const float D = length(sub(p, cam));
        const int lod = min(max(f2i(dlog2((float)tv.albedo.size / ((1.0f / D) * k))) + lod_bias, 0), 8);
        return sample_channel_level(tv.albedo, __ldg(tv.ids + id), u, v, lod, 3, tv.unorm) > 0.975f;
    }
};

}  // namespace vpt
