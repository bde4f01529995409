// Block texture arrays and the textured G-buffer pass (GenerateGBuffer.glsl).
//
// Sampling restates what the shader asks of OpenGL, with the choices the GL
// specification leaves to the implementation fixed here:
//   * textureGrad / texture on a GL_TEXTURE_2D_ARRAY with REPEAT wrap,
//     LINEAR magnification and LINEAR_MIPMAP_LINEAR minification
//     (BlockDatabase::SetTextureArraysFilteringLinear,
//     Core/BlockDatabase.cpp:507-517): the level of detail is
//     log2(max(|dP/dx|, |dP/dy|) * size) (isotropic; the 4x anisotropic
//     filtering of Core/GLClasses/TextureArray.cpp:71-77 is not restated),
//     lambda <= 0 samples level 0 bilinearly, otherwise levels floor(lambda)
//     and floor(lambda) + 1 (the last level from lambda >= q on) are sampled
//     bilinearly and mixed by fract(lambda); bilinear weights are fp32 and a
//     texel value is byte / 255, through the sRGB decode table for the albedo
//     array (GL_SRGB_ALPHA, TextureArray.cpp:29);
//   * mip levels (glGenerateMipmap) are the rounded mean of the 2 x 2 texels
//     above, per stored 8-bit channel;
//   * the screen-space derivatives dFdx / dFdy are the fine differences inside
//     the 2 x 2 pixel quad (pixel x | 1 minus pixel x & ~1, likewise in y),
//     with the quad partner's world position reconstructed from its own depth
//     and projected onto this pixel's face axes; a partner outside the image
//     gives a zero derivative.
#include "textures.cuh"

namespace vpt {

namespace {

__global__ void k_mip(const uint8_t* src, uint8_t* dst, int layers, int s2, int ch) {
    // dst: layers x s2 x s2 texels; src: layers x (2 s2) x (2 s2)
    const long long n = (long long)layers * s2 * s2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(q % s2), y = (int)((q / s2) % s2), l = (int)(q / ((long long)s2 * s2));
        const int s1 = 2 * s2;
        const uint8_t* r0 = src + (((long long)l * s1 + 2 * y) * s1 + 2 * x) * ch;
        const uint8_t* r1 = r0 + (long long)s1 * ch;
        for (int c = 0; c < ch; c++)
            dst[q * ch + c] = (uint8_t)(((int)r0[c] + (int)r0[ch + c] + (int)r1[c] + (int)r1[ch + c] + 2) >> 2);
    }
}

// world position of G-buffer texel (i, j): GetPositionAt (GenerateGBuffer.glsl:114-119)
template <typename S>
__device__ __forceinline__ v3 gbuffer_position(const CamView& cam, int W, int H, const S* t, int i, int j, float* dist) {
    const float d = 1.0f / (1.0f / ld(t + (size_t)j * W + i));
    *dist = d;
    return add(ray_origin(cam), muls(normalize(ray_dir_at(cam, texcoord(i, j, W, H))), d));
}

__device__ __forceinline__ float dot2(v2 a) { return a.x * a.x + a.y * a.y; }

// quad difference: value at the odd pixel minus value at the even one
__device__ __forceinline__ float quad_diff(bool odd, float self, float partner) { return odd ? self - partner : partner - self; }

template <typename S>
__global__ void __launch_bounds__(256) k_gbuffer_tex(CamView cam, int W, int H, const S* t, const uint8_t* face,
                                                     const uint8_t* block, BlockTexView tv, S* o_albedo, S* o_normal,
                                                     S* o_pbr, S* o_ao) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= W || j >= H) return;
    const size_t px = (size_t)j * W + i;
    float dist;
    const v3 pos = gbuffer_position(cam, W, H, t, i, j, &dist);
    if (dist < 0.0f) {   // sky (GenerateGBuffer.glsl main, :360-366)
        for (int c = 0; c < 3; c++) {
            st(o_albedo + px * 3 + c, 0.0f);
            st(o_normal + px * 3 + c, 1.0f);
        }
        for (int c = 0; c < 4; c++) st(o_pbr + px * 4 + c, 0.0f);
        st(o_ao + px, 0.0f);
        return;
    }
    const int f = min((int)__ldg(face + px), 5);
    const int bid = min(max((int)__ldg(block + px), 0), 127);
    // CalculateVectors (:440-509): UV = fract of the face coordinates, and
    // GetUVDerivative (:421-438) from the quad partners
    const v2 P = face_coords(pos, f);
    const v2 F = mk2(fract_f(P.x), fract_f(P.y));
    const v2 O = mk2(fract_f(F.x + 0.25f), fract_f(F.y + 0.25f));
    const int ix = i ^ 1, jy = j ^ 1;
    v2 Fx = F, Ox = O, Fy = F, Oy = O;
    if (ix < W) {
        float dn;
        const v2 Pn = face_coords(gbuffer_position(cam, W, H, t, ix, j, &dn), f);
        Fx = mk2(fract_f(Pn.x), fract_f(Pn.y));
        Ox = mk2(fract_f(Fx.x + 0.25f), fract_f(Fx.y + 0.25f));
    }
    if (jy < H) {
        float dn;
        const v2 Pn = face_coords(gbuffer_position(cam, W, H, t, i, jy, &dn), f);
        Fy = mk2(fract_f(Pn.x), fract_f(Pn.y));
        Oy = mk2(fract_f(Fy.x + 0.25f), fract_f(Fy.y + 0.25f));
    }
    const bool ox = i & 1, oy = j & 1;
    v2 dx = mk2(quad_diff(ox, F.x, Fx.x), quad_diff(ox, F.y, Fx.y));
    v2 dy = mk2(quad_diff(oy, F.x, Fy.x), quad_diff(oy, F.y, Fy.y));
    const v2 dx2 = mk2(quad_diff(ox, O.x, Ox.x), quad_diff(ox, O.y, Ox.y));
    const v2 dy2 = mk2(quad_diff(oy, O.x, Oy.x), quad_diff(oy, O.y, Oy.y));
    if (dot2(dx) + dot2(dy) > dot2(dx2) + dot2(dy2)) {
        dx = dx2;
        dy = dy2;
    }
    // GetTextureIDs (:518-550) with the grass override
    int ia = __ldg(tv.ids + bid), in_ = __ldg(tv.ids + 128 + bid), ip = __ldg(tv.ids + 256 + bid);
    const int ie = tv.emissive.texels ? __ldg(tv.ids + 384 + bid) : -1;
    if (bid == tv.grass[0]) {
        const int k = f == 2 ? 1 : (f == 3 ? 7 : 4);   // top, bottom, sides
        ia = tv.grass[k];
        in_ = tv.grass[k + 1];
        ip = tv.grass[k + 2];
    }
    // parallax off: UV = 1 - the flat UV (:388-390)
    const v2 uv = mk2(1.0f - F.x, 1.0f - F.y);
    const float lam = lod_of(tv.normal.size, dx.x, dx.y, dy.x, dy.y);
    // tangent basis of the face (:449-458)
    const v3 T = f < 4 ? mk3(1.0f, 0.0f, 0.0f) : mk3(0.0f, 0.0f, -1.0f);
    const v3 B = f < 2 ? mk3(0.0f, 1.0f, 0.0f) : (f < 4 ? mk3(0.0f, 0.0f, 1.0f) : mk3(0.0f, -1.0f, 0.0f));
    const v3 N = normal_from_id(f, 1.0f);
    float nm[4], pbr[4], alb[4];
    sample_lod(tv.normal, in_, uv.x, uv.y, lam, 3, tv.unorm, nm);
    for (int c = 0; c < 3; c++) nm[c] = nm[c] * 2.0f - 1.0f;
    // tbn * NormalMapped, columns tangent, bitangent, normal
    const v3 nmap = mk3((T.x * nm[0] + B.x * nm[1]) + N.x * nm[2], (T.y * nm[0] + B.y * nm[1]) + N.y * nm[2],
                        (T.z * nm[0] + B.z * nm[1]) + N.z * nm[2]);
    sample_lod(tv.pbr, ip, uv.x, uv.y, lam, 4, tv.unorm, pbr);
    float emis = 0.0f;
    if (ie > -1) {
        // texture() with the implicit derivatives of UV itself
        const v2 ux = mk2(1.0f - Fx.x, 1.0f - Fx.y), uy = mk2(1.0f - Fy.x, 1.0f - Fy.y);
        const float lam_e = lod_of(tv.emissive.size, quad_diff(ox, uv.x, ux.x), quad_diff(ox, uv.y, ux.y),
                                   quad_diff(oy, uv.x, uy.x), quad_diff(oy, uv.y, uy.y));
        float e[4];
        sample_lod(tv.emissive, ie, uv.x, uv.y, lam_e, 1, tv.unorm, e);
        emis = e[0];
    }
    sample_lod(tv.albedo, ia, uv.x, uv.y, lam, 3, tv.srgb, alb);
    // BloomLightLeakFix (:412-418)
    const float lb = 0.02f;
    const float inside = (uv.x > lb && uv.x < 1.0f - lb && uv.y > lb && uv.y < 1.0f - lb) ? 1.0f : 0.0f;
    st(o_albedo + px * 3 + 0, alb[0]);
    st(o_albedo + px * 3 + 1, alb[1]);
    st(o_albedo + px * 3 + 2, alb[2]);
    st(o_normal + px * 3 + 0, nmap.x);
    st(o_normal + px * 3 + 1, nmap.y);
    st(o_normal + px * 3 + 2, nmap.z);
    st(o_pbr + px * 4 + 0, clampf(pbr[0], 0.0f, 1.0f));
    st(o_pbr + px * 4 + 1, clampf(pbr[1], 0.0f, 1.0f));
    st(o_pbr + px * 4 + 2, clampf(pbr[2], 0.0f, 1.0f));
    st(o_pbr + px * 4 + 3, clampf(emis, 0.0f, 1.0f) * inside);
    st(o_ao + px, clampf(pbr[3], 0.00000001f, 1.0f));
}

}  // namespace

cudaError_t tex_build_mip(const TexArray& a, int level, uint8_t* texels, cudaStream_t s) {
    if (level < 0 || level + 1 >= a.levels) return cudaErrorInvalidValue;
    const int s2 = a.size >> (level + 1);
    const long long n = (long long)a.layers * s2 * s2;
    const int grid = (int)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535);
    k_mip<<<grid, 256, 0, s>>>(texels + a.level_off[level] * a.channels, texels + a.level_off[level + 1] * a.channels,
                               a.layers, s2, a.channels);
    return cudaGetLastError();
}

cudaError_t gbuffer_textured(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                             const uint8_t* block, const BlockTexView& tv, void* albedo, void* normal, void* pbr,
                             void* ao, cudaStream_t s) {
    dim3 grid((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8));
    dim3 blk(32, 8);
    if (fp16)
        k_gbuffer_tex<__half><<<grid, blk, 0, s>>>(cam, W, H, (const __half*)t, face, block, tv, (__half*)albedo,
                                                   (__half*)normal, (__half*)pbr, (__half*)ao);
    else
        k_gbuffer_tex<float><<<grid, blk, 0, s>>>(cam, W, H, (const float*)t, face, block, tv, (float*)albedo,
                                                  (float*)normal, (float*)pbr, (float*)ao);
    return cudaGetLastError();
}

}  // namespace vpt
