// Colour pass (ColorPassFrag.glsl main, :747-1083) for flat materials: the
// 3x3 joint-bilateral GI gather and shadow filter (SpatiallyUpscaleBuffers),
// Cook-Torrance direct sun/moon light with the traced shadow, SH irradiance
// decode of the denoised GI, VXAO and the DFG (Karis) indirect combine
// (u_UseDFG on, Core/Pipeline.cpp:3683). One thread per pixel, a streaming
// pass over the G-buffer and the denoised planes.
#include "kernels.cuh"

namespace vpt {

namespace {

// FresnelSchlickRoughness (ColorPassFrag.glsl:1205-1209)
__device__ __forceinline__ v3 fresnel_schlick_roughness(v3 eye, v3 n, v3 f0, float rough) {
    float cos_theta = clampf(dot(eye, n), 0.00001f, 1.0f);
    float k = dpow(1.0f - cos_theta, 5.0f);
    v3 m = mk3(fmaxf(1.0f - rough, f0.x), fmaxf(1.0f - rough, f0.y), fmaxf(1.0f - rough, f0.z));
    return add(f0, muls(sub(m, f0), k));
}

// CalculateDirectionalLight (ColorPassFrag.glsl:419-451) with ndfGGX (:394-400)
// and gaSchlickGGX (:402-412)
__device__ __forceinline__ v3 directional_light(v3 viewer, v3 wp, v3 light_dir, v3 radiance, v3 radiance_s,
                                                v3 albedo, v3 n, float rough, float metal, float shadow) {
    const float DIELECTRIC = 0.04f, Epsilon = 0.00001f;
    float sh = fminf(shadow, 1.0f);
    v3 lo = normalize(sub(viewer, wp));
    float cos_lo = fmaxf(0.0f, dot(n, lo));
    v3 f0 = vmix(mk3(DIELECTRIC, DIELECTRIC, DIELECTRIC), albedo, metal);
    v3 li = light_dir;
    v3 lh = normalize(add(li, lo));
    float cos_li = fmaxf(0.0f, dot(n, li));
    float cos_lh = fmaxf(0.0f, dot(n, lh));
    v3 F = fresnel_schlick_roughness(lo, n, f0, rough);
    float alpha = rough * rough;
    float alpha_sq = alpha * alpha;
    float denom = (cos_lh * cos_lh) * (alpha_sq - 1.0f) + 1.0f;
    float D = alpha_sq / ((kPI * denom) * denom);
    float r1 = rough + 1.0f;
    float k = (r1 * r1) / 8.0f;
    float G = (cos_li / (cos_li * (1.0f - k) + k)) * (cos_lo / (cos_lo * (1.0f - k) + k));
    v3 kd = vmix(sub(mk3(1.0f, 1.0f, 1.0f), F), mk3(0.0f, 0.0f, 0.0f), metal);
    v3 diffuse_brdf = mul(kd, albedo);
    v3 spec = divs(muls(muls(F, D), G), fmaxf(Epsilon, (4.0f * cos_li) * cos_lo));
    spec = vclamp(spec, 0.0f, 2.0f);
    v3 result = add(muls(mul(diffuse_brdf, radiance), cos_li), muls(mul(spec, radiance_s), cos_li));
    return muls(vclamp(result, 0.0f, 2.5f), clampf(1.0f - sh, 0.0f, 1.0f));
}

// BasicSaturation (ColorPassFrag.glsl:1227-1232)
__device__ __forceinline__ v3 basic_saturation(v3 c, float adj) {
    float l = dot(c, mk3(0.2125f, 0.7154f, 0.0721f));
    return vmix(mk3(l, l, l), c, adj);
}

// KarisEnvBRDFApprox (ColorPassFrag.glsl:384-391)
__device__ __forceinline__ v2 karis_env_brdf(float ndv, float rough) {
    float rx = rough * -1.0f + 1.0f;
    float ry = rough * -0.0275f + 0.0425f;
    float rz = rough * -0.572f + 1.040f;
    float rw = rough * 0.022f + -0.040f;
    float a004 = fminf(rx * rx, dexp2(-9.28f * ndv)) * rx + ry;
    return mk2(-1.04f * a004 + rz, 1.04f * a004 + rw);
}

struct UpscaledGI {
    float sh[4], cocg[2], ao, shadow, spec[4];
};

// SpatiallyUpscaleBuffers (ColorPassFrag.glsl:535-653), which the colour pass
// always runs (:828): a 3x3 joint-bilateral gather of the GI planes with the
// a-trous kernel, depth weight exp(-2|dd|)^5.25 and normal weight
// max(n.n', 1e-6)^16; beyond 128 units the sun shadow is filtered over the
// centre and its four immediate neighbours, otherwise read at the pixel; then
// +0.05 shadow bias (:641-643). Taps are one GI texel apart (TexelSize of
// u_DiffuseSHy, :565): on a GI grid d times coarser (kScaled) they land on
// G-buffer texel centres d texels apart (fetched, REPEAT wrapped: the shader
// has no screen-space test here) and between GI texels (bilinear); with d = 1
// every tap is a texel centre of both. With a reflection pass (kSpec) the
// specular indirect is gathered too, weighted by the GI weight /
// (12 |roughness - base roughness| + 1) * max(n.n', 0)^8 (:595-603; the
// G-buffer roughness and normal are the block's and the face's). All loads of
// a tap are issued before its weights are formed; taps in x-outer, y-inner
// order keep the sums' rounding identical to the shader's loop. With block
// textures (kTex) the specular gather reads the tap's roughness and
// normal-mapped normal from the textured G-buffer (u_GBufferPBR,
// u_GBufferNormals, :596-599) and compares with the base pixel's (base_hf).
// The GI planes and G-buffer around a 32 x 8 block of the colour pass on the
// GI's own grid (halo 1, REPEAT-wrapped as the taps are): per texel the SH;
// CoCg, AO and the depth as the taps use it, 1 / (1 / t); face | shadow << 8.
constexpr int kShadeTW = 34, kShadeTH = 10, kShadeN = kShadeTW * kShadeTH;
struct ShadeTile {
    const float4* A;
    const float4* B;
    const int* C;
    int lx, ly;   // this pixel's tile position
};

template <typename S, bool kScaled, bool kSpec, bool kTex>
__device__ __forceinline__ UpscaledGI upscale_gi(const WorldView& w, int W, int H, int d, int i, int j, v2 uv,
                                                 const S* t, const uint8_t* face, const uint8_t* block,
                                                 const uint8_t* shadow, const S* sh_p, const S* cocg_p,
                                                 const S* ao_p, const S* spec_p, int base_face, float base_d,
                                                 float base_rough, const S* gb_normal, const S* gb_pbr, v3 base_hf,
                                                 const ShadeTile* tile) {
    constexpr bool kTile = !kScaled && !kSpec;
    UpscaledGI u;
    // the normal weights for a clamped dot product of the decoded face
    // normals of 0, 1 or 3 (face_cos): max(n.n', 1e-6)^16 floored at 1e-4,
    // and max(n.n', 0)^8 for the specular gather
    const float nw0 = fmaxf(dpow(0.000001f, 16.0f), 0.0001f), nw1 = fmaxf(dpow(1.0f, 16.0f), 0.0001f),
                nw3 = fmaxf(dpow(3.0f, 16.0f), 0.0001f);
    const float sw1 = dpow(1.0f, 8.0f), sw3 = dpow(3.0f, 8.0f);
    float4 tsh = make_float4(0.0f, 0.0f, 0.0f, 0.0f), tsp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float tcc0 = 0.0f, tcc1 = 0.0f, tao = 0.0f, tw = 0.0f, tsw = 0.0f, tspw = 0.0f;
    const bool filter_shadows = base_d > 128.0f;
    float tshadow = filter_shadows ? 0.0f : (float)__ldg(shadow + (size_t)j * W + i);
    const int Wg = W / d, Hg = H / d;
    const float texel_x = 1.0f / (float)Wg, texel_y = 1.0f / (float)Hg;
    const bool inner = i >= d && j >= d && i < W - d && j < H - d;
    // rolled: the nine unrolled taps (each with its exponential and power)
    // overflow the instruction cache
#pragma unroll 1
    for (int x = -1; x <= 1; x++) {
        const int si = inner ? i + d * x : wrapi(i + d * x, W);
#pragma unroll 1
        for (int y = -1; y <= 1; y++) {
            const int sj = inner ? j + d * y : wrapi(j + d * y, H);
            const size_t q = (size_t)sj * W + si;
            float4 s4, sp4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            float2 c2;
            float a0, lda, sv;
            int fid;
            const bool cross = x == 0 || y == 0;
            if (kTile) {
                const int k = (tile->ly + y) * kShadeTW + tile->lx + x;
                s4 = tile->A[k];
                const float4 b = tile->B[k];
                const int c = tile->C[k];
                c2 = make_float2(b.x, b.y);
                a0 = b.z;
                lda = b.w;
                fid = c & 255;
                sv = (filter_shadows && cross) ? (float)(c >> 8) : 0.0f;
            } else {
                lda = 1.0f / (1.0f / ld(t + q));
                fid = __ldg(face + q);
                sv = (filter_shadows && cross) ? (float)__ldg(shadow + q) : 0.0f;
            }
            if (kTile) {
            } else if (kScaled) {
                const Bilin fg = bilin(mk2(uv.x + (float)x * texel_x, uv.y + (float)y * texel_y), Wg, Hg);
                s4 = bl4(sh_p, fg);
                c2 = bl2(cocg_p, fg);
                a0 = bl2(ao_p, fg).x;
                if (kSpec) sp4 = bl4(spec_p, fg);
            } else {
                s4 = ld4(sh_p + q * 4);
                c2 = ld2(cocg_p + q * 2);
                a0 = ld(ao_p + q * 2);
                if (kSpec) sp4 = ld4(spec_p + q * 4);
            }
            const int tap_block = (kSpec && !kTex) ? (int)__ldg(block + q) : 0;
            const float ed = dexp(-(fabsf(lda - base_d) * 2.0f));
            const float dw = dpow(ed, 5.25f);
            const int fc = face_cos(base_face, fid);
            const float nw = fc == 0 ? nw0 : (fc == 1 ? nw1 : nw3);
            const float kwt = (x == 0 ? 1.0f : 2.0f / 3.0f) * (y == 0 ? 1.0f : 2.0f / 3.0f);   // AtrousWeights
            float wgt = clampf((nw * dw) * kwt, 0.0f, 1.0f);
            if (kSpec) {
                float ra, nsp;
                if (kTex) {
                    ra = ld(gb_pbr + q * 4);
                    const v3 hf = mk3(ld(gb_normal + q * 3), ld(gb_normal + q * 3 + 1), ld(gb_normal + q * 3 + 2));
                    nsp = dpow(fmaxf(dot(hf, base_hf), 0.0f), 8.0f);
                } else {
                    ra = pbr_rough(w, tap_block);
                    nsp = fc == 0 ? 0.0f : (fc == 1 ? sw1 : sw3);
                }
                float spw = (wgt / ((fabsf(ra - base_rough) * 12.0f) + 1.0f)) * nsp;
                spw = fmaxf(spw, 0.00000001f);
                tsp.x += sp4.x * spw;
                tsp.y += sp4.y * spw;
                tsp.z += sp4.z * spw;
                tsp.w += sp4.w * spw;
                tspw += spw;
            }
            wgt = fmaxf(wgt, 0.00000001f);
            tsh.x += s4.x * wgt;
            tsh.y += s4.y * wgt;
            tsh.z += s4.z * wgt;
            tsh.w += s4.w * wgt;
            tcc0 += c2.x * wgt;
            tcc1 += c2.y * wgt;
            tao += a0 * wgt;
            tw += wgt;
            if (filter_shadows && cross) {   // IsImmediateNeighbour (:524-530)
                const float swt = (kwt * clampf(dpow(ed, 32.0f), 0.00001f, 1.0f)) * (nw * nw);
                tshadow += sv * swt;
                tsw += swt;
            }
        }
    }
    tw = fmaxf(tw, 0.0000001f);
    u.sh[0] = tsh.x / tw;
    u.sh[1] = tsh.y / tw;
    u.sh[2] = tsh.z / tw;
    u.sh[3] = tsh.w / tw;
    u.cocg[0] = tcc0 / tw;
    u.cocg[1] = tcc1 / tw;
    u.ao = tao / tw;
    tspw = fmaxf(tspw, 0.0000001f);
    u.spec[0] = tsp.x / tspw;
    u.spec[1] = tsp.y / tspw;
    u.spec[2] = tsp.z / tspw;
    u.spec[3] = tsp.w / tspw;
    if (filter_shadows) tshadow = tshadow / tsw;
    tshadow += 0.05f;
    u.shadow = clampf(tshadow, 0.00000000000001f, 1.0f);
    return u;
}

// kTex: albedo, normal-mapped normal, roughness / metalness / emissivity and
// texture AO from the textured G-buffer (u_GBufferAlbedos, u_GBufferNormals,
// u_GBufferPBR, u_GBufferAO, :797-803) instead of the block table and the
// face normal; the face normal stays where the shader reads u_NormalTexture.
template <typename S, bool kScaled, bool kSpec, bool kTex>
__global__ void __launch_bounds__(256, 4) k_shade(WorldView w, CamView cam, int W, int H, ShadeArgs a, const S* t,
                                               const uint8_t* face, const uint8_t* block, const uint8_t* shadow,
                                               const S* sh_p, const S* cocg_p, const S* ao_p, const S* spec_p,
                                               S* rgb) {
    constexpr bool kTile = !kScaled && !kSpec;
    __shared__ float4 s_ta[kTile ? kShadeN : 1], s_tb[kTile ? kShadeN : 1];
    __shared__ int s_tc[kTile ? kShadeN : 1];
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (kTile) {   // the 3x3 gather's texels, loaded once per block (GI grid = G-buffer grid)
        for (int q = threadIdx.y * 32 + threadIdx.x; q < kShadeN; q += 256) {
            const int ly = q / kShadeTW, lx = q - ly * kShadeTW;
            const int gi = wrapi((int)blockIdx.x * 32 - 1 + lx, W), gj = wrapi((int)blockIdx.y * 8 - 1 + ly, H);
            const size_t g = (size_t)gj * W + gi;
            const float4 sh = ld4(sh_p + 4 * g);
            const float2 cc = ld2(cocg_p + 2 * g);
            s_ta[q] = sh;
            s_tb[q] = make_float4(cc.x, cc.y, ld(ao_p + 2 * g), 1.0f / (1.0f / ld(t + g)));
            s_tc[q] = (int)__ldg(face + g) | ((int)__ldg(shadow + g) << 8);
        }
        __syncthreads();
    }
    if (i >= W || j >= H) return;
    const ShadeTile tile{s_ta, s_tb, s_tc, (int)threadIdx.x + 1, (int)threadIdx.y + 1};
    size_t px = (size_t)j * W + i;
    const v3 viewer = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    v2 uv = texcoord(i, j, W, H);
    v3 dir = normalize(ray_dir_at(cam, uv));
    // SamplePositionAt (:1122-1126) reads 1/t from the R32F depth plane
    float dist = 1.0f / (1.0f / ld(t + px));
    v3 wp = add(ray_origin(cam), muls(dir, dist));
    v3 n = normal_from_id(__ldg(face + px), 1.0f);
    v3 color;
    if (dist > 0.0f) {
        int bid = min(max((int)__ldg(block + px), 0), 127);
        const Material m = material(w, bid);
        v3 base_albedo = m.albedo, nh = n;
        float rough = m.rough, metal = m.metal, emissivity = (float)m.emissive, tex_ao = 1.0f;
        const S* gb_normal = (const S*)a.gb_normal;
        const S* gb_pbr = (const S*)a.gb_pbr;
        if (kTex) {
            const S* ga = (const S*)a.gb_albedo;
            base_albedo = mk3(ld(ga + px * 3), ld(ga + px * 3 + 1), ld(ga + px * 3 + 2));
            nh = mk3(ld(gb_normal + px * 3), ld(gb_normal + px * 3 + 1), ld(gb_normal + px * 3 + 2));
            rough = ld(gb_pbr + px * 4);
            metal = ld(gb_pbr + px * 4 + 1);
            emissivity = ld(gb_pbr + px * 4 + 3);
            tex_ao = ld((const S*)a.gb_ao + px);
        }
        v3 albedo = basic_saturation(base_albedo, 1.0f - 0.1f);
        if (metal >= 0.1f - 0.01f) albedo = basic_saturation(albedo, 0.9f);
        const UpscaledGI up = upscale_gi<S, kScaled, kSpec, kTex>(w, W, H, a.gi_div, i, j, uv, t, face, block,
                                                                  shadow, sh_p, cocg_p, ao_p, spec_p,
                                                                  (int)__ldg(face + px), dist, rough, gb_normal,
                                                                  gb_pbr, nh, &tile);
        float up_shadow = clampf(up.shadow, 0.0f, 1.0f);
        float rt_shadow = clampf(clampf(up_shadow + 0.0f, 0.0f, 1.0f), 0.0f, 1.0f);
        v3 indirect = sh_to_irradiance(up.sh, up.cocg, nh);   // IndirectN = NormalMapped (:834-840)
        const float vb = 0.00125f;
        if (a.vxao && uv.x > vb && uv.x < 1.0f - vb && uv.y > vb && uv.y < 1.0f - vb) {
            float ao = up.ao;
            float dxz = sqrtf((wp.x - viewer.x) * (wp.x - viewer.x) + (wp.z - viewer.z) * (wp.z - viewer.z));
            float fade = dxz < 256.0f ? 0.0f : 1.0f;
            ao = mixf(ao, 1.0f, fade);
            ao = dpow(ao, 2.2f);
            indirect = muls(indirect, clampf(ao, 0.05f, 1.0f));
        }
        float sampled_ao = dpow(tex_ao, 1.25f);
        v3 sun = mk3(a.sun[0], a.sun[1], a.sun[2]);
        v3 moon = mk3(a.moon[0], a.moon[1], a.moon[2]);
        v3 sun_color = mk3(a.sun_color[0], a.sun_color[1], a.sun_color[2]);
        v3 moon_color = mk3(a.moon_color[0], a.moon_color[1], a.moon_color[2]);
        v3 sun_direct = directional_light(viewer, wp, sun, sun_color, sun_color, albedo, nh, rough, metal, rt_shadow);
        v3 moon_direct = directional_light(viewer, wp, moon, moon_color, moon_color, albedo, nh, rough, metal, rt_shadow);
        v3 direct = vmixv(sun_direct, moon_direct, mk3(a.sun_vis * 1.0f, a.sun_vis * 1.0f, a.sun_vis * 1.0f));
        direct = muls(direct, (!(emissivity > 0.05f)) ? 1.0f : 0.0f);
        direct = vmax(direct, 0.000001f);
        v3 diffuse_indirect = mul(indirect, albedo);
        v3 I = normalize(sub(wp, viewer));
        float idn = dot(nh, I);
        v3 R = sub(I, muls(nh, 2.0f * idn));
        // SpecularIndirect (:901-909): the upscaled reflection times
        // clamp(max(n.n, 1e-8)^2 * 1.5, 0.1, 1) inside the 0.0035 border
        v3 spec_ind = mk3(0.0f, 0.0f, 0.0f);
        const float sb = 0.0035f;
        if (kSpec && uv.x > sb && uv.x < 1.0f - sb && uv.y > sb && uv.y < 1.0f - sb) {
            const float att = clampf(dpow(fmaxf(dot(n, nh), 0.00000001f), 2.0f) * 1.5f, 0.1f, 1.0f);
            spec_ind = muls(mk3(up.spec[0], up.spec[1], up.spec[2]), att);
        }
        spec_ind = vmax(spec_ind, 0.0001f);
        v3 Lo = normalize(sub(viewer, wp));
        v3 F0 = vmix(mk3(0.04f, 0.04f, 0.04f), albedo, metal);
        diffuse_indirect = muls(diffuse_indirect, clampf(sampled_ao, 0.2f, 1.01f));
        float nov = clampf(dot(nh, Lo), 0.0000000001f, 1.0f);
        // ComputeSpecularAO (:742-745) of the texture AO (1 without textures)
        float spec_ao = clampf(dpow(nov + tex_ao, dexp2(-16.0f * rough - 1.0f)) - 1.0f + tex_ao, 0.0f, 1.0f);
        spec_ao = dpow(spec_ao, 1.5f);
        float horizon = fminf(1.0f + dot(R, nh), 1.0f);
        horizon = (horizon * horizon) * horizon;
        if (metal >= 0.1f) spec_ind = muls(spec_ind, 1.3f);
        spec_ind = muls(spec_ind, spec_ao);
        spec_ind = muls(spec_ind, horizon);
        v3 F = vclamp(fresnel_schlick_roughness(Lo, nh, F0, rough), 0.0f, 1.0f);
        v3 kD = sub(mk3(1.0f, 1.0f, 1.0f), F);
        kD = muls(kD, 1.0f - metal);
        float ex = clampf(fmaxf(dot(neg(I), nh), 0.000001f), 0.0f, 1.0f);
        float ey = clampf(rough, 0.0f, 1.0f);
        v2 env = karis_env_brdf(ex, ey);
        v3 ind_spec = mul(spec_ind, mk3(F.x * env.x + env.y, F.y * env.x + env.y, F.z * env.x + env.y));
        v3 indirect_light = add(mul(kD, diffuse_indirect), ind_spec);
        color = add(direct, indirect_light);
    } else {
        color = sky_radiance(dir);
    }
    color = vmax(color, 0.000001f);
    st(rgb + px * 3 + 0, color.x);
    st(rgb + px * 3 + 1, color.y);
    st(rgb + px * 3 + 2, color.z);
}

template <typename S>
void launch_shade(bool scaled, bool sp, bool tx, dim3 grid, dim3 blk, cudaStream_t s, const WorldView& w,
                  const CamView& cam, int W, int H, const ShadeArgs& a, const void* t, const uint8_t* face,
                  const uint8_t* block, const uint8_t* shadow, const void* sh, const void* cocg, const void* aosky,
                  const void* spec, void* rgb) {
    using K = void (*)(WorldView, CamView, int, int, ShadeArgs, const S*, const uint8_t*, const uint8_t*,
                       const uint8_t*, const S*, const S*, const S*, const S*, S*);
    const K table[8] = {k_shade<S, false, false, false>, k_shade<S, false, false, true>, k_shade<S, false, true, false>,
                        k_shade<S, false, true, true>,   k_shade<S, true, false, false>,  k_shade<S, true, false, true>,
                        k_shade<S, true, true, false>,   k_shade<S, true, true, true>};
    const K k = table[(scaled ? 4 : 0) + (sp ? 2 : 0) + (tx ? 1 : 0)];
    pdl_launch(k, grid, blk, 0, s, w, cam, W, H, a, (const S*)t, face, block, shadow, (const S*)sh, (const S*)cocg,
               (const S*)aosky, (const S*)spec, (S*)rgb);
}

}  // namespace

cudaError_t shade(const WorldView& w, const CamView& cam, int W, int H, int fp16, const ShadeArgs& a,
                  const void* t, const uint8_t* face, const uint8_t* block, const uint8_t* shadow,
                  const void* sh, const void* cocg, const void* aosky, const void* spec, void* rgb, cudaStream_t s) {
    dim3 grid((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8));
    dim3 blk(32, 8);
    const bool scaled = a.gi_div > 1, sp = spec != nullptr, tx = a.gb_albedo != nullptr;
    if (fp16) {
        launch_shade<__half>(scaled, sp, tx, grid, blk, s, w, cam, W, H, a, t, face, block, shadow, sh, cocg, aosky, spec,
                             rgb);
    } else {
        launch_shade<float>(scaled, sp, tx, grid, blk, s, w, cam, W, H, a, t, face, block, shadow, sh, cocg, aosky, spec,
                            rgb);
    }
    return cudaGetLastError();
}

namespace {
__global__ void k_detmath(int op, const float* x, const float* y, float* out, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float a = x[k];
    float r;
    switch (op) {
        case 0: r = dexp(a); break;
        case 1: r = dexp2(a); break;
        case 2: r = dlog2(a); break;
        case 3: r = dpow(a, y[k]); break;
        case 4: r = dsin(a); break;
        case 5: r = dcos(a); break;
        // packed pairs, each lane against its scalar operation
        case 6: r = pmul(make_float2(a, y[k]), make_float2(y[k], a)).x; break;
        case 7: r = pmul(make_float2(y[k], a), make_float2(a, y[k])).y; break;
        case 8: r = padd(make_float2(a, y[k]), make_float2(y[k], a)).x; break;
        case 9: r = padd(make_float2(y[k], a), make_float2(a, y[k])).y; break;
        case 10: r = dexp_pair(a, y[k]).x; break;
        case 11: r = dexp_pair(y[k], a).y; break;
        case 12: r = pacc(make_float2(y[k], a), make_float2(a, y[k]), a).y; break;   // a + y * a
        case 15: r = div5(a); break;
        case 16: r = dexp_pair_np(a, y[k]).x; break;
        case 17: r = dexp_pair_np(y[k], a).y; break;
        default: {   // bilinear blend of (a, 2a, -a, y) at weights (frac(y), frac(2y))
            Bilin b;
            b.ax = y[k] - floorf(y[k]);
            b.ay = 2.0f * y[k] - floorf(2.0f * y[k]);
            b.bx = 1.0f - b.ax;
            b.by = 1.0f - b.ay;
            const float v00 = a, v10 = 2.0f * a, v01 = -a, v11 = y[k];
            if (op != 13 && op != 14) { r = 0.0f; break; }
            r = op == 13 ? blend1(b, v00, v10, v01, v11)
                         : blend2(b, make_float2(0.0f, v00), make_float2(0.0f, v10), make_float2(0.0f, v01),
                                  make_float2(0.0f, v11)).y;
            break;
        }
    }
    out[k] = r;
}
}  // namespace

cudaError_t detmath_eval(int op, const float* x, const float* y, float* out, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_detmath<<<(n + 255) / 256, 256, 0, s>>>(op, x, y, out, n);
    return cudaGetLastError();
}

}  // namespace vpt
