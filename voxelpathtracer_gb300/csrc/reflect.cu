// Reflections: ReflectionTraceFrag.glsl main (:717-1084) on the GI grid, one
// thread per texel, each warp on an 8x4 patch so its rays stay coherent;
// then the two bilateral passes over its hit distance and
// SpecularTemporalFilter.glsl (firefly rejection, reprojection, clipping,
// accumulation). Substitutions as in the diffuse trace: flat materials
// (albedo, roughness, metalness, emissive flag of the block; AO 1; the face
// normal as the normal map), PCG random numbers instead of hash2 / blue
// noise, the analytic sky, no LPV, cloud reflections or player, no jitter.
// With DenoiseReflections the x and y passes of ReflectionDenoiserNew.glsl
// follow; the colour pass reads their output (or the temporal output).
#include "pixel_passes.cuh"

namespace vpt {

namespace {

__device__ __forceinline__ void tile_pixel(int* i, int* j) {
    int tid = threadIdx.x;
    int warp = tid >> 5, lane = tid & 31;
    *i = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    *j = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
}

// SHToIrradianceA (ReflectionTraceFrag.glsl:466-476)
__device__ __forceinline__ v3 sh_to_irradiance_a(float4 sh, float2 cc) {
    const float Y = fmaxf(0.0f, 3.544905f * sh.w);
    const float k = (Y * 0.282095f) / (sh.w + 1e-6f);
    const float co = cc.x * k, cg = cc.y * k;
    const float T = Y - cg * 0.5f;
    const float G = cg + T;
    const float B = T - co * 0.5f;
    const float R = B + co;
    return mk3(fmaxf(R, 0.0f), fmaxf(G, 0.0f), fmaxf(B, 0.0f));
}

// ImportanceSampleGGX (ReflectionTraceFrag.glsl:345-365)
__device__ __forceinline__ v3 importance_sample_ggx(v3 N, float roughness, float xi_x, float xi_y) {
    const float alpha = roughness * roughness;
    const float alpha2 = alpha * alpha;
    const float phi = (2.0f * kPI) * xi_x;
    const float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (alpha2 - 1.0f) * xi_y));
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    const v3 H = mk3(dcos(phi) * sin_t, dsin(phi) * sin_t, cos_t);
    const v3 up = fabsf(N.z) < 0.999f ? mk3(0.0f, 0.0f, 1.0f) : mk3(1.0f, 0.0f, 0.0f);
    const v3 tangent = normalize(cross(up, N));
    const v3 bitangent = cross(N, tangent);
    const v3 s = mk3((tangent.x * H.x + bitangent.x * H.y) + N.x * H.z, (tangent.y * H.x + bitangent.y * H.y) + N.y * H.z,
                     (tangent.z * H.x + bitangent.z * H.y) + N.z * H.z);
    return normalize(s);
}

// GetReflectionDirection (ReflectionTraceFrag.glsl:621-646)
__device__ __forceinline__ v3 reflection_normal(v3 N, float R, uint32_t* rng) {
    R = fmaxf(R, 0.05f);
    float nearest = -100.0f;
    v3 best = N;
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        const float xi_x = rand01(rng) * 0.9f;
        const float xi_y = rand01(rng) * 0.65f;
        const v3 h = importance_sample_ggx(N, R, xi_x, xi_y);
        const float d = dot(h, N);
        if (d > nearest) {
            best = h;
            nearest = d;
        }
    }
    return best;
}

__device__ __forceinline__ v3 reflect3(v3 I, v3 N) { return sub(I, muls(N, 2.0f * dot(N, I))); }

// CalculateDirectionalLight of the reflection trace (:313-336): the specular
// radiance is scaled by 0, only the diffuse lobe remains.
__device__ __forceinline__ v3 reflection_directional_light(v3 viewer, v3 wp, v3 light_dir, v3 radiance, v3 albedo,
                                                           v3 n, float rough, float metal, float shadow) {
    const float Epsilon = 0.00001f;
    const float sh = fminf(shadow, 1.0f);
    const v3 Lo = normalize(sub(viewer, wp));
    const float cos_lo = fmaxf(0.0f, dot(n, Lo));
    const v3 F0 = vmix(mk3(0.04f, 0.04f, 0.04f), albedo, metal);
    const v3 Li = light_dir;
    const v3 Lh = normalize(add(Li, Lo));
    const float cos_li = fmaxf(0.0f, dot(n, Li));
    const float cos_lh = fmaxf(0.0f, dot(n, Lh));
    const float fk = dpow(1.0f - fmaxf(0.0f, dot(Lh, Lo)), 5.0f);
    const v3 F = add(F0, muls(sub(mk3(1.0f, 1.0f, 1.0f), F0), fk));
    const float alpha = rough * rough;
    const float alpha_sq = alpha * alpha;
    const float denom = (cos_lh * cos_lh) * (alpha_sq - 1.0f) + 1.0f;
    const float D = alpha_sq / ((kPI * denom) * denom);
    const float r1 = rough + 1.0f;
    const float k = (r1 * r1) / 8.0f;
    const float G = (cos_li / (cos_li * (1.0f - k) + k)) * (cos_lo / (cos_lo * (1.0f - k) + k));
    const v3 kd = vmix(sub(mk3(1.0f, 1.0f, 1.0f), F), mk3(0.0f, 0.0f, 0.0f), metal);
    const v3 diffuse_brdf = mul(kd, albedo);
    const v3 spec_brdf = divs(muls(muls(F, D), G), fmaxf(Epsilon, (4.0f * cos_li) * cos_lo));
    const v3 radiance_s = muls(muls(radiance, 0.05f), 0.0f);
    const v3 result = add(muls(mul(diffuse_brdf, radiance), cos_li), muls(mul(spec_brdf, radiance_s), cos_li));
    return muls(vmax(result, 0.0f), clampf(1.0f - sh, 0.0f, 1.0f));
}

// The face UV of CalculateVectors (:1388-1446), UV.y = 1 - UV.y (:848).
// the textured G-buffer read as its GL samplers would: PBR nearest,
// normal-mapped normal bilinear (REPEAT), on the W x H plane at uv
template <typename S>
__device__ __forceinline__ float gb_pbr_at(const S* p, int W, int H, v2 uv, int c) {
    const int x = wrapi(f2i_floor(uv.x * (float)W), W), y = wrapi(f2i_floor(uv.y * (float)H), H);
    return ld(p + ((size_t)y * W + x) * 4 + c);
}
template <typename S>
__device__ __forceinline__ v3 gb_normal_at(const S* p, int W, int H, v2 uv) {
    const Plane<S, 3> P{p, W, H};
    float n[3];
    P.linear(uv, n);
    return mk3(n[0], n[1], n[2]);
}

__device__ __forceinline__ v2 face_uv(v3 p, v3 n) {
    v2 uv;
    if (n.z != 0.0f) uv = mk2(fract(p.x), fract(p.y));
    else if (n.y != 0.0f) uv = mk2(fract(p.x), fract(p.z));
    else uv = mk2(fract(p.z), fract(p.y));
    uv.y = 1.0f - uv.y;
    return uv;
}

// texture() of the 0/1 sun-shadow plane as UNORM8 with GL_LINEAR + GL_REPEAT.
__device__ __forceinline__ float bl_u8(const uint8_t* p, const Bilin& b) {
    return blend(b, (float)__ldg(p + b.o00), (float)__ldg(p + b.o10), (float)__ldg(p + b.o01),
                 (float)__ldg(p + b.o11));
}

template <typename S>
__global__ void __launch_bounds__(256, 8) k_trace_reflection(WorldView w, CamView cam, int W, int H, int Wg, int Hg,
                                                          ReflectionArgs a, const S* t, const uint8_t* face,
                                                          const uint8_t* shadow, const S* tv, const uint8_t* fv,
                                                          const uint8_t* bv, const S* den_sh, const S* den_cocg,
                                                          const S* den_ao, S* o_spec, S* o_hit, S* o_mask,
                                                          Counters* stats) {
    int i, j;
    tile_pixel(&i, &j);
    unsigned nr = 0, ns = 0, nsr = 0, nss = 0;
    if (i < Wg && j < Hg) {
        const size_t q = (size_t)j * Wg + i;
        const v2 uv = texcoord(i, j, Wg, Hg);
        const Plane<S, 1> TV{tv, Wg, Hg};
        v4 P = position_fetch(cam, TV, i, j, uv);
        if (P.w < 0.0f) {
            st4(o_spec + 4 * q, 0.0f, 0.0f, 0.0f, 0.0f);
            st(o_hit + q, -1.0f);
            st(o_mask + q, 0.0f);
        } else {
            const v3 viewer = mk3(a.viewer[0], a.viewer[1], a.viewer[2]);
            const v3 cam_pos = ray_origin(cam);
            const v3 N = normal_from_id(__ldg(fv + q), 1.0f);
            // NormalMappedInitial (:794): the linear normal G-buffer at the
            // texel centre, the face normal itself on the G-buffer's grid
            v3 NM = (W == Wg && H == Hg) ? N : gnormal_linear(face, W, H, uv);
            const Material base = material(w, min(max((int)__ldg(bv + q), 0), 127));
            float base_rough = base.rough, base_metal = base.metal;
            if (a.gb_normal) {   // the textured G-buffer (u_GBufferPBR, u_GBufferNormals, :777-789)
                const S* gn = (const S*)a.gb_normal;
                base_rough = gb_pbr_at((const S*)a.gb_pbr, W, H, uv, 0);
                base_metal = gb_pbr_at((const S*)a.gb_pbr, W, H, uv, 1);
                NM = (W == Wg && H == Hg) ? mk3(ld(gn + q * 3), ld(gn + q * 3 + 1), ld(gn + q * 3 + 2))
                                          : gb_normal_at(gn, W, H, uv);
            }
            const v3 I = normalize(sub(mk3(P.x, P.y, P.z), viewer));
            P.x += N.x * 0.035f;
            P.y += N.y * 0.035f;
            P.z += N.z * 0.035f;
            const v3 pos = mk3(P.x, P.y, P.z);
            const v3 base_indirect = sh_to_irradiance_a(ld4(den_sh + 4 * q), ld2(den_cocg + 2 * q));
            const v3 light_dir = mk3(a.light_dir[0], a.light_dir[1], a.light_dir[2]);
            const v3 radiance = muls(mk3(a.mixed[0], a.mixed[1], a.mixed[2]), 0.6f);
            const Plane<S, 1> T{t, W, H};
            const Plane8 F{face, W, H};
            uint32_t rng = pcg_hash(pcg_hash((uint32_t)q + pcg_hash(a.frame_index + pcg_hash(a.seed))) ^ 0x5245464Cu);
            const int spp = min(max(a.spp, 1), 16);
            const float rbias = 0.85f;
            float total[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            float avg_hit = 0.001f, meaningful = 0.0f, emask = 0.0f, computed_shadow = 0.0f;
            int shadow_itr = 0, total_hits = 0;
#pragma unroll 1
            for (int s = 0; s < spp; s++) {
                const v3 rn = reflection_normal(NM, clampf(base_rough * rbias, 0.01f, 1.0f), &rng);
                const v3 R = reflect3(I, rn);
                const TraceResult tr = traverse<0>(w, pos, R, a.max_steps);
                nr += 1;
                ns += (unsigned)tr.steps;
                const float Tt = tr.t;
                const v3 hp = add(pos, muls(R, Tt));
                v3 computed;
                if (Tt > 0.0f) {
                    const v3 hn = tr.normal;
                    const int rid = min(max(tr.block, 0), 127);
                    const v4 pr = mat_mul4(a.view_proj, hp.x, hp.y, hp.z, 1.0f);
                    const v2 rc = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
                    const v4 pa = position_linear(cam, T, rc);
                    const v3 na = normal_from_id(F.nearest(rc), 1.0f);
                    const v3 pd = mk3(fabsf(pa.x - hp.x), fabsf(pa.y - hp.y), fabsf(pa.z - hp.z));
                    const float err = dot(pd, pd);
                    const float tb = 0.032593f;
                    const bool in_ss = rc.x > tb && rc.x < 1.0f - tb && rc.y > tb && rc.y < 1.0f - tb;
                    const bool success = err < 0.095f && na.x == hn.x && na.y == hn.y && na.z == hn.z && in_ss;
                    v3 ambient = base_indirect;
                    if (success) {
                        const Bilin fg = bilin(rc, Wg, Hg);
                        ambient = sh_to_irradiance_a(bl4(den_sh, fg), bl2(den_cocg, fg));
                        const float vxao = dpow(bl2(den_ao, fg).x, 0.75f);
                        if (pa.w > 0.0f && length(sub(mk3(pa.x, pa.y, pa.z), cam_pos)) < 40.0f)
                            ambient = muls(ambient, vxao);
                    }
                    Material m = material(w, rid);
                    float ao = dpow(1.0f, 2.0f);
                    v3 nmap = hn;
                    float emis_tex = -1.0f;   // the emissive texel, -1: none
                    if (a.textured) {
                        // the hit's textures (:887-960): ids with the grass override,
                        // albedo and PBR by texture() (taken at level 0), the normal
                        // map at level 3 through the face's tangent basis, the
                        // emissive texture at level 2
                        const BlockTexView& tx = a.tex;
                        const int f = normal_id(hn);
                        int ia = __ldg(tx.ids + rid), in_ = __ldg(tx.ids + 128 + rid), ip = __ldg(tx.ids + 256 + rid);
                        const int ie = tx.emissive.texels ? __ldg(tx.ids + 384 + rid) : -1;
                        if (rid == tx.grass[0]) {
                            const int k = f == 2 ? 1 : (f == 3 ? 7 : 4);
                            ia = tx.grass[k];
                            in_ = tx.grass[k + 1];
                            ip = tx.grass[k + 2];
                        }
                        const v2 fuv = face_uv(hp, hn);
                        float alb[4], pb[4], nm[4];
                        sample_level(tx.albedo, ia, fuv.x, fuv.y, 0, 3, tx.srgb, alb);
                        sample_level(tx.pbr, ip, fuv.x, fuv.y, 0, 4, tx.unorm, pb);
                        sample_level(tx.normal, in_, fuv.x, fuv.y, 3, 3, tx.unorm, nm);
                        m.albedo = mk3(alb[0], alb[1], alb[2]);
                        m.rough = pb[0];
                        m.metal = pb[1];
                        ao = dpow(pb[3], 2.0f);
                        for (int c = 0; c < 3; c++) nm[c] = nm[c] * 2.0f - 1.0f;
                        const v3 Tt = f < 4 ? mk3(1.0f, 0.0f, 0.0f) : mk3(0.0f, 0.0f, -1.0f);
                        const v3 Bt = f < 2 ? mk3(0.0f, 1.0f, 0.0f) : (f < 4 ? mk3(0.0f, 0.0f, 1.0f) : mk3(0.0f, -1.0f, 0.0f));
                        nmap = mk3((Tt.x * nm[0] + Bt.x * nm[1]) + hn.x * nm[2], (Tt.y * nm[0] + Bt.y * nm[1]) + hn.y * nm[2],
                                   (Tt.z * nm[0] + Bt.z * nm[1]) + hn.z * nm[2]);
                        if (ie > -1) {
                            float e[4];
                            sample_level(tx.emissive, ie, fuv.x, fuv.y, 2, 1, tx.unorm, e);
                            emis_tex = e[0];
                        }
                    }
                    if (shadow_itr < max(spp / 4, 1)) {
                        if (success && in_ss) {
                            computed_shadow = bl_u8(shadow, bilin(rc, W, H));
                        } else {
                            const TraceResult sr = traverse<0>(w, add(hp, muls(hn, 0.055f)), light_dir,
                                                               a.shadow_max_steps);
                            nsr += 1;
                            nss += (unsigned)sr.steps;
                            computed_shadow = sr.t > 0.0f ? 1.0f : 0.0f;
                        }
                        shadow_itr++;
                    }
                    ambient = mul(muls(muls(ambient, 1.0f), clampf(ao, 0.1f, 1.0f)), m.albedo);
                    v3 direct = add(ambient, reflection_directional_light(viewer, hp, light_dir, radiance, m.albedo,
                                                                          nmap, m.rough, m.metal, computed_shadow));
                    if (a.textured ? emis_tex > 0.1f : m.emissive != 0) {
                        float emissivity = a.textured ? emis_tex : 1.0f;
                        const v2 fuv = face_uv(hp, hn);
                        const float bx = 0.02501f, by = 0.03001f;
                        emissivity *= (fuv.x > bx && fuv.x < 1.0f - bx && fuv.y > by && fuv.y < 1.0f - by) ? 1.0f
                                                                                                          : 0.0f;
                        direct = muls(m.albedo, fmaxf(emissivity * 19.0f * 1.0f, 2.0f));
                        emask = 1.0f;
                    }
                    computed = direct;
                    avg_hit += Tt;
                    meaningful += 1.0f;
                } else {
                    computed = muls(sky_radiance(normalize(R)), mixf(1.0f, 1.175f, base_metal > 0.05f ? 1.0f : 0.0f));
                }
                total[0] += computed.x;
                total[1] += computed.y;
                total[2] += computed.z;
                total[3] += 1.0f;
                total_hits++;
            }
            avg_hit /= fmaxf(meaningful, 0.01f);
            const float nh = (float)total_hits;
            st4(o_spec + 4 * q, clampf(total[0] / nh, 0.0000001f, 100.0f), clampf(total[1] / nh, 0.0000001f, 100.0f),
                clampf(total[2] / nh, 0.0000001f, 100.0f), clampf(total[3] / nh, 0.0000001f, 100.0f));
            st(o_hit + q, clampf(meaningful > 0.01f ? avg_hit : -1.0f, -10.0f, 200.0f));
            st(o_mask + q, clampf(emask, 0.0f, 1.0f));
        }
    }
    if (stats) {
        count_rays(stats, kRayReflection, nr, ns);
        count_rays(stats, kRayReflectionShadow, nsr, nss);
    }
}

// BlurHitDistance_Bilateral.glsl (pass 1, 3x3) and
// BlurHitDistancePass2_Bilateral.glsl (pass 2, 3 x 5 taps), two GI texels
// apart, REPEAT wrap; depth and face from the GI-grid views.
template <typename S>
__global__ void __launch_bounds__(256) k_spec_hit_blur(int Wg, int Hg, int pass, const S* tv, const uint8_t* fv,
                                                       const S* hin, S* hout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Wg || j >= Hg) return;
    const size_t q = (size_t)j * Wg + i;
    const float bd = ld(tv + q), bh = ld(hin + q);
    const int bf = __ldg(fv + q);
    const int ry = pass == 2 ? 2 : 1;
    float tw = 1.0f, td = bh;
    for (int x = -1; x <= 1; x++) {
        const int si = wrapi(i + 2 * x, Wg);
        for (int y = -ry; y <= ry; y++) {
            if (x == 0 && y == 0) continue;
            const size_t n = (size_t)wrapi(j + 2 * y, Hg) * Wg + si;
            const float e = fabsf(ld(tv + n) - bd);
            const float ha = ld(hin + n);
            if (e > 1.0f || ha < 0.0f || (int)__ldg(fv + n) != bf) continue;
            const float wx = x == 0 ? 1.0f : 2.0f / 3.0f;
            const float wy = y == 0 ? 1.0f : ((y == 1 || y == -1) ? 2.0f / 3.0f : 1.0f / 6.0f);
            const float wgt = wx * wy;
            td += ha * wgt;
            tw += wgt;
        }
    }
    st(hout + q, td / fmaxf(tw, 0.001f));
}

// ClipToAABB (SpecularTemporalFilter.glsl:146-156)
__device__ __forceinline__ v3 clip_to_aabb(v3 prev, v3 mn, v3 mx) {
    const v3 pc = muls(add(mx, mn), 0.5f);
    const v3 ec = muls(sub(mx, mn), 0.5f);
    const v3 vc = sub(prev, pc);
    const v3 vu = mk3(vc.x / ec.x, vc.y / ec.y, vc.z / ec.z);
    const float denom = fmaxf(fabsf(vu.x), fmaxf(fabsf(vu.y), fabsf(vu.z)));
    return denom > 1.0f ? add(pc, divs(vc, denom)) : prev;
}

__device__ __forceinline__ float dist_sq(v3 a, v3 b) {
    const v3 c = sub(a, b);
    return dot(c, c);
}

// SpecularTemporalFilter.glsl main (:316-510) with USE_NEW_REPROJECTION,
// u_SmartClip, u_RoughnessWeight, u_TemporallyStabializeHitDistance and
// aggressive firefly rejection on (Core/Pipeline.cpp:3226-3262); with
// TEMPORAL_SPEC off the output is the firefly-rejected current colour.
template <typename S>
__global__ void __launch_bounds__(256, 6) k_spec_temporal(WorldView w, CamView cam, SpecTemporalArgs a, int W, int H,
                                                       int Wg, int Hg, const S* tv, const uint8_t* fv,
                                                       const uint8_t* bv, const S* prev_t, const uint8_t* prev_face,
                                                       const S* spec, const S* hit, const S* mask, const S* prev_out,
                                                       const S* prev_hit, const S* prev_stable, S* out, S* acc,
                                                       S* stable) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Wg || j >= Hg) return;
    const size_t q = (size_t)j * Wg + i;
    const v2 uv = texcoord(i, j, Wg, Hg);
    const Plane<S, 1> TV{tv, Wg, Hg};
    const v4 P = position_fetch(cam, TV, i, j, uv);
    const v3 n0 = normal_from_id(__ldg(fv + q), 1.0f);
    const float4 c0 = ld4(spec + 4 * q);
    float cc[4] = {c0.x, c0.y, c0.z, c0.w};
    float o_acc = 0.0f;
    const float hc = ld(hit + q);
    float o_col[4], o_stable;
    if (ld(mask + q) > 0.05f) {
        const int ox[4] = {1, 0, -1, 0}, oy[4] = {0, 1, 0, -1};
        float a4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        int unlit = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const size_t n = (size_t)wrapi(j + oy[k], Hg) * Wg + wrapi(i + ox[k], Wg);
            if (ld(mask + n) < 0.01f) {
                const float4 c = ld4(spec + 4 * n);
                a4[0] += c.x;
                a4[1] += c.y;
                a4[2] += c.z;
                a4[3] += c.w;
                unlit++;
            }
        }
        if (unlit >= 3)
            for (int c = 0; c < 4; c++) cc[c] = a4[c] / (float)unlit;
    }
    if (P.w > 0.0f && a.temporal) {
        const bool sky = hc < 0.0f;
        const Material mt = material(w, min(max((int)__ldg(bv + q), 0), 127));
        const float pr = a.gb_pbr ? gb_pbr_at((const S*)a.gb_pbr, W, H, uv, 0) : mt.rough;
        const float rough = mixf(0.095f, pr, 1.0f), metal = a.gb_pbr ? gb_pbr_at((const S*)a.gb_pbr, W, H, uv, 1) : mt.metal;
        const v3 cur_pos = mk3(a.cur_pos[0], a.cur_pos[1], a.cur_pos[2]);
        const v3 prev_pos = mk3(a.prev_pos[0], a.prev_pos[1], a.prev_pos[2]);
        const v3 ro = ray_origin(cam);
        const v3 p3 = mk3(P.x, P.y, P.z);
        bool less_valid = false;
        v2 rep = mk2(0.0f, 0.0f);
        if (hc > 0.0f && !sky && rough <= 0.875f + 0.01f) {
            const v3 I = normalize(sub(ro, p3));
            const v3 rp = sub(p3, muls(I, hc));
            const v4 pr = mat_mul4(a.prev_view_proj, rp.x, rp.y, rp.z, 1.0f);
            rep = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
            const float pt = bl1(prev_hit, bilin(rep, Wg, Hg));
            if (fabsf(pt - hc) >= 3.8f) less_valid = true;
        } else if (!sky) {
            const v3 off = muls(sub(cur_pos, prev_pos), 0.6f);
            const v3 wp = sub(p3, off);
            const v4 pr = mat_mul4(a.prev_view_proj, wp.x, wp.y, wp.z, 1.0f);
            rep = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
        }
        if (sky) {
            const v3 I = normalize(sub(ro, p3));
            const v3 rp = sub(p3, muls(I, 64.0f));
            const v4 pr = mat_mul4(a.prev_view_proj, rp.x, rp.y, rp.z, 1.0f);
            rep = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
        }
        const Plane<S, 1> PT{prev_t, W, H};
        const Plane8 PF{prev_face, W, H};
        const v4 pp = position_linear(cam, PT, rep);
        const float d = fabsf(length(sub(mk3(pp.x, pp.y, pp.z), p3)));
        const float rb = 0.01f;
        const v3 pn = normal_from_id(PF.nearest(rep), 1.0f);
        if (rep.x > 0.0f + rb && rep.x < 1.0f - rb && rep.y > 0.0f + rb && rep.y < 1.0f - rb && d < 1.0f &&
            pn.x == n0.x && pn.y == n0.y && pn.z == n0.z) {
            const Bilin fg = bilin(rep, Wg, Hg);
            const float4 p4 = bl4(prev_out, fg);
            float pc[4] = {p4.x, p4.y, p4.z, p4.w};
            const v3 base_prev = mk3(pc[0], pc[1], pc[2]);
            const bool moved = dist_sq(cur_pos, prev_pos) > 0.0001f;
            if (rough < 0.5f + 0.01f && moved) {
                // ReflectionClipping (:163-243) around this texel
                float mn[4] = {1000.0f, 1000.0f, 1000.0f, 1000.0f}, mx[4] = {-1000.0f, -1000.0f, -1000.0f, -1000.0f};
                float add_max = 0.0f;
                for (int x = -1; x <= 1; x++) {
                    const int si = wrapi(i + x, Wg);
                    for (int y = -1; y <= 1; y++) {
                        const size_t n = (size_t)wrapi(j + y, Hg) * Wg + si;
                        if (!(ld(mask + n) < 0.01f)) add_max += 0.1f;
                        const float4 sv = ld4(spec + 4 * n);
                        const float s4[4] = {sv.x, sv.y, sv.z, sv.w};
                        for (int c = 0; c < 4; c++) {
                            mn[c] = fminf(s4[c], mn[c]);
                            mx[c] = fmaxf(s4[c], mx[c]);
                        }
                    }
                }
                const v3 omn = mk3(mn[0], mn[1], mn[2]), omx = mk3(mx[0], mx[1], mx[2]);
                const float rt = 0.275f + 0.01f;
                const bool smoothish = rough < rt;
                const bool roughish = rough > rt && rough < 0.50f + 0.01f;
                if (smoothish) {
                    const float pr2 = rough * rough;
                    const float rt2 = rt * rt;
                    const float rr = 0.0f + (clampf((pr2 - 0.0f) / (rt2 - 0.0f), 0.0f, 1.0f) * (1.0f - 0.0f));
                    float bias = mixf(0.01f, 0.085f, rr);
                    if (rough > 0.235f) bias *= 1.55f;
                    for (int c = 0; c < 4; c++) {
                        mn[c] -= bias * 0.95f;
                        mx[c] += (bias * 0.95f) + add_max;
                    }
                } else if (roughish) {
                    for (int c = 0; c < 4; c++) {
                        mn[c] -= 0.37f;
                        mx[c] += 0.37f + (add_max * 1.1f);
                    }
                }
                const float imp = mixf(0.05f, 0.25f, metal > 0.05f ? 1.0f : 0.0f);
                v3 mn3 = vmix(mk3(mn[0], mn[1], mn[2]), omn, imp);
                v3 mx3 = vmix(mk3(mx[0], mx[1], mx[2]), omx, imp);
                const float bm = less_valid ? 0.5f : 0.0f;
                mn3 = vmix(mn3, omn, bm);
                mx3 = vmix(mx3, omx, bm);
                mn[0] = mn3.x; mn[1] = mn3.y; mn[2] = mn3.z;
                mx[0] = mx3.x; mx[1] = mx3.y; mx[2] = mx3.z;
                const v3 prev3 = mk3(pc[0], pc[1], pc[2]);
                const v3 cl = clip_to_aabb(prev3, mn3, mx3);
                if (!(cl.x == prev3.x && cl.y == prev3.y && cl.z == prev3.z)) {
                    if (dist_sq(cl, mn3) > dist_sq(cl, mx3))
                        for (int c = 0; c < 4; c++) pc[c] = mx[c];
                    else
                        for (int c = 0; c < 4; c++) pc[c] = mn[c];
                }
            }
            // GetAccumulationFactor (:308-313)
            const float vx = (uv.x - rep.x) * (float)Wg, vy = (uv.y - rep.y) * (float)Hg;
            float af = clampf(dexp(-sqrtf(vx * vx + vy * vy)) * 0.9f + 0.750f, 0.00000001f, 0.96f);
            af = clampf(af, 0.001f, 0.95f);
            for (int c = 0; c < 4; c++) o_col[c] = mixf(fmaxf(cc[c], 0.0f), fmaxf(pc[c], 0.0f), af);
            o_acc = af;
            o_stable = hc;
            if (dist_sq(base_prev, mk3(fmaxf(pc[0], 0.0f), fmaxf(pc[1], 0.0f), fmaxf(pc[2], 0.0f))) < 0.2f)
                o_stable = mixf(hc, bl1(prev_stable, fg), clampf(af * 1.1f, 0.0f, 0.9f));
        } else {
            for (int c = 0; c < 4; c++) o_col[c] = cc[c];
            o_acc = 0.0f;
            o_stable = hc;
        }
    } else {
        for (int c = 0; c < 4; c++) o_col[c] = cc[c];
        o_stable = hc;
    }
    if (!a.temporal) o_acc = -1.0f;
    st4(out + 4 * q, o_col[0], o_col[1], o_col[2], o_col[3]);
    st(acc + q, o_acc);
    st(stable + q, o_stable);
}

__constant__ float kGauss33[33] = {0.004013f, 0.005554f, 0.007527f, 0.00999f,  0.012984f, 0.016524f, 0.020594f,
                                   0.025133f, 0.030036f, 0.035151f, 0.040283f, 0.045207f, 0.049681f, 0.053463f,
                                   0.056341f, 0.058141f, 0.058754f, 0.058141f, 0.056341f, 0.053463f, 0.049681f,
                                   0.045207f, 0.040283f, 0.035151f, 0.030036f, 0.025133f, 0.020594f, 0.016524f,
                                   0.012984f, 0.00999f,  0.007527f, 0.005554f, 0.004013f};

// ReflectionDenoiserNew.glsl main (:140-473), one separable pass (dir 1: x,
// 0: y) of the 33-tap Gaussian with depth, normal, luminance, normal-map and
// roughness weights and the settings of Core/Pipeline.cpp:3314-3440
// (u_ResolutionScale = 1 / gi_divisor, u_TemporalWeight = TEMPORAL_SPEC; the
// jitter int((noise - 0.5) * 0.75) is 0). Taps at fractional offsets sample
// the full-resolution depth, face, block and normal planes; the centre tap
// reads the GI-grid views.
template <typename S>
__global__ void __launch_bounds__(256, 6) k_spec_denoise(WorldView w, CamView cam, SpecDenoiseArgs a, int W, int H,
                                                      int Wg, int Hg, const S* t, const uint8_t* face,
                                                      const uint8_t* block, const S* tv, const uint8_t* fv,
                                                      const uint8_t* bv, const S* in, const S* hit_data,
                                                      const S* frames, S* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= Wg || j >= Hg) return;
    const size_t q = (size_t)j * Wg + i;
    const v2 uv = texcoord(i, j, Wg, Hg);
    const Plane<S, 1> TV{tv, Wg, Hg}, T{t, W, H};
    const Plane8 F{face, W, H}, B{block, W, H};
    const v4 bp = position_fetch(cam, TV, i, j, uv);
    const v3 bn = normal_from_id(__ldg(fv + q), 1.0f);
    const int bf = __ldg(fv + q);
    // pow(max(n.n', 1e-11), 32) for a clamped dot product of 0, 1 or 3 (face_cos)
    const float nw0 = dpow(0.00000000001f, 32.0f), nw3 = dpow(3.0f, 32.0f);
    const bool base_sky = bp.w < 0.0f;
    const float4 bc = ld4(in + 4 * q);
    const float base_lum = dot(mk3(bc.x, bc.y, bc.z), mk3(0.299f, 0.587f, 0.114f));
    const int bblock = __ldg(bv + q);
    const S* gbp = (const S*)a.gb_pbr;
    const S* gbn = (const S*)a.gb_normal;
    const float pbr_x = gbp ? gb_pbr_at(gbp, W, H, uv, 0) : pbr_rough(w, bblock);
    const float pbr_y = gbp ? gb_pbr_at(gbp, W, H, uv, 1) : pbr_metal(w, bblock);
    float br = pbr_x + 0.001f;
    const float raw_rough = br;
    br *= mixf(1.0f, 0.91f, 1.0f);
    const bool same_grid = W == Wg && H == Hg;
    const v3 nm_base = gbn ? (same_grid ? mk3(ld(gbn + q * 3), ld(gbn + q * 3 + 1), ld(gbn + q * 3 + 2))
                                        : gb_normal_at(gbn, W, H, uv))
                           : (same_grid ? bn : gnormal_linear(face, W, H, uv));
    float hd = ld(hit_data + q) + 0.0001f;
    if (hd < 0.001f) hd = 1.75f;
    else hd = dpow(hd, 1.0f / 1.3f);
    if (br <= 0.25f + 0.05f) hd = clampf(hd, 0.0f, 8.0f);
    if (br <= 0.2f) hd = clampf(hd, 0.0f, 5.5f);
    const float shd = fmaxf(hd, 0.01f) * (raw_rough < 0.51f ? 0.5f : 0.85f);
    const v4 vs = mat_mul4(a.view, bp.x, bp.y, bp.z, 1.0f);
    const float vlen = length(mk3(vs.x, vs.y, vs.z));
    float vlw = 0.001f + vlen;
    if (br > 0.135f) vlw = fmaxf(vlw, 0.750f);
    else vlw = fmaxf(vlw, 3.0f);
    if (br < 0.125f) vlw = clampf(vlw, 0.000001f, 6.0f);
    else if (br < 0.25f) vlw = clampf(vlw, 0.000001f, 8.0f + 1.0f);
    else if (br < 0.5f) vlw = clampf(vlw, 0.000001f, 16.0f);
    else if (br < 0.75f) vlw = clampf(vlw, 0.000001f, 24.0f);
    else vlw = clampf(vlw, 0.000001f, 32.0f);
    float tc = shd / fmaxf(shd + vlw, 0.00001f);
    if (raw_rough < 0.535f && bp.w < 50.0f) {
        const float rr = (((raw_rough - 0.0f) / (0.535f - 0.0f)) * (1.0f - 0.0f)) + 0.0f;
        const float te = mixf(3.5f, 2.0f, dpow(rr, 4.0f));
        tc = dpow(tc, te + 0.8125f);
    }
    const float rad_e = dpow(1.0f - br, 1.0f / 1.4f) * 5.0f;
    const float radius = clampf(dpow(mixf(1.0f * br, 1.0f, tc), rad_e), 0.0f, 1.0f);
    const float nm_radius = 1.0f - clampf(dpow(mixf(1.0f * br, 1.0f, tc), rad_e), 0.0f, 1.0f);
    int er = f2i_floor(radius * 15.0f);
    er = min(max(er, 1), 15);
    if (br > 0.897511f) er = 15;
    const int jitter = 0;
    float scale = mixf(1.0f, 2.0f, clampf(a.res_scale, 0.0000001f, 1.0f)) + 0.5f;
    const float EPS = 0.001f;
    int rbias = 0;
    if (pbr_y > 0.1f - EPS && br > 0.4f - EPS) rbias += 2;
    er = min(max(er + rbias + 0, 1), 15);
    if (raw_rough >= 0.5f - 0.01f) er += 1;
    scale *= 1.0f;
    float tw_t = 0.0f, afc = 0.01f;
    if (a.temporal_weight) {
        const float af = ld(frames + q);
        afc = af < -0.1f ? 0.0f : (1.0f - af);
        afc = clampf(afc, 0.000001f, 1.0f);
        tw_t = clampf(afc * 0.85f, 0.0f, 1.0f);
        float flt = (float)er;
        flt = mixf(flt, flt + 2.0f, afc * 1.05f);
        er = f2i(flt);
    }
    float hf_e = (64.0f * 0.750f) * 1.350f;
    hf_e *= dpow(nm_radius, 1.0f / 1.33f);
    float hf_add = mixf(0.0f, 0.005f, br > 0.45f ? 1.0f : 0.0f);
    hf_add += mixf(0.0f, 0.0125f, br > 0.525f ? 1.0f : 0.0f);
    hf_add += mixf(0.0f, 0.022f, br > 0.625f ? 1.0f : 0.0f);
    hf_add += mixf(0.0f, 0.026f, br > 0.725f ? 1.0f : 0.0f);
    hf_add += mixf(0.0f, 0.031f, br > 0.75f ? 1.0f : 0.0f);
    er = min(max(er, 1), 15);
    const float texel = a.dir ? 1.0f / (float)Wg : 1.0f / (float)Hg;
    const float hf_gate = ((0.185f + 0.001f) + 0.001f) + 0.0001f;
    float fc[4] = {0.0f, 0.0f, 0.0f, 0.0f}, tw = 0.0f;
#pragma unroll 1
    for (int s = -er; s <= er; s++) {
        const float so = (float)s;
        v2 sc = a.dir ? mk2(uv.x + ((so * scale) * texel), uv.y) : mk2(uv.x, uv.y + ((so * scale) * texel));
        sc.x += ((float)jitter * texel) * 0.75f;
        sc.y += ((float)jitter * texel) * 0.75f;
        const float bias = 0.01f;
        if (!(sc.x > 0.0f + bias && sc.x < 1.0f - bias && sc.y > 0.0f + bias && sc.y < 1.0f - bias)) continue;
        float sdepth;
        float4 sd;
        int sface, sblock;
        v3 nm_at;
        if (s == 0) {
            sdepth = TV.at_in(i, j, 0);
            sface = __ldg(fv + q);
            sblock = bblock;
            sd = bc;
            nm_at = nm_base;
        } else {
            sdepth = bl1(t, bilin(sc, W, H));
            sface = F.nearest(sc);
            sblock = B.nearest(sc);
            sd = bl4(in, bilin(sc, Wg, Hg));
            nm_at = gbn ? gb_normal_at(gbn, W, H, sc) : gnormal_linear(face, W, H, sc);
        }
        const bool sample_sky = sdepth < 0.0f;
        if (sample_sky != base_sky) continue;
        const float dd = fabsf(sdepth - bp.w) * 1.5f;
        const float de = dexp(-dd);
        const float dw = de * de;   // pow(e, 2) for e in [0, 1]
        const int ncls = face_cos(bf, sface);
        const float nw = ncls == 0 ? nw0 : (ncls == 1 ? dpow(1.0f, 32.0f) : nw3);
        float lw = 1.0f;
        const float srough = gbp ? (s == 0 ? pbr_x : gb_pbr_at(gbp, W, H, sc, 0)) : pbr_rough(w, sblock);
        const bool too_rough = srough >= 0.89f;
        if (!too_rough) {
            const float luma = dot(mk3(sd.x, sd.y, sd.z), mk3(0.299f, 0.587f, 0.114f));
            float le = 1.0f / fabsf(luma - base_lum);
            le = dpow(le, 1.7f);
            const float lwe = mixf(0.001f, 8.0f, dpow(srough, 16.0f));
            lw = dpow(le, lwe + 0.8f);
            lw = clampf(lw, 0.0000000001f, 1.0f);
            lw = mixf(lw, 1.0f, tw_t);
            lw = clampf(lw, 0.0000000001f, 1.0f);
        }
        float hfw = 1.0f;
        if (!too_rough && br < 0.8f && afc <= hf_gate) {
            const float angle = dot(nm_at, nm_base);
            hfw = dpow(clampf(angle, 0.00000001f, 1.0f), hf_e);
            hfw = clampf(hfw + ((hf_add * 1.075f) * 1.4f), 0.00000000001f, 1.0f);
        }
        const float re = fabsf(srough - br);
        float rtw = 1.0f / re;
        rtw = dpow(rtw, 12.0f);
        rtw = clampf(rtw, 0.00000000001f, 1.0f);
        const float kw = kGauss33[min(max(16 + s, 0), 32)];
        float cw = 1.0f;
        cw *= dw;
        cw *= nw;
        cw *= hfw;
        cw *= lw;
        cw *= rtw;
        cw *= kw;
        cw = clampf(cw, 0.000000001f, 1.0f);
        fc[0] += sd.x * cw;
        fc[1] += sd.y * cw;
        fc[2] += sd.z * cw;
        fc[3] += sd.w * cw;
        tw += cw;
    }
    const float bcv[4] = {bc.x, bc.y, bc.z, bc.w};
    float o[4];
    if (tw > 0.001f) {
        for (int c = 0; c < 4; c++) fc[c] = fc[c] / tw;
        float smf = 1.0f;
        if (br <= 0.1f + 0.007f) {
            smf = br * 16.0f;
            smf = 1.0f - smf;
            smf = dpow(smf, 4.0f);
            smf = clampf(smf, 0.1f, 0.999f);
        }
        for (int c = 0; c < 4; c++) o[c] = mixf(bcv[c], fc[c], smf);
    } else {
        for (int c = 0; c < 4; c++) o[c] = bcv[c];
    }
    st4(out + 4 * q, o[0], o[1], o[2], o[3]);
}

}  // namespace

cudaError_t trace_reflection(const WorldView& w, const CamView& cam, int W, int H, int Wg, int Hg, int fp16,
                             const ReflectionArgs& a, const void* t, const uint8_t* face, const uint8_t* shadow,
                             const void* tv, const uint8_t* fv, const uint8_t* bv, const void* den_sh,
                             const void* den_cocg, const void* den_ao, void* spec, void* hit, void* mask,
                             Counters* stats, cudaStream_t s) {
    const dim3 grid((unsigned)((Wg + 15) / 16), (unsigned)((Hg + 15) / 16));
    if (fp16)
        k_trace_reflection<__half><<<grid, 256, 0, s>>>(
            w, cam, W, H, Wg, Hg, a, (const __half*)t, face, shadow, (const __half*)tv, fv, bv, (const __half*)den_sh,
            (const __half*)den_cocg, (const __half*)den_ao, (__half*)spec, (__half*)hit, (__half*)mask, stats);
    else
        k_trace_reflection<float><<<grid, 256, 0, s>>>(
            w, cam, W, H, Wg, Hg, a, (const float*)t, face, shadow, (const float*)tv, fv, bv, (const float*)den_sh,
            (const float*)den_cocg, (const float*)den_ao, (float*)spec, (float*)hit, (float*)mask, stats);
    return cudaGetLastError();
}

cudaError_t spec_hit_blur(int Wg, int Hg, int fp16, int pass, const void* tv, const uint8_t* fv, const void* hin,
                          void* hout, cudaStream_t s) {
    const dim3 grid((unsigned)((Wg + 31) / 32), (unsigned)((Hg + 7) / 8)), blk(32, 8);
    if (fp16)
        k_spec_hit_blur<__half><<<grid, blk, 0, s>>>(Wg, Hg, pass, (const __half*)tv, fv, (const __half*)hin,
                                                     (__half*)hout);
    else
        k_spec_hit_blur<float><<<grid, blk, 0, s>>>(Wg, Hg, pass, (const float*)tv, fv, (const float*)hin,
                                                    (float*)hout);
    return cudaGetLastError();
}

cudaError_t spec_temporal(const WorldView& w, const CamView& cam, const SpecTemporalArgs& a, int W, int H, int Wg,
                          int Hg, int fp16, const void* tv, const uint8_t* fv, const uint8_t* bv, const void* prev_t,
                          const uint8_t* prev_face, const void* spec, const void* hit, const void* mask,
                          const void* prev_out, const void* prev_hit, const void* prev_stable, void* out, void* acc,
                          void* stable, cudaStream_t s) {
    const dim3 grid((unsigned)((Wg + 31) / 32), (unsigned)((Hg + 7) / 8)), blk(32, 8);
    if (fp16)
        k_spec_temporal<__half><<<grid, blk, 0, s>>>(
            w, cam, a, W, H, Wg, Hg, (const __half*)tv, fv, bv, (const __half*)prev_t, prev_face, (const __half*)spec,
            (const __half*)hit, (const __half*)mask, (const __half*)prev_out, (const __half*)prev_hit,
            (const __half*)prev_stable, (__half*)out, (__half*)acc, (__half*)stable);
    else
        k_spec_temporal<float><<<grid, blk, 0, s>>>(
            w, cam, a, W, H, Wg, Hg, (const float*)tv, fv, bv, (const float*)prev_t, prev_face, (const float*)spec,
            (const float*)hit, (const float*)mask, (const float*)prev_out, (const float*)prev_hit,
            (const float*)prev_stable, (float*)out, (float*)acc, (float*)stable);
    return cudaGetLastError();
}

cudaError_t spec_denoise(const WorldView& w, const CamView& cam, const SpecDenoiseArgs& a, int W, int H, int Wg,
                         int Hg, int fp16, const void* t, const uint8_t* face, const uint8_t* block, const void* tv,
                         const uint8_t* fv, const uint8_t* bv, const void* in, const void* hit_data,
                         const void* frames, void* out, cudaStream_t s) {
    const dim3 grid((unsigned)((Wg + 31) / 32), (unsigned)((Hg + 7) / 8)), blk(32, 8);
    if (fp16)
        k_spec_denoise<__half><<<grid, blk, 0, s>>>(w, cam, a, W, H, Wg, Hg, (const __half*)t, face, block,
                                                    (const __half*)tv, fv, bv, (const __half*)in,
                                                    (const __half*)hit_data, (const __half*)frames, (__half*)out);
    else
        k_spec_denoise<float><<<grid, blk, 0, s>>>(w, cam, a, W, H, Wg, Hg, (const float*)t, face, block,
                                                   (const float*)tv, fv, bv, (const float*)in,
                                                   (const float*)hit_data, (const float*)frames, (float*)out);
    return cudaGetLastError();
}

}  // namespace vpt
