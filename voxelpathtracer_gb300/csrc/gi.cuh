// The diffuse GI path of one sample (CalculateDiffuse,
// DiffuseRayTraceFrag.glsl:535-664), shared by the diffuse trace pass and the
// ground-truth accumulator.
#pragma once
#include "dda.cuh"
#include "kernels.cuh"
#include "textures.cuh"

namespace vpt {

struct GICount {
    unsigned diffuse_rays, diffuse_steps, shadow_rays, shadow_steps;
};

// How calculate_diffuse gets its traversals. kLive: it traces the bounce and
// shadow rays itself. The staged one-bounce kernel splits a sample in three:
// kBounceOnly traces the first bounce ray, reports its hit (StagedBounce) and
// whether a sun-shadow ray is needed from where, and stops; the shadow rays
// are traced separately; kGiven then runs the whole sample again with that
// bounce hit and shadow result supplied instead of tracing, so every value
// comes out of the same arithmetic as in kLive.
enum DiffuseMode { kDiffuseLive = 0, kDiffuseBounceOnly = 1, kDiffuseGiven = 2 };

struct StagedBounce {
    float t;        // hit distance of the first bounce ray (-1: miss)
    int face;       // normal_id of its hit normal
    int block;      // block id at the hit (0: miss)
};

// CalculateDiffuse (DiffuseRayTraceFrag.glsl:535-664); B is the distance-field
// layout. kTex: the bounce hit's albedo, roughness and emission come from the
// block textures (:569-584): textureLod of the albedo array at level 3 and of
// the PBR array at level 2, both at the block's albedo layer as the shader
// indexes them, at CalculateUV's coordinates; the emissive texture (texture(),
// whose implicit derivatives across a pixel quad's unrelated bounce hits are
// taken as zero) at level 0.
//
// kMode (DiffuseMode), for one bounce only: kDiffuseBounceOnly fills *staged,
// *need_shadow and *shadow_origin and returns; kDiffuseGiven takes *staged
// and given_shadow (the shadow ray's verdict, 1 = occluded) instead of tracing.
template <int B = 0, bool kTex = false, int kMode = kDiffuseLive>
__device__ __forceinline__ v4 calculate_diffuse(const WorldView& w, const DiffuseArgs& a, v3 initial_origin,
                                                v3 input_normal, uint32_t* rng, v3* odir, bool* skyhit,
                                                GICount* cnt, StagedBounce* staged = nullptr,
                                                bool* need_shadow = nullptr, v3* shadow_origin = nullptr,
                                                float given_shadow = 0.0f) {
    const GILighting& L = a.lighting;
    const v3 light_dir = mk3(L.light_dir[0], L.light_dir[1], L.light_dir[2]);
    const v3 light_color = mk3(L.light_color[0], L.light_color[1], L.light_color[2]);
    *skyhit = false;
    const float bias = 0.06f;
    v3 ro = add(initial_origin, muls(input_normal, bias));
    v3 rd = cos_hemisphere(input_normal, rng);
    float ao = 1.0f;
    v3 contribution = mk3(0.0f, 0.0f, 0.0f);
    v3 throughput = mk3(1.0f, 1.0f, 1.0f);
    const int bounces = kMode == kDiffuseLive ? a.bounces : 1;
    for (int i = 0; i < bounces; i++) {
        if (i == 0) *odir = rd;
        TraceResult tr;
        if (kMode == kDiffuseGiven) {
            tr.t = staged->t;
            tr.block = staged->block;
            tr.normal = staged->block > 0 ? normal_from_id(staged->face, 1.0f) : mk3(0.0f, 0.0f, 0.0f);
        } else {
            tr = traverse<B>(w, ro, rd, a.diffuse_max_steps);
            cnt->diffuse_rays += 1;
            cnt->diffuse_steps += (unsigned)tr.steps;
        }
        float T = tr.t;
        bool intersect = T > 0.0f;
        v3 ip = add(ro, muls(rd, T));
        if (kMode == kDiffuseBounceOnly) {
            const bool hit = intersect && tr.block > 0;
            staged->t = T;
            staged->block = hit ? tr.block : 0;
            staged->face = hit ? normal_id(tr.normal) : 0;
            *need_shadow = hit && !L.moon_stronger && !(fmaxf(dot(tr.normal, light_dir), 0.0f) < 0.001f);
            *shadow_origin = add(ip, muls(tr.normal, 0.045f));
            return v4{};
        }
        if (intersect && tr.block > 0) {
            const int bid = min(max(tr.block, 0), 127);
            Material m = material(w, bid);
            v3 hn = tr.normal;
            float emissivity = 0.0f;
            if (kTex) {
                const BlockTexView& tv = a.tex;
                const v2 P = face_coords(ip, normal_id(hn));
                const float u = P.x - floorf(P.x), v = P.y - floorf(P.y);
                const int layer = __ldg(tv.ids + bid), el = __ldg(tv.ids + 384 + bid);
                float alb[4], pbr[4];
                sample_level(tv.albedo, layer, u, v, 3, 3, tv.srgb, alb);
                sample_level(tv.pbr, layer, u, v, 2, 3, tv.unorm, pbr);
                m.albedo = mk3(alb[0], alb[1], alb[2]);
                m.rough = pbr[0];
                if (tv.emissive.texels && el >= 0) {
                    float e[4];
                    sample_level(tv.emissive, el, u, v, 0, 1, tv.unorm, e);
                    emissivity = e[0] * L.emissivity_multiplier * L.diffuse_light_intensity;
                }
            } else if (m.emissive) {
                emissivity = 1.0f * L.emissivity_multiplier * L.diffuse_light_intensity;
            }
            float ndl = fmaxf(dot(hn, light_dir), 0.0f);
            v3 bias_shadow = muls(hn, 0.045f);
            float shadow_at;
            if (L.moon_stronger) {
                shadow_at = 1.0f;
            } else if (ndl < 0.001f) {
                shadow_at = 0.0f;
            } else if (kMode == kDiffuseGiven) {
                shadow_at = given_shadow;
            } else {
                // GetShadowAt (:1202-1222)
                TraceResult sr = traverse<B>(w, add(ip, bias_shadow), light_dir, a.bounce_shadow_max_steps);
                cnt->shadow_rays += 1;
                cnt->shadow_steps += (unsigned)sr.steps;
                shadow_at = sr.t > 0.0f ? 1.0f : 0.0f;
            }
            v3 emissive_color = muls(m.albedo, emissivity * mixf(1.0f, 1.0f, L.sun_visibility));
            float hs = diffuse_hammon(hn, neg(rd), light_dir, m.rough);
            v3 sun_brdf = muls(muls(mul(muls(m.albedo, hs), muls(light_color, 3.5f)), 1.0f - shadow_at), kPI);
            v3 new_dir = cos_hemisphere(hn, rng);
            float cos_theta = clampf(dot(hn, new_dir), 0.0f, 1.0f);
            float pdf = fmaxf(cos_theta / kPI, 0.00001f);
            float att = diffuse_hammon(hn, neg(rd), new_dir, m.rough);
            contribution = add(contribution, mul(throughput, sun_brdf));
            contribution = add(contribution, mul(emissive_color, throughput));
            throughput = mul(throughput, divs(muls(m.albedo, att), pdf));
            rd = new_dir;
            ro = add(ip, muls(hn, bias));
        } else {
            float x = mixf(1.0f, 1.05f, L.sun_visibility);
            x = clampf(x * 1.0f * L.gi_sky_strength, 0.0f, 5.0f);
            v3 sky = muls(sky_color_at(rd), x);
            contribution = add(contribution, mul(sky, throughput));
            *skyhit = true;
            break;
        }
        if (i == 0) {
            const float dao = 2.0f;
            if (T < dao && T > 0.0f) ao = fmaxf(T / dao, 0.0f);
        }
    }
    v4 r;
    r.x = contribution.x; r.y = contribution.y; r.z = contribution.z; r.w = ao;
    return r;
}

}  // namespace vpt
