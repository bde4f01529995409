// The three trace passes for one pixel: primary ray (G-buffer), sun-shadow
// ray and the diffuse GI samples. The one-thread-per-pixel kernels of trace.cu
// and the batched multi-world kernel of batch.cu both run these, so their
// outputs are the same bits. B is the distance-field layout (df_index), S the
// storage type of the float planes.
#pragma once
#include "gi.cuh"
#include "kernels.cuh"

namespace vpt {

__device__ __forceinline__ float stored_value(float v, const float*) { return v; }
__device__ __forceinline__ float stored_value(float v, const __half*) { return __half2float(__float2half_rn(v)); }

template <typename S>
__device__ __forceinline__ unsigned primary_store(const TraceResult& r, size_t px, S* out_t, uint8_t* out_face,
                                                  uint8_t* out_block, int32_t* out_hit, uint16_t* out_steps,
                                                  float* t_stored, int* face_id);

// InitialRayTraceFrag.glsl main (:417-468). Writes the G-buffer texel `px`;
// returns the step count and, for the passes that follow, the hit distance as
// stored and the face id.
// kAlpha: the alpha-tested traversal (u_ShouldAlphaTest) with `stop`.
template <int B, typename S, bool kAlpha = false>
__device__ __forceinline__ unsigned primary_pixel(const WorldView& w, const CamView& cam, int W, int H, int i, int j,
                                                  int max_steps, size_t px, S* out_t, uint8_t* out_face,
                                                  uint8_t* out_block, int32_t* out_hit, uint16_t* out_steps,
                                                  float* t_stored, int* face_id, const AlphaStop* stop = nullptr) {
    const v3 r0 = ray_origin(cam);
    const v3 dir = normalize(ray_dir_at(cam, texcoord(i, j, W, H)));
    const TraceResult r = kAlpha ? traverse_alpha<B>(w, r0, dir, max_steps, *stop) : traverse<B>(w, r0, dir, max_steps);
    return primary_store(r, px, out_t, out_face, out_block, out_hit, out_steps, t_stored, face_id);
}

// The G-buffer texel `px` of a traced primary ray (InitialRayTraceFrag.glsl:438-468).
template <typename S>
__device__ __forceinline__ unsigned primary_store(const TraceResult& r, size_t px, S* out_t, uint8_t* out_face,
                                                  uint8_t* out_block, int32_t* out_hit, uint16_t* out_steps,
                                                  float* t_stored, int* face_id) {
    const bool intersect = r.t > 0.0f && r.block > 0;
    const int face = intersect ? normal_id(r.normal) : kFaceMiss;
    st(out_t + px, r.t);
    out_face[px] = (uint8_t)face;
    out_block[px] = (uint8_t)(intersect ? r.block : 0);
    out_hit[px * 3 + 0] = r.cell[0];
    out_hit[px * 3 + 1] = r.cell[1];
    out_hit[px * 3 + 2] = r.cell[2];
    out_steps[px] = (uint16_t)r.steps;
    *t_stored = stored_value(r.t, out_t);
    *face_id = face;
    return (unsigned)r.steps;
}

// Two primary rays of one thread, their traversals interleaved (traverse2);
// the same G-buffer texels as two primary_pixel calls.
template <int B, typename S>
__device__ __forceinline__ void primary_pixel2(const WorldView& w, const CamView& cam, int W, int H, const int (&i)[2],
                                               const int (&j)[2], const bool (&live)[2], int max_steps, S* out_t,
                                               uint8_t* out_face, uint8_t* out_block, int32_t* out_hit,
                                               uint16_t* out_steps, float (&t_stored)[2], int (&face_id)[2],
                                               unsigned (&steps)[2]) {
    const v3 r0 = ray_origin(cam);
    v3 dir[2];
    for (int k = 0; k < 2; k++) dir[k] = live[k] ? normalize(ray_dir_at(cam, texcoord(i[k], j[k], W, H))) : r0;
    TraceResult r[2];
    traverse2<B>(w, r0, dir[0], max_steps, live[0], r0, dir[1], max_steps, live[1], &r[0], &r[1]);
    for (int k = 0; k < 2; k++) {
        steps[k] = 0;
        if (live[k])
            steps[k] = primary_store(r[k], (size_t)j[k] * W + i[k], out_t, out_face, out_block, out_hit, out_steps,
                                     &t_stored[k], &face_id[k]);
    }
}

// ShadowRayTraceFrag.glsl main (:414-513): one hard shadow ray towards the sun
// from the G-buffer texel with hit distance d and face id `face`.
// kAlpha: the alpha-tested traversal (u_ShouldAlphaTest = ShouldAlphaTestShadows) with `stop`.
template <int B, bool kAlpha = false>
__device__ __forceinline__ uint8_t shadow_pixel(const WorldView& w, const CamView& cam, int W, int H, int i, int j,
                                                int max_steps, v3 L, float d, int face, unsigned* nrays,
                                                unsigned* nsteps, const AlphaStop* stop = nullptr) {
    if (d < 0.0f) return 0;
    const v3 pos = add(ray_origin(cam), muls(normalize(ray_dir_at(cam, texcoord(i, j, W, H))), d));
    const v3 n = normal_from_id(face, 1.0f);
    const float ndl = dot(n, L);
    if (ndl <= 0.01f) return 1;
    const v3 o = add(pos, mul(n, mk3(0.06f, 0.06f, 0.06f)));
    const int block_at = get_voxel(w, f2i_floor(o.x), f2i_floor(o.y), f2i_floor(o.z));
    float T = -1.0f;
    if (d > 0.0f) {
        const TraceResult r = kAlpha ? traverse_alpha<B>(w, o, L, max_steps, *stop) : traverse<B>(w, o, L, max_steps);
        T = r.t;
        *nrays += 1;
        *nsteps += (unsigned)r.steps;
    }
    return (T > 0.0f || block_at > 0) ? 1 : 0;
}

// Two sun-shadow rays of one thread (texels k = 0, 1 with hit distances d[k]
// and faces face[k]), the traversals interleaved; the same bytes as
// shadow_pixel without alpha testing.
template <int B>
__device__ __forceinline__ void shadow_pixel2(const WorldView& w, const CamView& cam, int W, int H, const int (&i)[2],
                                              const int (&j)[2], const bool (&live)[2], int max_steps, v3 L,
                                              const float (&d)[2], const int (&face)[2], uint8_t (&out)[2],
                                              unsigned* nrays, unsigned* nsteps) {
    v3 o[2];
    int block_at[2] = {0, 0};
    bool trace[2] = {false, false};
    for (int k = 0; k < 2; k++) {
        out[k] = 0;
        o[k] = mk3(0.0f, 0.0f, 0.0f);
        if (!live[k] || d[k] < 0.0f) continue;
        const v3 pos = add(ray_origin(cam), muls(normalize(ray_dir_at(cam, texcoord(i[k], j[k], W, H))), d[k]));
        const v3 n = normal_from_id(face[k], 1.0f);
        const float ndl = dot(n, L);
        if (ndl <= 0.01f) {
            out[k] = 1;
            continue;
        }
        o[k] = add(pos, mul(n, mk3(0.06f, 0.06f, 0.06f)));
        block_at[k] = get_voxel(w, f2i_floor(o[k].x), f2i_floor(o[k].y), f2i_floor(o[k].z));
        trace[k] = d[k] > 0.0f;
        if (!trace[k]) out[k] = block_at[k] > 0 ? 1 : 0;
    }
    TraceResult r[2];
    traverse2<B>(w, o[0], L, max_steps, trace[0], o[1], L, max_steps, trace[1], &r[0], &r[1]);
    for (int k = 0; k < 2; k++) {
        if (!trace[k]) continue;
        *nrays += 1;
        *nsteps += (unsigned)r[k].steps;
        out[k] = (r[k].t > 0.0f || block_at[k] > 0) ? 1 : 0;
    }
}

// DiffuseRayTraceFrag.glsl main (:822-935): `spp` GI samples of the texel.
// kOneSample: the caller guarantees one sample (spp <= 1, sun stronger than
// the moon), so nothing of the per-texel sums stays live across the traversal;
// the arithmetic is the same.
//
// kMode (DiffuseMode, gi.cuh) splits a one-sample, one-bounce texel for the
// staged kernel: kDiffuseBounceOnly traces its bounce ray into *staged (and
// the shadow-ray request) and writes nothing; kDiffuseGiven finishes it from
// *staged and given_shadow and writes the outputs. Sky texels (d < 0) are
// written by kDiffuseLive only.
template <int B, typename S, bool kOneSample = false, bool kTex = false, int kMode = kDiffuseLive>
__device__ __forceinline__ void diffuse_pixel(const WorldView& w, const CamView& cam, int W, int H, int i, int j,
                                              const DiffuseArgs& a, size_t px, float d, int face, S* o_sh,
                                              S* o_cocg, S* o_luma, S* o_aosky, GICount* cnt,
                                              StagedBounce* staged = nullptr, bool* need_shadow = nullptr,
                                              v3* shadow_origin = nullptr, float given_shadow = 0.0f) {
    static_assert(kMode == kDiffuseLive || kOneSample, "the staged modes run one sample");
    const v3 dir = normalize(ray_dir_at(cam, texcoord(i, j, W, H)));
    const v3 pos = add(ray_origin(cam), muls(dir, d));
    const v3 n = normal_from_id(face, 0.5f);
    float sh[4], cocg[2];
    if (kMode == kDiffuseLive && d < 0.0f) {
        irradiance_to_sh(muls(sky_radiance(dir), 2.66f), n, sh, cocg);
        for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, sh[c]);
        st(o_cocg + px * 2 + 0, cocg[0]);
        st(o_cocg + px * 2 + 1, cocg[1]);
        st(o_luma + px, luminance(mk3(0.0f, 0.0f, 0.0f)));
        st(o_aosky + px * 2 + 0, 1.0f);
        st(o_aosky + px * 2 + 1, 0.0f);
        return;
    }
    uint32_t rng = pcg_hash((uint32_t)px + pcg_hash(a.frame_index + pcg_hash(a.seed)));
    int spp = kOneSample ? 1 : min(max(a.spp, 1), 32);
    if (!kOneSample && a.lighting.moon_stronger) spp *= 2;
    float tsh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, tcc[2] = {0.0f, 0.0f};
    v3 radiance = mk3(0.0f, 0.0f, 0.0f);
    float acc_ao = 0.0f, skyhits = 0.0f;
    for (int s = 0; s < spp; s++) {
        v3 odir = mk3(0.0f, 0.0f, 0.0f);
        bool ss = false;
        const v4 x = calculate_diffuse<B, kTex, kMode>(w, a, pos, n, &rng, &odir, &ss, cnt, staged, need_shadow,
                                                        shadow_origin, given_shadow);
        if (kMode == kDiffuseBounceOnly) return;
        const v3 xc = vclamp(mk3(x.x, x.y, x.z), 0.0f, 8.0f);
        radiance = add(radiance, xc);
        acc_ao += x.w;
        irradiance_to_sh(xc, odir, sh, cocg);
        for (int c = 0; c < 4; c++) tsh[c] += sh[c];
        tcc[0] += cocg[0];
        tcc[1] += cocg[1];
        skyhits += ss ? 1.0f : 0.0f;
    }
    const float fs = (float)spp;
    acc_ao /= fs;
    for (int c = 0; c < 4; c++) tsh[c] /= fs;
    tcc[0] /= fs;
    tcc[1] /= fs;
    radiance = divs(radiance, fs);
    skyhits /= fs;
    for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, clampf(tsh[c], -100.0f, 100.0f));
    st(o_cocg + px * 2 + 0, clampf(tcc[0], -100.0f, 100.0f));
    st(o_cocg + px * 2 + 1, clampf(tcc[1], -100.0f, 100.0f));
    st(o_luma + px, clampf(fmaxf(luminance(radiance), 0.01f), 0.001f, 64.0f));
    st(o_aosky + px * 2 + 0, clampf(acc_ao, 0.0f, 1.0f));
    st(o_aosky + px * 2 + 1, clampf(skyhits, 0.0f, 1.0f));
}

// Warp-aggregated ray and step counts (the statistics counters).
__device__ __forceinline__ void count_rays(Counters* c, int kind, unsigned rays, unsigned steps) {
    const unsigned r = __reduce_add_sync(0xffffffffu, rays);
    const unsigned s = __reduce_add_sync(0xffffffffu, steps);
    if ((threadIdx.x & 31) == 0 && (r | s)) {
        atomicAdd(&c->rays[kind], (unsigned long long)r);
        atomicAdd(&c->steps[kind], (unsigned long long)s);
    }
}

}  // namespace vpt
