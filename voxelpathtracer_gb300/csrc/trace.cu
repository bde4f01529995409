// The three trace passes as separate kernels, one thread per pixel: primary
// (G-buffer), sun shadow and diffuse GI. They back the pass-by-pass entry
// points of the C ABI; the frame path uses the fused persistent kernel in
// trace_frame.cu. The traversal is dda.cuh.
#include "gi.cuh"
#include "kernels.cuh"

namespace vpt {

namespace {

// Pixel of thread `tid` in a 16x16 tile: each warp covers an 8x4 patch so its
// rays stay spatially coherent.
__device__ __forceinline__ void tile_pixel(int* i, int* j) {
    int tid = threadIdx.x;
    int warp = tid >> 5, lane = tid & 31;
    *i = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    *j = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
}

__device__ __forceinline__ void count_rays(Counters* c, int kind, unsigned rays, unsigned steps) {
    unsigned r = __reduce_add_sync(0xffffffffu, rays);
    unsigned s = __reduce_add_sync(0xffffffffu, steps);
    if ((threadIdx.x & 31) == 0 && (r | s)) {
        atomicAdd(&c->rays[kind], (unsigned long long)r);
        atomicAdd(&c->steps[kind], (unsigned long long)s);
    }
}

// InitialRayTraceFrag.glsl main (:417-468)
template <typename S>
__global__ void __launch_bounds__(256) k_trace_primary(WorldView w, CamView cam, int W, int H, int max_steps,
                                                       S* out_t, uint8_t* out_face, uint8_t* out_block,
                                                       int32_t* out_hit, uint16_t* out_steps, Counters* stats) {
    int i, j;
    tile_pixel(&i, &j);
    bool valid = i < W && j < H;
    unsigned nsteps = 0;
    if (valid) {
        size_t px = (size_t)j * W + i;
        v3 r0 = ray_origin(cam);
        v3 dir = normalize(ray_dir_at(cam, texcoord(i, j, W, H)));
        TraceResult r = traverse(w, r0, dir, max_steps);
        bool intersect = r.t > 0.0f && r.block > 0;
        st(out_t + px, r.t);
        out_face[px] = (uint8_t)(intersect ? normal_id(r.normal) : kFaceMiss);
        out_block[px] = (uint8_t)(intersect ? r.block : 0);
        out_hit[px * 3 + 0] = r.cell[0];
        out_hit[px * 3 + 1] = r.cell[1];
        out_hit[px * 3 + 2] = r.cell[2];
        out_steps[px] = (uint16_t)r.steps;
        nsteps = (unsigned)r.steps;
    }
    if (stats) count_rays(stats, kRayPrimary, valid ? 1u : 0u, nsteps);
}

// ShadowRayTraceFrag.glsl main (:414-513): one hard shadow ray towards the sun.
template <typename S>
__global__ void __launch_bounds__(256) k_trace_shadow(WorldView w, CamView cam, int W, int H, int max_steps,
                                                      float lx, float ly, float lz, const S* t,
                                                      const uint8_t* face, uint8_t* shadow, Counters* stats) {
    int i, j;
    tile_pixel(&i, &j);
    unsigned nrays = 0, nsteps = 0;
    if (i < W && j < H) {
        size_t px = (size_t)j * W + i;
        float d = ld(t + px);
        uint8_t out;
        if (d < 0.0f) {
            out = 0;
        } else {
            v3 L = mk3(lx, ly, lz);
            v3 pos = add(ray_origin(cam), muls(normalize(ray_dir_at(cam, texcoord(i, j, W, H))), d));
            v3 n = normal_from_id(__ldg(face + px), 1.0f);
            float ndl = dot(n, L);
            if (ndl <= 0.01f) {
                out = 1;
            } else {
                v3 o = add(pos, mul(n, mk3(0.06f, 0.06f, 0.06f)));
                int block_at = get_voxel(w, f2i_floor(o.x), f2i_floor(o.y), f2i_floor(o.z));
                float T = -1.0f;
                if (d > 0.0f) {
                    TraceResult r = traverse(w, o, L, max_steps);
                    T = r.t;
                    nrays = 1;
                    nsteps = (unsigned)r.steps;
                }
                out = (T > 0.0f || block_at > 0) ? 1 : 0;
            }
        }
        shadow[px] = out;
    }
    if (stats) count_rays(stats, kRayShadow, nrays, nsteps);
}

// DiffuseRayTraceFrag.glsl main (:822-935)
template <typename S>
__global__ void __launch_bounds__(256) k_trace_diffuse(WorldView w, CamView cam, int W, int H, DiffuseArgs a,
                                                       const S* t, const uint8_t* face, S* o_sh, S* o_cocg,
                                                       S* o_luma, S* o_aosky, Counters* stats) {
    int i, j;
    tile_pixel(&i, &j);
    GICount cnt = {0u, 0u, 0u, 0u};
    if (i < W && j < H) {
        size_t px = (size_t)j * W + i;
        v3 dir = normalize(ray_dir_at(cam, texcoord(i, j, W, H)));
        float d = ld(t + px);
        v3 pos = add(ray_origin(cam), muls(dir, d));
        v3 n = normal_from_id(__ldg(face + px), 0.5f);
        float sh[4], cocg[2];
        if (d < 0.0f) {
            irradiance_to_sh(muls(sky_radiance(dir), 2.66f), n, sh, cocg);
            for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, sh[c]);
            st(o_cocg + px * 2 + 0, cocg[0]);
            st(o_cocg + px * 2 + 1, cocg[1]);
            st(o_luma + px, luminance(mk3(0.0f, 0.0f, 0.0f)));
            st(o_aosky + px * 2 + 0, 1.0f);
            st(o_aosky + px * 2 + 1, 0.0f);
        } else {
            uint32_t rng = pcg_hash((uint32_t)px + pcg_hash(a.frame_index + pcg_hash(a.seed)));
            int spp = min(max(a.spp, 1), 32);
            if (a.lighting.moon_stronger) spp *= 2;
            float tsh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, tcc[2] = {0.0f, 0.0f};
            v3 radiance = mk3(0.0f, 0.0f, 0.0f);
            float acc_ao = 0.0f, skyhits = 0.0f;
            for (int s = 0; s < spp; s++) {
                v3 odir = mk3(0.0f, 0.0f, 0.0f);
                bool ss = false;
                v4 x = calculate_diffuse(w, a, pos, n, &rng, &odir, &ss, &cnt);
                v3 xc = vclamp(mk3(x.x, x.y, x.z), 0.0f, 8.0f);
                radiance = add(radiance, xc);
                acc_ao += x.w;
                irradiance_to_sh(xc, odir, sh, cocg);
                for (int c = 0; c < 4; c++) tsh[c] += sh[c];
                tcc[0] += cocg[0];
                tcc[1] += cocg[1];
                skyhits += ss ? 1.0f : 0.0f;
            }
            float fs = (float)spp;
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
    }
    if (stats) {
        count_rays(stats, kRayDiffuse, cnt.diffuse_rays, cnt.diffuse_steps);
        count_rays(stats, kRayBounceShadow, cnt.shadow_rays, cnt.shadow_steps);
    }
}

inline dim3 tile_grid(int W, int H) { return dim3((unsigned)((W + 15) / 16), (unsigned)((H + 15) / 16)); }

}  // namespace

cudaError_t trace_primary(const WorldView& w, const CamView& cam, int W, int H, int max_steps, int fp16,
                          GBufferOut out, Counters* stats, cudaStream_t s) {
    if (fp16)
        k_trace_primary<__half><<<tile_grid(W, H), 256, 0, s>>>(w, cam, W, H, max_steps, (__half*)out.t, out.face,
                                                                out.block, out.hit, out.steps, stats);
    else
        k_trace_primary<float><<<tile_grid(W, H), 256, 0, s>>>(w, cam, W, H, max_steps, (float*)out.t, out.face,
                                                               out.block, out.hit, out.steps, stats);
    return cudaGetLastError();
}

cudaError_t trace_shadow(const WorldView& w, const CamView& cam, int W, int H, int max_steps, const float sun[3],
                         int fp16, const void* t, const uint8_t* face, uint8_t* shadow, Counters* stats,
                         cudaStream_t s) {
    if (fp16)
        k_trace_shadow<__half><<<tile_grid(W, H), 256, 0, s>>>(w, cam, W, H, max_steps, sun[0], sun[1], sun[2],
                                                               (const __half*)t, face, shadow, stats);
    else
        k_trace_shadow<float><<<tile_grid(W, H), 256, 0, s>>>(w, cam, W, H, max_steps, sun[0], sun[1], sun[2],
                                                              (const float*)t, face, shadow, stats);
    return cudaGetLastError();
}

cudaError_t trace_diffuse(const WorldView& w, const CamView& cam, int W, int H, const DiffuseArgs& a, int fp16,
                          const void* t, const uint8_t* face, GIOut out, Counters* stats, cudaStream_t s) {
    if (fp16)
        k_trace_diffuse<__half><<<tile_grid(W, H), 256, 0, s>>>(w, cam, W, H, a, (const __half*)t, face,
                                                                (__half*)out.sh, (__half*)out.cocg,
                                                                (__half*)out.luma, (__half*)out.aosky, stats);
    else
        k_trace_diffuse<float><<<tile_grid(W, H), 256, 0, s>>>(w, cam, W, H, a, (const float*)t, face,
                                                               (float*)out.sh, (float*)out.cocg, (float*)out.luma,
                                                               (float*)out.aosky, stats);
    return cudaGetLastError();
}

}  // namespace vpt
