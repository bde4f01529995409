// The three trace passes as separate kernels, one thread per pixel: primary
// (G-buffer), sun shadow and diffuse GI. The per-pixel work is
// pixel_passes.cuh; the traversal is dda.cuh.
#include "pixel_passes.cuh"

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

// InitialRayTraceFrag.glsl main (:417-468)
template <typename S, bool kAlpha>
__global__ void __launch_bounds__(256) k_trace_primary(WorldView w, CamView cam, int W, int H, int max_steps,
                                                       S* out_t, uint8_t* out_face, uint8_t* out_block,
                                                       int32_t* out_hit, uint16_t* out_steps, Counters* stats,
                                                       AlphaStop stop) {
    int i, j;
    tile_pixel(&i, &j);
    const bool valid = i < W && j < H;
    unsigned nsteps = 0;
    if (valid) {
        float d;
        int face;
        nsteps = primary_pixel<0, S, kAlpha>(w, cam, W, H, i, j, max_steps, (size_t)j * W + i, out_t, out_face,
                                             out_block, out_hit, out_steps, &d, &face, &stop);
    }
    if (stats) count_rays(stats, kRayPrimary, valid ? 1u : 0u, nsteps);
}

// ShadowRayTraceFrag.glsl main (:414-513): one hard shadow ray towards the sun.
template <typename S, bool kAlpha>
__global__ void __launch_bounds__(256) k_trace_shadow(WorldView w, CamView cam, int W, int H, int max_steps,
                                                      float lx, float ly, float lz, const S* t,
                                                      const uint8_t* face, uint8_t* shadow, Counters* stats,
                                                      AlphaStop stop) {
    int i, j;
    tile_pixel(&i, &j);
    unsigned nrays = 0, nsteps = 0;
    if (i < W && j < H) {
        const size_t px = (size_t)j * W + i;
        shadow[px] = shadow_pixel<0, kAlpha>(w, cam, W, H, i, j, max_steps, mk3(lx, ly, lz), ld(t + px),
                                             __ldg(face + px), &nrays, &nsteps, &stop);
    }
    if (stats) count_rays(stats, kRayShadow, nrays, nsteps);
}

// DiffuseRayTraceFrag.glsl main (:822-935)
template <typename S, bool kOneSample, bool kTex>
__global__ void __launch_bounds__(256, 8) k_trace_diffuse(WorldView w, CamView cam, int W, int H, DiffuseArgs a,
                                                       const S* t, const uint8_t* face, S* o_sh, S* o_cocg,
                                                       S* o_luma, S* o_aosky, Counters* stats) {
    int i, j;
    tile_pixel(&i, &j);
    GICount cnt = {0u, 0u, 0u, 0u};
    if (i < W && j < H) {
        const size_t px = (size_t)j * W + i;
        diffuse_pixel<0, S, kOneSample, kTex>(w, cam, W, H, i, j, a, px, ld(t + px), __ldg(face + px), o_sh, o_cocg, o_luma, o_aosky,
                         &cnt);
    }
    if (stats) {
        count_rays(stats, kRayDiffuse, cnt.diffuse_rays, cnt.diffuse_steps);
        count_rays(stats, kRayBounceShadow, cnt.shadow_rays, cnt.shadow_steps);
    }
}

// The same pass for one sample and one bounce, reorganised so that rays of
// one kind fill whole warps (DiffuseRayTraceFrag.glsl main :822-935,
// CalculateDiffuse :535-664 with one bounce). A CTA of 128 threads owns a
// 32x16-pixel tile (16 patches of 8x4 pixels):
//   0. sky texels (no G-buffer hit) are written at once; the texels with a hit
//      are listed in shared memory, patch by patch;
//   1. each listed texel's bounce ray is set up (origin, cosine-weighted
//      direction) by one thread per texel;
//   2. the bounce rays are traversed from a pool: every warp keeps its lanes
//      busy by taking the next listed ray whenever at least kRefill lanes have
//      finished theirs, so a warp no longer waits for its slowest of 32 fixed
//      rays; a finished ray leaves only its final DDA state behind;
//   3. one thread per texel turns that state into the hit (ray_finish) and the
//      sun-shadow request (about one hit in eight faces the sun);
//   4. the shadow requests, compacted, are traced by consecutive threads;
//   5. one thread per texel finishes the sample (calculate_diffuse replayed
//      with the recorded hit and shadow verdict) and writes the GI planes.
// Outputs and ray counts are those of k_trace_diffuse.
constexpr int kPoolTileW = 32, kPoolTileH = 16, kPoolTexels = kPoolTileW * kPoolTileH, kPoolThreads = 128;
constexpr int kRefill = 8;   // idle lanes that make a warp take new rays

template <typename S, bool kTex>
__global__ void __launch_bounds__(kPoolThreads, 6) k_trace_diffuse_staged(WorldView w, CamView cam, int W, int H,
                                                                           DiffuseArgs a, const S* t,
                                                                           const uint8_t* face, S* o_sh, S* o_cocg,
                                                                           S* o_luma, S* o_aosky, Counters* stats) {
    __shared__ uint32_t s_pix[kPoolTexels];          // listed texels: i | j << 16
    __shared__ float s_ro[kPoolTexels][3];           // bounce ray origin
    __shared__ float s_rd[kPoolTexels][3];           // and direction
    __shared__ float4 s_end[kPoolTexels];            // final DDA position, step count; then the shadow ray origin
    __shared__ uint8_t s_meta[kPoolTexels];          // final MinIdx | Intersection << 2
    __shared__ float s_bt[kPoolTexels];              // bounce hit distance
    __shared__ uint8_t s_bface[kPoolTexels], s_bblock[kPoolTexels], s_need[kPoolTexels], s_shadow[kPoolTexels];
    __shared__ uint16_t s_slist[kPoolTexels];        // texels with a shadow request
    __shared__ int s_n[3];                           // listed texels, pool position, shadow requests
    const int tid = threadIdx.x, lane = tid & 31;
    const unsigned full = 0xffffffffu;
    if (tid < 3) s_n[tid] = 0;
    __syncthreads();
    GICount cnt = {0u, 0u, 0u, 0u};
    const GILighting& L = a.lighting;

    // 0. sky texels now, hit texels listed (a warp takes one 8x4 patch per pass)
    for (int p = tid; p < kPoolTexels; p += kPoolThreads) {
        const int patch = p >> 5;
        const int i = blockIdx.x * kPoolTileW + (patch & 3) * 8 + (lane & 7);
        const int j = blockIdx.y * kPoolTileH + (patch >> 2) * 4 + (lane >> 3);
        bool hit = false;
        if (i < W && j < H) {
            const size_t px = (size_t)j * W + i;
            const float d = ld(t + px);
            if (d < 0.0f)
                diffuse_pixel<0, S, true, kTex>(w, cam, W, H, i, j, a, px, d, __ldg(face + px), o_sh, o_cocg, o_luma,
                                                o_aosky, &cnt);
            else
                hit = true;
        }
        const unsigned m = __ballot_sync(full, hit);
        int base = 0;
        if (lane == 0 && m) base = atomicAdd(&s_n[0], __popc(m));
        base = __shfl_sync(full, base, 0);
        if (hit) s_pix[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i | ((uint32_t)j << 16);
    }
    __syncthreads();
    const int n_hit = s_n[0];

    // 1. bounce rays
    for (int k = tid; k < n_hit; k += kPoolThreads) {
        const int i = (int)(s_pix[k] & 0xffffu), j = (int)(s_pix[k] >> 16);
        const size_t px = (size_t)j * W + i;
        v3 dir, pos, n, ro, rd;
        uint32_t rng;
        diffuse_texel_setup(cam, W, H, i, j, a, px, ld(t + px), __ldg(face + px), &dir, &pos, &n, &rng);
        diffuse_bounce_ray(pos, n, &rng, &ro, &rd);
        s_ro[k][0] = ro.x; s_ro[k][1] = ro.y; s_ro[k][2] = ro.z;
        s_rd[k][0] = rd.x; s_rd[k][1] = rd.y; s_rd[k][2] = rd.z;
    }
    __syncthreads();

    // 2. the pool: lanes take rays as they become free
    {
        RayState r;
        bool active = false, drained = false;   // drained is the same on every lane of the warp
        int item = 0;
        for (;;) {
            if (!drained) {
                const unsigned idle = __ballot_sync(full, !active);
                const int n_idle = __popc(idle);
                if (n_idle >= kRefill || idle == full) {
                    const int leader = __ffs(idle) - 1;
                    int base = 0;
                    if (lane == leader) base = atomicAdd(&s_n[1], n_idle);
                    base = __shfl_sync(full, base, leader);
                    if (base + n_idle >= n_hit) drained = true;
                    if (!active) {
                        const int q = base + __popc(idle & ((1u << lane) - 1u));
                        if (q < n_hit) {
                            ray_start(r, mk3(s_ro[q][0], s_ro[q][1], s_ro[q][2]),
                                      mk3(s_rd[q][0], s_rd[q][1], s_rd[q][2]), a.diffuse_max_steps);
                            item = q;
                            active = true;
                        }
                    }
                }
            }
            if (!__any_sync(full, active)) {
                if (drained) break;
                continue;
            }
            if (active && dda_step<0>(w, r)) {
                s_end[item] = make_float4(r.o.x, r.o.y, r.o.z, __int_as_float(r.itr));
                s_meta[item] = (uint8_t)(r.min_idx | (r.inter << 2));
                cnt.diffuse_rays += 1;
                cnt.diffuse_steps += (unsigned)r.itr;
                active = false;
            }
        }
    }
    __syncthreads();

    // 3. hits and shadow requests
    for (int k = tid; k < n_hit; k += kPoolThreads) {
        RayState r;
        const v3 ro = mk3(s_ro[k][0], s_ro[k][1], s_ro[k][2]);
        ray_start(r, ro, mk3(s_rd[k][0], s_rd[k][1], s_rd[k][2]), a.diffuse_max_steps);
        const float4 e = s_end[k];
        r.o = mk3(e.x, e.y, e.z);
        r.itr = __float_as_int(e.w);
        r.min_idx = s_meta[k] & 3;
        r.inter = s_meta[k] >> 2;
        const TraceResult tr = ray_finish(w, r);
        StagedBounce sb;
        bool need = false;
        v3 so;
        staged_record(tr, ro, r.d, L, &sb, &need, &so);
        s_bt[k] = sb.t;
        s_bface[k] = (uint8_t)sb.face;
        s_bblock[k] = (uint8_t)sb.block;
        s_need[k] = need ? 1 : 0;
        s_shadow[k] = 0;
        s_end[k] = make_float4(so.x, so.y, so.z, 0.0f);
    }
    __syncthreads();
    for (int k0 = 0; k0 < n_hit; k0 += kPoolThreads) {   // compaction, in texel order
        const int k = k0 + tid;
        const bool need = k < n_hit && s_need[k];
        const unsigned m = __ballot_sync(full, need);
        int base = 0;
        if (lane == 0 && m) base = atomicAdd(&s_n[2], __popc(m));
        base = __shfl_sync(full, base, 0);
        if (need) s_slist[base + __popc(m & ((1u << lane) - 1u))] = (uint16_t)k;
    }
    __syncthreads();

    // 4. GetShadowAt (DiffuseRayTraceFrag.glsl:1202-1222) for the requests
    const int n_sh = s_n[2];
    const v3 light_dir = mk3(L.light_dir[0], L.light_dir[1], L.light_dir[2]);
    for (int k = tid; k < n_sh; k += kPoolThreads) {
        const int item = s_slist[k];
        const float4 o = s_end[item];
        const TraceResult sr = traverse<0>(w, mk3(o.x, o.y, o.z), light_dir, a.bounce_shadow_max_steps);
        cnt.shadow_rays += 1;
        cnt.shadow_steps += (unsigned)sr.steps;
        s_shadow[item] = sr.t > 0.0f ? 1 : 0;
    }
    __syncthreads();

    // 5. the samples, finished
    for (int k = tid; k < n_hit; k += kPoolThreads) {
        const int i = (int)(s_pix[k] & 0xffffu), j = (int)(s_pix[k] >> 16);
        const size_t px = (size_t)j * W + i;
        const StagedBounce sb{s_bt[k], (int)s_bface[k], (int)s_bblock[k]};
        diffuse_pixel<0, S, true, kTex, kDiffuseGiven>(w, cam, W, H, i, j, a, px, ld(t + px), __ldg(face + px), o_sh,
                                                       o_cocg, o_luma, o_aosky, &cnt, &sb,
                                                       s_shadow[k] ? 1.0f : 0.0f);
    }
    if (stats) {
        count_rays(stats, kRayDiffuse, cnt.diffuse_rays, cnt.diffuse_steps);
        count_rays(stats, kRayBounceShadow, cnt.shadow_rays, cnt.shadow_steps);
    }
}

inline dim3 tile_grid(int W, int H) { return dim3((unsigned)((W + 15) / 16), (unsigned)((H + 15) / 16)); }

template <typename S>
void launch_diffuse(bool one, bool tex, dim3 grid, cudaStream_t s, const WorldView& w, const CamView& cam, int W,
                    int H, const DiffuseArgs& a, const void* t, const uint8_t* face, GIOut out, Counters* stats) {
    using K = void (*)(WorldView, CamView, int, int, DiffuseArgs, const S*, const uint8_t*, S*, S*, S*, S*, Counters*);
    const K table[4] = {k_trace_diffuse<S, false, false>, k_trace_diffuse<S, false, true>,
                        k_trace_diffuse<S, true, false>, k_trace_diffuse<S, true, true>};
    table[(one ? 2 : 0) + (tex ? 1 : 0)]<<<grid, 256, 0, s>>>(w, cam, W, H, a, (const S*)t, face, (S*)out.sh,
                                                               (S*)out.cocg, (S*)out.luma, (S*)out.aosky, stats);
}

}  // namespace

cudaError_t trace_primary(const WorldView& w, const CamView& cam, int W, int H, int max_steps, int fp16,
                          GBufferOut out, Counters* stats, cudaStream_t s, const AlphaStop* alpha) {
    const AlphaStop st = alpha ? *alpha : AlphaStop{};
    if (fp16)
        (alpha ? k_trace_primary<__half, true> : k_trace_primary<__half, false>)<<<tile_grid(W, H), 256, 0, s>>>(
            w, cam, W, H, max_steps, (__half*)out.t, out.face, out.block, out.hit, out.steps, stats, st);
    else
        (alpha ? k_trace_primary<float, true> : k_trace_primary<float, false>)<<<tile_grid(W, H), 256, 0, s>>>(
            w, cam, W, H, max_steps, (float*)out.t, out.face, out.block, out.hit, out.steps, stats, st);
    return cudaGetLastError();
}

cudaError_t trace_shadow(const WorldView& w, const CamView& cam, int W, int H, int max_steps, const float sun[3],
                         int fp16, const void* t, const uint8_t* face, uint8_t* shadow, Counters* stats,
                         cudaStream_t s, const AlphaStop* alpha) {
    const AlphaStop st = alpha ? *alpha : AlphaStop{};
    if (fp16)
        (alpha ? k_trace_shadow<__half, true> : k_trace_shadow<__half, false>)<<<tile_grid(W, H), 256, 0, s>>>(
            w, cam, W, H, max_steps, sun[0], sun[1], sun[2], (const __half*)t, face, shadow, stats, st);
    else
        (alpha ? k_trace_shadow<float, true> : k_trace_shadow<float, false>)<<<tile_grid(W, H), 256, 0, s>>>(
            w, cam, W, H, max_steps, sun[0], sun[1], sun[2], (const float*)t, face, shadow, stats, st);
    return cudaGetLastError();
}

cudaError_t trace_diffuse(const WorldView& w, const CamView& cam, int W, int H, const DiffuseArgs& a, int fp16,
                          const void* t, const uint8_t* face, GIOut out, Counters* stats, cudaStream_t s) {
    const bool one = a.spp <= 1 && !a.lighting.moon_stronger, tex = a.textured != 0;
    if (one && a.bounces == 1 && W < 65536 && H < 65536) {
        const dim3 g((unsigned)((W + kPoolTileW - 1) / kPoolTileW), (unsigned)((H + kPoolTileH - 1) / kPoolTileH));
        if (fp16)
            (tex ? k_trace_diffuse_staged<__half, true> : k_trace_diffuse_staged<__half, false>)<<<g, kPoolThreads, 0, s>>>(
                w, cam, W, H, a, (const __half*)t, face, (__half*)out.sh, (__half*)out.cocg, (__half*)out.luma,
                (__half*)out.aosky, stats);
        else
            (tex ? k_trace_diffuse_staged<float, true> : k_trace_diffuse_staged<float, false>)<<<g, kPoolThreads, 0, s>>>(
                w, cam, W, H, a, (const float*)t, face, (float*)out.sh, (float*)out.cocg, (float*)out.luma,
                (float*)out.aosky, stats);
        return cudaGetLastError();
    }
    if (fp16)
        launch_diffuse<__half>(one, tex, tile_grid(W, H), s, w, cam, W, H, a, t, face, out, stats);
    else
        launch_diffuse<float>(one, tex, tile_grid(W, H), s, w, cam, W, H, a, t, face, out, stats);
    return cudaGetLastError();
}

}  // namespace vpt
