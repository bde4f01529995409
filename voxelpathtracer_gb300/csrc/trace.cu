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
    pdl_enter();
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
    pdl_enter();
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
    pdl_enter();
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

// The same pass for one sample and one bounce, staged inside the CTA so that
// rays of one kind fill whole warps (DiffuseRayTraceFrag.glsl main :822-935,
// CalculateDiffuse :535-664 with one bounce):
//   0. sky texels (no G-buffer hit) are written at once; texels with a hit are
//      appended to a list in shared memory (ballot + one atomic per warp, so
//      each warp's 8x4 patch stays together);
//   1. one thread per listed texel traces its bounce ray and records the hit
//      and, when the hit faces the sun, a sun-shadow ray request;
//   2. one thread per request traces the shadow ray (about one bounce in
//      eight needs one: without this stage nearly every warp would wait for a
//      few lanes' shadow rays);
//   3. one thread per listed texel finishes the sample from the recorded hit
//      and shadow verdict and writes the GI planes.
// Outputs and ray counts are those of k_trace_diffuse. A block covers kR
// 16x16 tiles stacked in y (a thread lists kR texels and works through the
// listed ones kR at a time): with two, each lane's work is the sum of two
// bounce rays' step counts, which differ less from lane to lane than single
// ones, and a block's shadow-request stage fills more of its warps.
template <typename S, bool kTex, int kR>
__global__ void __launch_bounds__(256, 6) k_trace_diffuse_staged(WorldView w, CamView cam, int W, int H,
                                                                  DiffuseArgs a, const S* t, const uint8_t* face,
                                                                  S* o_sh, S* o_cocg, S* o_luma, S* o_aosky,
                                                                  Counters* stats) {
    constexpr int N = 256 * kR;             // texels of the block: a 16 x 16kR tile
    pdl_enter();
    __shared__ uint32_t s_pix[N];           // listed texels: i | j << 16
    __shared__ float s_bt[N];               // their bounce hit distance
    __shared__ uint8_t s_bface[N], s_bblock[N], s_shadow[N];
    __shared__ float4 s_ray[N];             // shadow ray origin xyz, w = listed texel
    __shared__ int s_n[2];                  // listed texels, shadow requests
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < 2) s_n[tid] = 0;
    __syncthreads();
    GICount cnt = {0u, 0u, 0u, 0u};
#pragma unroll 1
    for (int r = 0; r < kR; r++) {
        const int i = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
        const int j = blockIdx.y * 16 * kR + r * 16 + (warp >> 1) * 4 + (lane >> 3);
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
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        int base = 0;
        if (lane == 0 && m) base = atomicAdd(&s_n[0], __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (hit) s_pix[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i | ((uint32_t)j << 16);
    }
    __syncthreads();
    const int n_hit = s_n[0];
#pragma unroll 1
    for (int k0 = 0; k0 < n_hit; k0 += 256) {   // uniform rounds; lane k = k0 + tid
        const int k = k0 + tid;
        bool need = false;
        v3 so;
        if (k < n_hit) {
            const int i = (int)(s_pix[k] & 0xffffu), j = (int)(s_pix[k] >> 16);
            const size_t px = (size_t)j * W + i;
            StagedBounce sb;
            diffuse_pixel<0, S, true, kTex, kDiffuseBounceOnly>(w, cam, W, H, i, j, a, px, ld(t + px),
                                                                __ldg(face + px), o_sh, o_cocg, o_luma, o_aosky, &cnt,
                                                                &sb, &need, &so);
            s_bt[k] = sb.t;
            s_bface[k] = (uint8_t)sb.face;
            s_bblock[k] = (uint8_t)sb.block;
            s_shadow[k] = 0;
        }
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&s_n[1], __popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) s_ray[base + __popc(m & ((1u << lane) - 1u))] = make_float4(so.x, so.y, so.z, __int_as_float(k));
        }
    }
    __syncthreads();
    const int n_sh = s_n[1];
#pragma unroll 1
    for (int k = tid; k < n_sh; k += 256) {
        // GetShadowAt (DiffuseRayTraceFrag.glsl:1202-1222)
        const float4 r = s_ray[k];
        const GILighting& L = a.lighting;
        const TraceResult sr = traverse<0>(w, mk3(r.x, r.y, r.z), mk3(L.light_dir[0], L.light_dir[1], L.light_dir[2]),
                                           a.bounce_shadow_max_steps);
        cnt.shadow_rays += 1;
        cnt.shadow_steps += (unsigned)sr.steps;
        s_shadow[__float_as_int(r.w)] = sr.t > 0.0f ? 1 : 0;
    }
    __syncthreads();
#pragma unroll 1
    for (int k = tid; k < n_hit; k += 256) {
        const int i = (int)(s_pix[k] & 0xffffu), j = (int)(s_pix[k] >> 16);
        const size_t px = (size_t)j * W + i;
        StagedBounce sb{s_bt[k], (int)s_bface[k], (int)s_bblock[k]};
        diffuse_pixel<0, S, true, kTex, kDiffuseGiven>(w, cam, W, H, i, j, a, px, ld(t + px), __ldg(face + px), o_sh,
                                                       o_cocg, o_luma, o_aosky, &cnt, &sb, nullptr, nullptr,
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
    pdl_launch(table[(one ? 2 : 0) + (tex ? 1 : 0)], grid, 256, 0, s, w, cam, W, H, a, (const S*)t, face, (S*)out.sh,
               (S*)out.cocg, (S*)out.luma, (S*)out.aosky, stats);
}

}  // namespace

cudaError_t trace_primary(const WorldView& w, const CamView& cam, int W, int H, int max_steps, int fp16,
                          GBufferOut out, Counters* stats, cudaStream_t s, const AlphaStop* alpha) {
    const AlphaStop st = alpha ? *alpha : AlphaStop{};
    if (fp16)
        pdl_launch((alpha ? k_trace_primary<__half, true> : k_trace_primary<__half, false>), tile_grid(W, H), 256, 0, s,
            w, cam, W, H, max_steps, (__half*)out.t, out.face, out.block, out.hit, out.steps, stats, st);
    else
        pdl_launch((alpha ? k_trace_primary<float, true> : k_trace_primary<float, false>), tile_grid(W, H), 256, 0, s,
            w, cam, W, H, max_steps, (float*)out.t, out.face, out.block, out.hit, out.steps, stats, st);
    return cudaGetLastError();
}

cudaError_t trace_shadow(const WorldView& w, const CamView& cam, int W, int H, int max_steps, const float sun[3],
                         int fp16, const void* t, const uint8_t* face, uint8_t* shadow, Counters* stats,
                         cudaStream_t s, const AlphaStop* alpha) {
    const AlphaStop st = alpha ? *alpha : AlphaStop{};
    if (fp16)
        pdl_launch((alpha ? k_trace_shadow<__half, true> : k_trace_shadow<__half, false>), tile_grid(W, H), 256, 0, s,
            w, cam, W, H, max_steps, sun[0], sun[1], sun[2], (const __half*)t, face, shadow, stats, st);
    else
        pdl_launch((alpha ? k_trace_shadow<float, true> : k_trace_shadow<float, false>), tile_grid(W, H), 256, 0, s,
            w, cam, W, H, max_steps, sun[0], sun[1], sun[2], (const float*)t, face, shadow, stats, st);
    return cudaGetLastError();
}

cudaError_t trace_diffuse(const WorldView& w, const CamView& cam, int W, int H, const DiffuseArgs& a, int fp16,
                          const void* t, const uint8_t* face, GIOut out, Counters* stats, cudaStream_t s) {
    const bool one = a.spp <= 1 && !a.lighting.moon_stronger, tex = a.textured != 0;
    if (one && a.bounces == 1 && W < 65536 && H < 65536) {
        // 16x32 texels per block where that still gives every SM two waves
        // of its six resident blocks (the 1080p frame: 1.668 -> 1.658 ms),
        // else 16x16 (a 480x270 GI grid has too few blocks for two waves)
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const unsigned gx = (unsigned)((W + 15) / 16), gy2 = (unsigned)((H + 31) / 32);
        const bool two = (long long)gx * gy2 >= 2LL * 6 * (sms > 0 ? sms : 1);
        const dim3 g(gx, two ? gy2 : (unsigned)((H + 15) / 16));
        if (fp16) {
            using K = void (*)(WorldView, CamView, int, int, DiffuseArgs, const __half*, const uint8_t*, __half*,
                               __half*, __half*, __half*, Counters*);
            const K k = two ? (tex ? k_trace_diffuse_staged<__half, true, 2> : k_trace_diffuse_staged<__half, false, 2>)
                            : (tex ? k_trace_diffuse_staged<__half, true, 1> : k_trace_diffuse_staged<__half, false, 1>);
            pdl_launch(k, g, 256, 0, s, w, cam, W, H, a, (const __half*)t, face, (__half*)out.sh, (__half*)out.cocg,
                       (__half*)out.luma, (__half*)out.aosky, stats);
        } else {
            using K = void (*)(WorldView, CamView, int, int, DiffuseArgs, const float*, const uint8_t*, float*, float*,
                               float*, float*, Counters*);
            const K k = two ? (tex ? k_trace_diffuse_staged<float, true, 2> : k_trace_diffuse_staged<float, false, 2>)
                            : (tex ? k_trace_diffuse_staged<float, true, 1> : k_trace_diffuse_staged<float, false, 1>);
            pdl_launch(k, g, 256, 0, s, w, cam, W, H, a, (const float*)t, face, (float*)out.sh, (float*)out.cocg,
                       (float*)out.luma, (float*)out.aosky, stats);
        }
        return cudaGetLastError();
    }
    if (fp16)
        launch_diffuse<__half>(one, tex, tile_grid(W, H), s, w, cam, W, H, a, t, face, out, stats);
    else
        launch_diffuse<float>(one, tex, tile_grid(W, H), s, w, cam, W, H, a, t, face, out, stats);
    return cudaGetLastError();
}

}  // namespace vpt
