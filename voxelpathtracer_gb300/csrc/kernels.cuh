// Launch interfaces of the libvpt kernels (one translation unit per group).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace vpt {

// Programmatic dependent launch for the frame's kernel chain. A kernel
// launched by pdl_launch may be scheduled onto the SMs its predecessor on the
// stream frees while that predecessor's last blocks still run; pdl_enter,
// the first statement of such a kernel, waits for the predecessor grid to
// complete (its writes visible) before any global access and then lets the
// kernel's own successor be scheduled early in turn. The wait is the
// hardware's grid dependency, not a spin, and the successor can only be
// scheduled once every block of this grid has started, so it never holds
// SM room this grid still needs. Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... KArgs, typename... Args>
cudaError_t pdl_launch(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// Device counters filled when statistics are on (layout of vpt_stats).
struct Counters {
    unsigned long long rays[6];
    unsigned long long steps[6];
};
enum RayKind {
    kRayPrimary = 0, kRayShadow = 1, kRayDiffuse = 2, kRayBounceShadow = 3, kRayReflection = 4,
    kRayReflectionShadow = 5
};

// ---------------------------------------------------------------- df.cu --
// Manhattan distance field, min(min(254, X+Y+Z), L1 distance to the nearest
// solid voxel): three sweeps along x, y and z. `launches` counts kernels.
cudaError_t df_build(const uint8_t* vox, uint8_t* df, int X, int Y, int Z, cudaStream_t s, int* launches);
// After the voxels of [ex0, ex1) x [ey0, ey1) x [ez0, ez1) changed: recompute
// the field where the edit can change it, bit-identical to df_build.
cudaError_t df_update(const uint8_t* vox, uint8_t* df, int X, int Y, int Z, int ex0, int ey0, int ez0, int ex1,
                      int ey1, int ez1, cudaStream_t s, int* launches);

// Per-frame constants of DiffuseRayTraceFrag main (:832-839), evaluated on
// the host with the shader's operation order.
inline GILighting gi_lighting(const vpt_frame* f) {
    const v3 SUN_COLOR = muls(divs(mk3(192.0f, 216.0f, 255.0f), 255.0f), 16.0f);
    const v3 NIGHT_COLOR = muls(divs(mk3(96.0f, 192.0f, 255.0f), 255.0f), 1.5f);
    const v3 DUSK_COLOR = muls(divs(mk3(96.0f, 192.0f, 255.0f), 255.0f), 0.9f);
    v3 sun = mk3(f->sun_dir[0], f->sun_dir[1], f->sun_dir[2]);
    bool sun_stronger = -sun.y < 0.01f;
    float dusk = clampf(dpow(fabsf(sun.y - 1.0f), 2.9f), 0.0f, 1.0f);
    v3 sun_color = vmix(SUN_COLOR, DUSK_COLOR, dusk);
    v3 lc = sun_stronger ? sun_color : NIGHT_COLOR;
    lc = muls(lc, 0.4f * f->gi_sun_strength);
    v3 ld = sun_stronger ? sun : normalize(mk3(-sun.x, -sun.y, sun.z));
    GILighting L;
    L.light_color[0] = lc.x; L.light_color[1] = lc.y; L.light_color[2] = lc.z;
    L.light_dir[0] = ld.x; L.light_dir[1] = ld.y; L.light_dir[2] = ld.z;
    L.moon_stronger = sun_stronger ? 0 : 1;
    L.emissivity_multiplier = sun_stronger ? 12.0f : 13.0f;
    L.sun_visibility = clampf(dot(sun, mk3(0.0f, 1.0f, 0.0f)) + 0.05f, 0.0f, 0.1f) * 12.0f;
    L.gi_sky_strength = f->gi_sky_strength;
    L.diffuse_light_intensity = f->diffuse_light_intensity;
    return L;
}

// ------------------------------------------------------------- trace.cu --
struct GBufferOut {
    void* t;            // storage type
    uint8_t* face;
    uint8_t* block;
    int32_t* hit;       // 3 per pixel
    uint16_t* steps;
};
// One block texture array on the device: `layers` layers of `size`^2 texels
// of `channels` 8-bit channels per mip level, levels stored one after the
// other (level l: layers x (size >> l)^2 texels from element offset
// level_off[l] * channels).
struct TexArray {
    const uint8_t* texels;
    int layers, channels, size, levels;
    long long level_off[11];
};
// The arrays, the per-block layer ids [albedo 128 | normal 128 | PBR 128 |
// emissive 128 | transparent flag 128], the grass override and the byte -> value tables (256
// entries each: sRGB decode for albedo, byte / 255 for the others).
struct BlockTexView {
    TexArray albedo, normal, pbr, emissive;   // emissive.texels NULL: none
    const int* ids;
    int grass[10];
    const float* srgb;
    const float* unorm;   // byte / 255 (256 entries)
};
struct DiffuseArgs {
    int diffuse_max_steps;
    int bounce_shadow_max_steps;
    int bounces;
    int spp;
    uint32_t frame_index;
    uint32_t seed;
    GILighting lighting;
    // block textures for the bounce hits (textured = 0: the block table)
    int textured = 0;
    BlockTexView tex{};
};
struct GIOut {
    void* sh;           // 4 ch
    void* cocg;         // 2 ch
    void* luma;         // 1 ch
    void* aosky;        // 2 ch
};

struct AlphaStop;   // textures.cuh: StopRay of the alpha-tested traversal
// alpha: the alpha-tested traversal (u_ShouldAlphaTest), or NULL
cudaError_t trace_primary(const WorldView& w, const CamView& cam, int W, int H, int max_steps, int fp16,
                          GBufferOut out, Counters* stats, cudaStream_t s, const AlphaStop* alpha = nullptr);
cudaError_t trace_shadow(const WorldView& w, const CamView& cam, int W, int H, int max_steps, const float sun[3],
                         int fp16, const void* t, const uint8_t* face, uint8_t* shadow, Counters* stats,
                         cudaStream_t s, const AlphaStop* alpha = nullptr);
cudaError_t trace_diffuse(const WorldView& w, const CamView& cam, int W, int H, const DiffuseArgs& a, int fp16,
                          const void* t, const uint8_t* face, GIOut out, Counters* stats, cudaStream_t s);

// -------------------------------------------------------- trace_frame.cu --
// Every ray of a frame (primary, sun shadow, diffuse bounces and their
// shadow rays) in one persistent kernel; same outputs as the three passes.
struct FrameTraceArgs {
    WorldView w;
    CamView cam;
    int W, H;
    int tiles_x;             // 8x4 pixel tiles per row
    int n_items;             // tiles * 32 queue entries
    int primary_max_steps;
    int shadow_max_steps;
    float sun[3];
    int refill_threshold;    // waiting lanes that trigger a warp-wide refill (1..32)
    DiffuseArgs d;
    void* t;
    uint8_t* face;
    uint8_t* block;
    int32_t* hit;
    uint16_t* steps;
    uint8_t* shadow;
    void* sh;
    void* cocg;
    void* luma;
    void* aosky;
    int* queue;              // work counter, zero at launch
    Counters* stats;
};
// blocks_hint <= 0 sizes the grid to fill every SM once.
cudaError_t trace_frame(const FrameTraceArgs& a, int fp16, int blocks_hint, cudaStream_t s);

// -------------------------------------------------------------- batch.cu --
// Many worlds, each with its own camera and ray tile, traced in one
// persistent launch: warps take 8x4-pixel tiles of all worlds from one queue
// and run primary, sun-shadow and diffuse GI for their 32 pixels.
struct BatchWorld {
    WorldView w;              // df points at the layout the launch is built for
    CamView cam;
    int W, H;
    int tiles_x;              // 8x4 tiles per row
    int tile_begin;           // first queue entry of this world
    float* t;
    uint8_t* face;
    uint8_t* block;
    int32_t* hit;
    uint16_t* steps;
    uint8_t* shadow;
    float* sh;
    float* cocg;
    float* luma;
    float* aosky;
};
struct BatchFrame {           // per-frame constants, read from device memory
    int primary_max_steps;
    int shadow_max_steps;
    float sun[3];
    DiffuseArgs d;
};
struct BatchLaunch {
    const BatchWorld* worlds;
    const int* tile_begin;    // n_worlds + 1 prefix sums (tile_begin[n] = n_tiles)
    const BatchFrame* frame;
    int n_worlds;
    int n_tiles;
    int tiles_per_grab;       // queue entries a warp takes at once
    int* queue;               // zero at launch (the phased launch: one counter per pass, queue[0..2])
    Counters* stats;
};
constexpr int kBatchMaxWorlds = 1024;
// df_brick: 0, 4 or 8; blocks <= 0 fills every SM to its occupancy limit;
// phased: the primary, shadow and diffuse passes as three persistent kernels
// (rays_per_lane 1) instead of one.
// The phased launch's shadow pass may run on `side` beside the diffuse pass
// (forked after the primary pass with `fork`, joined with `join`).
struct BatchSide {
    cudaStream_t side;
    cudaEvent_t fork, join;
};
cudaError_t batch_trace(const BatchLaunch& a, int df_brick, int block_threads, int rays_per_lane, int blocks,
                        int phased, cudaStream_t s, const BatchSide* side = nullptr);
int batch_max_blocks(int df_brick, int block_threads, int rays_per_lane, int device);
// Copies an x-fastest distance field into the BxBxB brick layout of df_index.
cudaError_t df_to_bricks(const uint8_t* df, uint8_t* out, int X, int Y, int Z, int brick, cudaStream_t s);

// ------------------------------------------------------- groundtruth.cu --
// FP64 Welford accumulation of `spp` diffuse samples over a crop (fp32 G-buffer).
struct GroundTruthArgs {
    WorldView w;
    CamView cam;
    int W, H;
    DiffuseArgs d;
    const float* t;
    const uint8_t* face;
    int x0, y0, cw, ch;      // crop
    int spp, chunk, nchunks;
    uint32_t seed;
    double* part;            // cw*ch*nchunks records of (n, mean[7], m2[7])
    double* mean;            // cw*ch*7
    double* m2;              // cw*ch*7
};
cudaError_t ground_truth(const GroundTruthArgs& a, cudaStream_t s);

// -------------------------------------------------------------- svgf.cu --
struct GIIn {
    const void* sh;
    const void* cocg;
    const void* luma;
    const void* aosky;
};
struct HistIO {          // util has 4 channels: frames, moment, luma, 0
    void* sh;
    void* cocg;
    void* util;
    void* aosky;
};
struct FiltIO {
    void* sh;
    void* cocg;
    void* variance;
    void* aosky;
};
struct TemporalArgs {
    float prev_view_proj[16];   // u_PrevProjection * u_PrevView, evaluated on the host
    int be_useful;
};
struct AtrousArgs {
    int step;
    float add_scale;            // mix(1, 2.4, u_ResolutionScale)
    float phi_bias;             // max(u_ColorPhiBias, 0.1)
    float tmod500;              // mod(u_Time * 100.493850275, 500)
};

cudaError_t svgf_spatial_initial(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                                 GIIn in, GIOut out, cudaStream_t s);
// W x H: the GI grid; Wf x Hf: the G-buffer (equal unless the GI grid is coarser).
cudaError_t svgf_temporal(const CamView& cam, int W, int H, int Wf, int Hf, int fp16, const TemporalArgs& a,
                          const void* t, const uint8_t* face, const uint8_t* block,
                          const void* prev_t, const uint8_t* prev_face, const uint8_t* prev_block,
                          GIIn cur, HistIO prev, HistIO out, cudaStream_t s);
// Spatial3x3Initial and the temporal pass fused (one launch; the
// pre-filtered planes `pre` are written as svgf_spatial_initial writes them).
// The temporal pass split in two (GI on the G-buffer's grid): the history
// taps' sums into `sums` (64 bytes a texel), then their blend with the
// pre-filtered planes; together bit-identical to svgf_temporal.
cudaError_t svgf_temporal_gather(const CamView& cam, int W, int H, int fp16, const TemporalArgs& a, const void* t,
                                 const uint8_t* face, const uint8_t* block, const void* prev_t,
                                 const uint8_t* prev_face, const uint8_t* prev_block, HistIO prev, void* sums,
                                 cudaStream_t s);
cudaError_t svgf_temporal_blend(int W, int H, int fp16, const TemporalArgs& a, const void* sums, GIIn cur,
                                HistIO out, cudaStream_t s);
cudaError_t svgf_pre_temporal(const CamView& cam, int W, int H, int Wf, int Hf, int fp16, const TemporalArgs& a,
                              const void* t, const uint8_t* face, const uint8_t* block, const void* prev_t,
                              const uint8_t* prev_face, const uint8_t* prev_block, GIIn gi, GIOut pre, HistIO prev,
                              HistIO out, cudaStream_t s);
cudaError_t svgf_variance(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                          HistIO in, FiltIO out, cudaStream_t s);
cudaError_t svgf_atrous(const CamView& cam, int W, int H, int Wf, int Hf, int fp16, const AtrousArgs& a,
                        const void* t, const uint8_t* face, const void* tf, const uint8_t* ff,
                        const void* temporal_util, FiltIO in, const void* in_aosky, FiltIO out, cudaStream_t s);
// The G-buffer (W x H) read at the texel centres of the Wg x Hg GI grid.
cudaError_t gi_view(int W, int H, int Wg, int Hg, int fp16, const void* t, const uint8_t* face, const uint8_t* block,
                    void* tv, uint8_t* fv, uint8_t* bv, cudaStream_t s);

// ------------------------------------------------------ plain_filter.cu --
// The non-SVGF path: temporal -> variance -> `iterations` a-trous passes
// ping-ponging between out[0] and out[1] (the last one lands in
// out[(iterations - 1) & 1]).
struct PlainDenoiseIO {
    const void* t;         // this frame's depth on the GI grid
    const void* prev_t;    // the previous frame's depth at the G-buffer's Wf x Hf
    int Wf, Hf;
    const uint8_t* face;
    const uint8_t* block;
    GIIn cur;          // raw GI planes
    HistIO prev;       // last frame's temporal output (sh, cocg used)
    HistIO temporal;   // this frame's temporal output
    void* variance;
    FiltIO out[2];
    int iterations;
};
cudaError_t plain_denoise(const CamView& cam, int W, int H, int fp16, const TemporalArgs& ta,
                          const PlainDenoiseIO& io, cudaStream_t s);

// ----------------------------------------------------------- reflect.cu --
struct ReflectionArgs {
    int spp;                    // ReflectionSPP, 1..16
    int max_steps;              // u_ReflectionTraceLength
    int shadow_max_steps;       // 150
    uint32_t frame_index, seed;
    float view_proj[16];        // u_Projection * u_View
    float light_dir[3];         // u_StrongerLightDirection
    float mixed[3];             // SAMPLED_COLOR_MIXED: sun / moon radiance by sun visibility
    float viewer[3];            // u_ViewerPosition
    // with block textures: the textured G-buffer's normal-mapped normal (3 ch)
    // and PBR (4 ch) at W x H for the base pixel, and the arrays for the hits;
    // NULL / 0: the block table and the face normals
    const void* gb_normal = nullptr;
    const void* gb_pbr = nullptr;
    int textured = 0;
    BlockTexView tex{};
};
// W x H: the G-buffer (t, face, shadow); Wg x Hg: the GI grid (views, denoised
// GI, outputs spec 4 ch, hit, mask).
cudaError_t trace_reflection(const WorldView& w, const CamView& cam, int W, int H, int Wg, int Hg, int fp16,
                             const ReflectionArgs& a, const void* t, const uint8_t* face, const uint8_t* shadow,
                             const void* tv, const uint8_t* fv, const uint8_t* bv, const void* den_sh,
                             const void* den_cocg, const void* den_ao, void* spec, void* hit, void* mask,
                             Counters* stats, cudaStream_t s);
cudaError_t spec_hit_blur(int Wg, int Hg, int fp16, int pass, const void* tv, const uint8_t* fv, const void* hin,
                          void* hout, cudaStream_t s);
struct SpecTemporalArgs {
    float prev_view_proj[16];   // u_PrevProjection * u_PrevView
    float cur_pos[3], prev_pos[3];
    int temporal;               // TEMPORAL_SPEC
    const void* gb_pbr = nullptr;   // textured G-buffer PBR (4 ch, W x H), or NULL: the block table
};
struct SpecDenoiseArgs {
    float view[16];             // u_View
    float res_scale;            // u_ResolutionScale (ReflectionSuperSampleResolution) = 1 / gi_divisor
    int dir;                    // u_Dir: 1 = x, 0 = y
    int temporal_weight;        // u_TemporalWeight && TEMPORAL_SPEC
    const void* gb_normal = nullptr;   // textured G-buffer normal (3 ch) and PBR (4 ch) at W x H,
    const void* gb_pbr = nullptr;      // or NULL: face normals and the block table
};
cudaError_t spec_denoise(const WorldView& w, const CamView& cam, const SpecDenoiseArgs& a, int W, int H, int Wg,
                         int Hg, int fp16, const void* t, const uint8_t* face, const uint8_t* block, const void* tv,
                         const uint8_t* fv, const uint8_t* bv, const void* in, const void* hit_data,
                         const void* frames, void* out, cudaStream_t s);
cudaError_t spec_temporal(const WorldView& w, const CamView& cam, const SpecTemporalArgs& a, int W, int H, int Wg,
                          int Hg, int fp16, const void* tv, const uint8_t* fv, const uint8_t* bv, const void* prev_t,
                          const uint8_t* prev_face, const void* spec, const void* hit, const void* mask,
                          const void* prev_out, const void* prev_hit, const void* prev_stable, void* out, void* acc,
                          void* stable, cudaStream_t s);

// ------------------------------------------------------------- shade.cu --
struct ShadeArgs {
    float sun[3], moon[3];
    float sun_color[3], moon_color[3];
    float sun_vis;             // 1 - clamp(dot(sun, up) + 0.05, 0, 0.1) * 12
    int vxao;                  // u_DoVXAO && u_SVGFEnabled: the GI AO darkens the indirect term
    int gi_div;                // the GI planes are (W / gi_div) x (H / gi_div)
    // the textured G-buffer (albedo 3, normal 3, PBR 4, AO 1 channels in the
    // storage type), or all NULL: flat materials from the block table
    const void* gb_albedo = nullptr;
    const void* gb_normal = nullptr;
    const void* gb_pbr = nullptr;
    const void* gb_ao = nullptr;
};
// spec: the resolved reflection on the GI grid (4 ch), or NULL without a
// reflection pass.
cudaError_t shade(const WorldView& w, const CamView& cam, int W, int H, int fp16, const ShadeArgs& a,
                  const void* t, const uint8_t* face, const uint8_t* block, const uint8_t* shadow,
                  const void* sh, const void* cocg, const void* aosky, const void* spec, void* rgb, cudaStream_t s);

// ----------------------------------------------------------- learned.cu --
// 16-channel BF16 features of the crop [x0, x0+w) x [y0, y0+h) into out
// (w*h*16), and the network's FP32 output [W*H][16] back into the colour plane.
cudaError_t learned_features(int W, int H, int x0, int y0, int w, int h, int fp16, const void* color,
                             const void* color_raw, const void* t,
                             const uint8_t* face, const uint8_t* block, const vpt_block* blocks, int n_blocks,
                             const void* var, void* out, cudaStream_t s);
cudaError_t learned_unpack(int W, int H, int fp16, const float* net_out, void* color, cudaStream_t s);

// ---------------------------------------------------------- textures.cu --
// Level l + 1 of every layer from level l (rounded 2 x 2 mean per channel).
cudaError_t tex_build_mip(const TexArray& a, int level, uint8_t* texels, cudaStream_t s);
// GenerateGBuffer.glsl main over the W x H G-buffer: albedo (3), normal (3),
// PBR (4) and AO (1) planes in the storage type.
cudaError_t gbuffer_textured(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                             const uint8_t* block, const BlockTexView& tv, void* albedo, void* normal, void* pbr,
                             void* ao, cudaStream_t s);

// Deterministic-math probe: evaluates op `op` (0 exp, 1 exp2, 2 log2, 3 pow,
// 4 sin, 5 cos) over n inputs on the device.
cudaError_t detmath_eval(int op, const float* x, const float* y, float* out, int n, cudaStream_t s);

}  // namespace vpt
