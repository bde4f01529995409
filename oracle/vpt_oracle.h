/* CPU oracle for the VoxelPathTracer hot path -- C API.
 *
 * TEST INFRASTRUCTURE ONLY: a C++17 restatement of the reference shaders
 * (Core/Shaders/ManhattanDistance{X,Y,Z}.comp, InitialRayTraceFrag.glsl,
 * ShadowRayTraceFrag.glsl, DiffuseRayTraceFrag.glsl, Spatial3x3Initial.glsl,
 * SVGF/{TemporalFilter,VarianceEstimate,SpatialFilter}.glsl, ColorPassFrag.glsl).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
 * as the checker or the timed CPU baseline; the product never does.
 *
 * Parity is unpinned by the reference itself: the reference has no tests,
 * golden vectors or CPU implementation of this path, and its GLSL needs an
 * OpenGL context. The oracle is pinned instead by analytic known-answer tests
 * (tests/test_oracle_kat.py) and brute-force cross-checks.
 *
 * Struct layouts match include/vpt.h byte for byte so the same host buffers
 * can be handed to both.
 */
#ifndef VPT_ORACLE_H
#define VPT_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct vpto_camera {
    float view[16];      /* column-major, m[col*4+row] */
    float proj[16];
    float inv_view[16];
    float inv_proj[16];
    float position[3];
    float pad;
} vpto_camera;

typedef struct vpto_block {
    uint8_t albedo[3];
    uint8_t roughness;
    uint8_t metalness;
    uint8_t emissive;
} vpto_block;

typedef struct vpto_frame {
    float sun_dir[3];
    float time;
    float sun_radiance[3];
    uint32_t frame_index;
    float moon_radiance[3];
    uint32_t seed;
    float gi_sun_strength;
    float gi_sky_strength;
    float diffuse_light_intensity;
    int32_t temporal;
} vpto_frame;

typedef struct vpto_params {
    int32_t width, height;
    int32_t primary_max_steps;
    int32_t shadow_max_steps;
    int32_t diffuse_max_steps;
    int32_t bounce_shadow_max_steps;
    int32_t bounces;
    int32_t spp;
    int32_t storage;            /* 0 = fp32 planes, 1 = fp16 planes */
    int32_t atrous_iterations;
    float resolution_scale;
    float color_phi_bias;
    int32_t device;
    int32_t denoiser;           /* 0 = SVGF, 1 = temporal + 5x5 a-trous */
    int32_t gi_divisor;         /* GI grid = G-buffer / gi_divisor (0 or 1: same grid) */
    int32_t reflection_spp;     /* reflection samples per texel (0: no reflection pass) */
    int32_t reflection_max_steps;
    int32_t reflection_shadow_max_steps;
    int32_t reflection_temporal;  /* TEMPORAL_SPEC */
    int32_t reflection_denoise;   /* DenoiseReflections */
    int32_t alpha_test;           /* u_ShouldAlphaTest */
    int32_t alpha_test_shadows;   /* ShouldAlphaTestShadows */
    int32_t reserved[1];
} vpto_params;

typedef struct vpto_world {
    const uint8_t* vox;
    const uint8_t* df;
    int32_t X, Y, Z;
    const vpto_block* blocks;
    int32_t n_blocks;
} vpto_world;

/* Planes consumed / produced by the passes (W*H pixels, row 0 = bottom). */
typedef struct vpto_gbuffer {
    float* t;          /* hit distance, -1 on miss */
    uint8_t* face;     /* 0..5 (+Z,-Z,+Y,-Y,-X,+X), 10 on miss */
    uint8_t* block;    /* block id at the hit, 0 on miss */
    int32_t* hit;      /* 3 per pixel: ivec3(floor(origin)) at loop exit */
    uint16_t* steps;   /* DDA iterations executed */
} vpto_gbuffer;

typedef struct vpto_gi {   /* DiffuseRawTraceFBO-like planes */
    float* sh;         /* 4 per pixel */
    float* cocg;       /* 2 per pixel */
    float* luma;       /* 1 per pixel (o_Utility) */
    float* aosky;      /* 2 per pixel */
} vpto_gi;

typedef struct vpto_history {   /* DiffuseTemporalFBO-like planes */
    float* sh;
    float* cocg;
    float* util;       /* 4 per pixel: accumulated frames, moment, luma, 0 */
    float* aosky;
} vpto_history;

typedef struct vpto_filtered {  /* VarianceFBO / DiffuseDenoiseFBO-like planes */
    float* sh;
    float* cocg;
    float* variance;
    float* aosky;      /* unused by the variance pass */
} vpto_filtered;

int vpto_omp_threads(void);
/* Counters (12 x uint64: rays then DDA steps for primary, shadow, diffuse,
 * bounce shadow, reflection, reflection shadow) that the trace functions add
 * to; NULL disables counting. */
void vpto_set_counters(uint64_t* counters);

/* ManhattanDistance{X,Y,Z}.comp driven as in World::GenerateDistanceField. */
void vpto_build_df(const uint8_t* vox, int X, int Y, int Z, uint8_t* df);

/* InitialRayTraceFrag.glsl main, rows [row0, row1). */
void vpto_trace_primary(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                        int row0, int row1, vpto_gbuffer* out);

/* ShadowRayTraceFrag.glsl main (hard sun shadow, one ray per pixel). */
void vpto_trace_shadow(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                       const vpto_frame* f, const float* t, const uint8_t* face,
                       int row0, int row1, uint8_t* shadow);

/* The G-buffer as the GI passes read it at their own texel centres when the
 * GI grid is gi_divisor times coarser: texture() of the depth (bilinear) and
 * nearest face and block at each GI texel centre, the depth stored in the
 * storage type. With gi_divisor 1 this is the G-buffer itself. */
void vpto_gi_view(const vpto_params* p, const float* t, const uint8_t* face, const uint8_t* block,
                  float* t_view, uint8_t* face_view, uint8_t* block_view);

/* Passes below that take t / face / block "views" read them on the GI grid
 * (vpto_gi_view); prev_t / prev_face / prev_block and the a-trous pass's
 * t / face are the full-resolution G-buffer, sampled at arbitrary points.
 * GI planes are (width / gi_divisor) x (height / gi_divisor). */

/* DiffuseRayTraceFrag.glsl main with CalculateDiffuse, on the GI grid
 * (rows of the GI grid). */
void vpto_trace_diffuse(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                        const vpto_frame* f, const float* t, const uint8_t* face,
                        int row0, int row1, vpto_gi* out);

/* Spatial3x3Initial.glsl */
void vpto_spatial_initial(const vpto_camera* cam, const vpto_params* p,
                          const float* t, const uint8_t* face, const vpto_gi* in, vpto_gi* out);

/* SVGF/TemporalFilter.glsl */
/* The oracle's vector builtins (dot, cross, length, normalize, mix, mat4 *
 * vec4) over n inputs, for the comparison with the reference's glm. */
void vpto_vecmath(int op, const float* a, const float* b, const float* c, float* out, int n);
/* The SH / YCoCg encoding of a diffuse sample (op 0: radiance (3) and
 * direction (3) per item in, SH (4) and CoCg (2) out) and its decoding for a
 * normal (op 1: SH (4), CoCg (2) and normal (3) in, irradiance (3) out), over
 * n items, for the comparison with the reference's shader functions. */
void vpto_sh_codec(int op, int n, const float* in, float* out);
/* The Hammon diffuse BRDF of a bounce ray over n items (normal (3), incident
 * direction (3), new direction (3), roughness in; DiffuseRayBRDF's value out). */
void vpto_diffuse_brdf(int n, const float* in, float* out);
/* Inputs x (bit patterns in [lo, hi)) for which q = x * RN(1/c) corrected once
   by the exact remainder, fma(fma(-q, c, x), RN(1/c), q), differs from x / c. */
uint64_t vpto_check_div_const(float c, uint32_t lo, uint32_t hi);
/* ProjectPositionPrevious / Reprojection (SVGF/TemporalFilter.glsl:61-73) of
 * every texel of the W x H hit-distance plane t, as the temporal pass computes
 * them: the world position (3 floats per texel) and the previous frame's
 * texture coordinate (2 floats per texel). */
void vpto_reproject(const vpto_camera* cam, const vpto_camera* prev_cam, int W, int H, const float* t, float* pos,
                    float* uv_prev);
void vpto_temporal(const vpto_camera* cam, const vpto_camera* prev_cam, const vpto_params* p,
                   const vpto_frame* f,
                   const float* t, const uint8_t* face, const uint8_t* block,
                   const float* prev_t, const uint8_t* prev_face, const uint8_t* prev_block,
                   const vpto_gi* cur, const vpto_history* prev, vpto_history* out);

/* SVGF/VarianceEstimate.glsl */
void vpto_variance(const vpto_camera* cam, const vpto_params* p,
                   const float* t, const uint8_t* face, const vpto_history* in, vpto_filtered* out);

/* SVGF/SpatialFilter.glsl, one a-trous iteration with step `step`. */
void vpto_atrous(const vpto_camera* cam, const vpto_params* p, const vpto_frame* f, int step,
                 const float* t, const uint8_t* face, const float* t_view, const uint8_t* face_view,
                 const float* temporal_util,
                 const vpto_filtered* in, const float* in_aosky, vpto_filtered* out);

/* ReflectionTraceFrag.glsl main on the GI grid: t / face / shadow are the
 * full-resolution G-buffer and sun shadow, the views the GI-grid reading of
 * the G-buffer, den_* the denoised diffuse GI. Writes spec (4 ch), hit and
 * mask on the GI grid, rows [row0, row1) of it. */
void vpto_trace_reflection(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                           const float* t, const uint8_t* face, const uint8_t* shadow, const float* t_view,
                           const uint8_t* face_view, const uint8_t* block_view, const float* den_sh,
                           const float* den_cocg, const float* den_aosky, int row0, int row1, float* spec,
                           float* hit, float* mask);
/* The two bilateral passes over the reflection hit distance (pass 1 or 2). */
void vpto_spec_hit_blur(const vpto_params* p, int pass, const float* t_view, const uint8_t* face_view,
                        const float* hit_in, float* hit_out);
/* SpecularTemporalFilter.glsl (firefly rejection, reprojection by the hit
 * distance, clipping, accumulation; TEMPORAL_SPEC = reflection_temporal). prev_*
 * are last frame's full-resolution G-buffer and its reflection planes. */
void vpto_spec_temporal(const vpto_world* w, const vpto_camera* cam, const vpto_camera* prev_cam,
                        const vpto_params* p, const float* t_view, const uint8_t* face_view,
                        const uint8_t* block_view, const float* prev_t, const uint8_t* prev_face,
                        const float* spec, const float* hit, const float* mask, const float* prev_out,
                        const float* prev_hit, const float* prev_stable, float* out, float* acc, float* stable);

/* ReflectionDenoiserNew.glsl, one separable pass (dir 1: x, 0: y): t / face
 * / block the full-resolution G-buffer, the views its GI-grid reading, in the
 * reflection (4 ch), hit_data the (stabilised) hit distance, frames the
 * temporal accumulation factor; all but the G-buffer on the GI grid. */
void vpto_spec_denoise(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, int dir, const float* t,
                       const uint8_t* face, const uint8_t* block, const float* t_view, const uint8_t* face_view,
                       const uint8_t* block_view, const float* in, const float* hit_data, const float* frames,
                       float* out);

/* ColorPassFrag.glsl main: joint-bilateral GI upscale, direct GGX +
 * indirect-diffuse combine, flat materials. t / face / block / shadow at the
 * G-buffer's resolution, sh / cocg / aosky on the GI grid. */
void vpto_shade(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                const vpto_frame* f, const float* t, const uint8_t* face, const uint8_t* block,
                const uint8_t* shadow, const float* sh, const float* cocg, const float* aosky,
                const float* spec, int row0, int row1, float* rgb);

/* The colour pass with block textures: albedo (3), normal-mapped normal (3),
 * PBR (4) and texture AO (1) from the textured G-buffer (W*H each). */
void vpto_shade_textured(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                         const float* t, const uint8_t* face, const uint8_t* block, const uint8_t* shadow,
                         const float* sh, const float* cocg, const float* aosky, const float* spec, int row0, int row1,
                         float* rgb, const float* gb_albedo, const float* gb_normal, const float* gb_pbr,
                         const float* gb_ao);

/* The non-SVGF denoiser path (USE_SVGF off, Core/Pipeline.cpp:2618-2786):
 * TemporalFilter.glsl (diffuse mode), SampleVarianceCompute.glsl and one
 * AtrousSpatialFilter.glsl iteration. */
void vpto_plain_temporal(const vpto_camera* cam, const vpto_camera* prev_cam, const vpto_params* p,
                         const float* t, const float* prev_t, const vpto_gi* cur, const vpto_history* prev,
                         vpto_history* out);
void vpto_plain_variance(const vpto_params* p, const float* sh, float* variance);
void vpto_plain_atrous(const vpto_camera* cam, const vpto_params* p, int step, const float* t, const uint8_t* face,
                       const uint8_t* block, const float* sh, const float* cocg, const float* aosky, float* out_sh,
                       float* out_cocg, float* out_aosky);

/* High-spp FP64 Welford ground truth of the diffuse GI over a crop
 * (channels SH 4, CoCg 2, AO), as vpt_ground_truth computes it. */
void vpto_ground_truth(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                       const float* t, const uint8_t* face, int x0, int y0, int cw, int ch, int spp, int chunk,
                       uint32_t seed, double* mean_out, double* m2_out);

/* Block texture arrays, laid out as vpt_block_textures (level-0 texels;
 * the oracle builds the mip levels itself). */
typedef struct vpto_block_textures {
    int32_t size;
    const uint8_t* albedo;
    int32_t albedo_layers;
    const uint8_t* normal;
    int32_t normal_layers;
    const uint8_t* pbr;
    int32_t pbr_layers;
    const uint8_t* emissive;
    int32_t emissive_layers;
    int32_t albedo_id[128];
    int32_t normal_id[128];
    int32_t pbr_id[128];
    int32_t emissive_id[128];
    int32_t grass[10];
    int32_t transparent[128];
} vpto_block_textures;

/* Block textures for the diffuse bounce hits of vpto_trace_diffuse (and the
 * ground truth); NULL returns to the block table's flat materials. */
void vpto_set_block_textures(const vpto_block_textures* tx);

/* The textured G-buffer (normal 3 ch, PBR 4 ch, W*H) the reflection passes
 * read instead of the block table and the face normals; NULLs turn it off.
 * The pointers must stay valid while the passes run. */
void vpto_set_textured_gbuffer(const float* normal, const float* pbr, int W, int H);

/* GenerateGBuffer.glsl main (parallax off, no lava): albedo (3), normal (3),
 * PBR (4) and texture AO (1) per pixel of the W x H G-buffer. */
void vpto_generate_gbuffer(const vpto_camera* cam, const vpto_params* p, const vpto_block_textures* tx,
                           const float* t, const uint8_t* face, const uint8_t* block, float* albedo, float* normal,
                           float* pbr, float* ao);

/* Deterministic math, exported so tests can check its error bounds. */
float vpto_exp(float x);
float vpto_exp2(float x);
float vpto_log2(float x);
float vpto_pow(float x, float y);
float vpto_sin(float x);
float vpto_cos(float x);
float vpto_half_round(float x);

#ifdef __cplusplus
}
#endif
#endif
