/* libvpt -- GB300-native VoxelPathTracer hot path, C ABI.
 *
 * The reference (swr06/VoxelPathTracer) drives its hot path from
 * Core/Pipeline.cpp through OpenGL objects: a voxel 3-D texture and a block
 * table SSBO go in, framebuffer colour attachments come out. This header is
 * the drop-in boundary for those passes: the same contracts over device
 * buffers owned by a context, plain pointers and sizes, no C++ or torch types.
 *
 * Conventions
 *   - Every call returns vpt_status; nothing throws across the ABI.
 *   - One context per host thread. Calls are ordered on the context's CUDA
 *     stream; calls that return data to host memory synchronise it.
 *   - Voxel volumes are uint8 block ids (0 = air), x fastest:
 *     index = x + X*(y + Y*z) (Core/World.h:46-49).
 *   - Image planes are W*H pixels, row 0 at the bottom (OpenGL convention),
 *     channels interleaved per pixel.
 *   - Matrices are column-major float[16] (glm layout).
 */
#ifndef VPT_H
#define VPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VPT_ABI_VERSION 3

typedef enum vpt_status {
    VPT_OK = 0,
    VPT_ERR_INVALID_ARG = 1,     /* bad pointer, size or enum value */
    VPT_ERR_OOM = 2,             /* device or host allocation failed */
    VPT_ERR_DEVICE_TIMEOUT = 3,  /* a bounded device-side wait gave up */
    VPT_ERR_CUDA = 4,            /* a CUDA runtime call failed */
    VPT_ERR_STATE = 5,           /* call out of order (e.g. trace before a world) */
    VPT_ERR_NO_DEVICE = 6        /* no usable CUDA device */
} vpt_status;

typedef enum vpt_storage {
    VPT_STORAGE_F32 = 0,         /* plain path: fp32 planes */
    VPT_STORAGE_F16 = 1          /* precision variant: fp16 planes, fp32 arithmetic */
} vpt_storage;

typedef struct vpt_ctx vpt_ctx;

/* Frame-loop settings; the reference keeps these as static globals at the
 * top of Core/Pipeline.cpp (:17-320). */
typedef struct vpt_config {
    int32_t width, height;           /* G-buffer resolution (GI: over gi_divisor) */
    int32_t primary_max_steps;       /* u_RenderDistance (Core/Pipeline.cpp:55, clamped to 350 at :4824) */
    int32_t shadow_max_steps;        /* 350 (ShadowRayTraceFrag.glsl:233) */
    int32_t diffuse_max_steps;       /* u_DiffuseTraceLength = 48 (Core/Pipeline.cpp:75) */
    int32_t bounce_shadow_max_steps; /* 128 (DiffuseRayTraceFrag.glsl:1220) */
    int32_t bounces;                 /* MAX_BOUNCE_LIMIT (DiffuseRayTraceFrag.glsl:17) */
    int32_t spp;                     /* u_SPP */
    int32_t storage;                 /* vpt_storage */
    int32_t atrous_iterations;       /* 5 (Core/Pipeline.cpp:2499) */
    float resolution_scale;          /* u_ResolutionScale (DiffuseIndirectSuperSampleRes, :79) */
    float color_phi_bias;            /* ColorPhiBias = 3.325 (:85) */
    int32_t device;                  /* CUDA device ordinal */
    int32_t denoiser;                /* vpt_denoiser: USE_SVGF (Core/Pipeline.cpp:84) true or false */
    int32_t gi_divisor;              /* 1 (or 0), 2, 4 ...: DiffuseTraceResolution = DiffuseIndirectSuperSampleRes
                                        = 1 / gi_divisor (Core/Pipeline.cpp:72, :79; 4 by default, 2 in the
                                        higher presets :1256-1282); width and height must be multiples */
    int32_t reflection_spp;          /* 0: no reflection pass (no specular indirect in the colour pass);
                                        else ReflectionSPP (Core/Pipeline.cpp:103, 2), 1..16. The
                                        reflections run on the GI grid (ReflectionTraceResolution = 1/4
                                        = DiffuseTraceResolution by default, :101) */
    int32_t reflection_max_steps;    /* u_ReflectionTraceLength = 64 (:100) */
    int32_t reflection_shadow_max_steps; /* 150 (ReflectionTraceFrag.glsl:1098) */
    int32_t reflection_temporal;     /* TEMPORAL_SPEC (Core/Pipeline.cpp:124): 1 (default) runs
                                        SpecularTemporalFilter's reprojection and accumulation */
    int32_t reflection_denoise;      /* DenoiseReflections (:105): 1 (default) runs the two separable
                                        passes of ReflectionDenoiserNew.glsl before the colour pass */
    int32_t alpha_test;              /* u_ShouldAlphaTest (Core/Pipeline.cpp:141, off by default): with block
                                        textures the primary trace passes through texels of transparent
                                        blocks whose albedo alpha is at most 0.975 */
    int32_t alpha_test_shadows;      /* ShouldAlphaTestShadows (Core/Pipeline.cpp:142, off by default): the
                                        same for the sun-shadow rays */
    int32_t reserved[1];
} vpt_config;

typedef enum vpt_denoiser {
    VPT_DENOISER_SVGF = 0,           /* Core/Pipeline.cpp:2284-2615 (default) */
    VPT_DENOISER_ATROUS = 1          /* temporal + 5x5 a-trous path, Core/Pipeline.cpp:2618-2786 */
} vpt_denoiser;

/* Camera uniforms: u_View, u_Projection, u_InverseView, u_InverseProjection
 * and u_ViewerPosition as Core/Pipeline.cpp sets them per pass. */
typedef struct vpt_camera {
    float view[16];
    float proj[16];
    float inv_view[16];
    float inv_proj[16];
    float position[3];
    float pad;
} vpt_camera;

/* One block-table entry. Replaces the BlockDataSSBO texture-layer arrays
 * (Core/BlockDataSSBO.cpp:9-35) with flat material values. */
typedef struct vpt_block {
    uint8_t albedo[3];
    uint8_t roughness;
    uint8_t metalness;
    uint8_t emissive;                /* 0 or 1 */
} vpt_block;

/* Per-frame uniforms of the trace, filter and colour passes. */
typedef struct vpt_frame {
    float sun_dir[3];                /* normalised, towards the sun (u_SunDirection) */
    float time;                      /* u_Time in seconds (filter jitter noise) */
    float sun_radiance[3];           /* colour-pass sun colour (SAMPLED_SUN_COLOR) */
    uint32_t frame_index;            /* per-pixel random stream index */
    float moon_radiance[3];          /* colour-pass moon colour */
    uint32_t seed;                   /* random seed */
    float gi_sun_strength;           /* GISunStrength = 1.0 (Core/Pipeline.cpp:280) */
    float gi_sky_strength;           /* GISkyStrength = 1.125 (:281) */
    float diffuse_light_intensity;   /* DiffuseLightIntensity = 1.25 (:74) */
    int32_t temporal;                /* DO_SVGF_TEMPORAL -> u_BeUseful */
} vpt_frame;

/* Image planes owned by the context (see vpt_plane_info for sizes). */
typedef enum vpt_plane {
    VPT_PLANE_T = 0,          /* hit distance (o_HitDistance), storage type, 1 ch */
    VPT_PLANE_FACE = 1,       /* face id 0..5 (+Z,-Z,+Y,-Y,-X,+X), 10 = miss; u8 */
    VPT_PLANE_BLOCK = 2,      /* block id at the hit, 0 = miss; u8 */
    VPT_PLANE_HIT = 3,        /* ivec3(floor(origin)) at loop exit; i32 x3 */
    VPT_PLANE_STEPS = 4,      /* DDA iterations; u16 */
    VPT_PLANE_SHADOW = 5,     /* sun shadow 0/1; u8 */
    VPT_PLANE_GI_SH = 6,      /* DiffuseRawTraceFBO: SH (4), CoCg (2), luma (1), AO+sky (2) */
    VPT_PLANE_GI_COCG = 7,
    VPT_PLANE_GI_LUMA = 8,
    VPT_PLANE_GI_AOSKY = 9,
    VPT_PLANE_PRE_SH = 10,    /* DiffusePreTemporal_SpatialFBO */
    VPT_PLANE_PRE_COCG = 11,
    VPT_PLANE_PRE_LUMA = 12,
    VPT_PLANE_PRE_AOSKY = 13,
    VPT_PLANE_TEMP_SH = 14,   /* DiffuseTemporalFBO of this frame; util = frames, moment, luma, 0 */
    VPT_PLANE_TEMP_COCG = 15,
    VPT_PLANE_TEMP_UTIL = 16,
    VPT_PLANE_TEMP_AOSKY = 17,
    VPT_PLANE_HIST_SH = 18,   /* PrevDiffuseTemporalFBO (history from the last frame) */
    VPT_PLANE_HIST_COCG = 19,
    VPT_PLANE_HIST_UTIL = 20,
    VPT_PLANE_HIST_AOSKY = 21,
    VPT_PLANE_PREV_T = 22,    /* InitialTraceFBOPrev */
    VPT_PLANE_PREV_FACE = 23,
    VPT_PLANE_PREV_BLOCK = 24,
    VPT_PLANE_VAR_SH = 25,    /* VarianceFBO */
    VPT_PLANE_VAR_COCG = 26,
    VPT_PLANE_VAR_VARIANCE = 27,
    VPT_PLANE_DEN_SH = 28,    /* output of the last a-trous iteration */
    VPT_PLANE_DEN_COCG = 29,
    VPT_PLANE_DEN_VARIANCE = 30,
    VPT_PLANE_DEN_AOSKY = 31,
    VPT_PLANE_COLOR = 32,     /* ColoredFBO: RGB radiance */
    VPT_PLANE_SPEC = 33,      /* ReflectionTraceFBO: reflected radiance RGB + 1 (4 ch), GI grid */
    VPT_PLANE_SPEC_HIT = 34,  /* its mean hit distance, -1 when every sample missed */
    VPT_PLANE_SPEC_MASK = 35, /* 1 where a sample hit an emissive block */
    VPT_PLANE_SPEC_OUT = 36,  /* ReflectionTemporalFBO: the specular indirect the colour pass reads */
    VPT_PLANE_SPEC_ACC = 37,  /* its accumulation factor (-1 with the temporal filter off) */
    VPT_PLANE_SPEC_STABLE_HIT = 38, /* its temporally stabilised hit distance */
    VPT_PLANE_SPEC_DEN = 39,  /* ReflectionDenoised_2: the spatially denoised reflection (4 ch) */
    VPT_PLANE_GB_ALBEDO = 40, /* GBuffer (GenerateGBuffer.glsl): albedo RGB (3 ch), with block textures */
    VPT_PLANE_GB_NORMAL = 41, /* normal-mapped normal (3 ch) */
    VPT_PLANE_GB_PBR = 42,    /* roughness, metalness, displacement, emissivity (4 ch) */
    VPT_PLANE_GB_AO = 43,     /* texture ambient occlusion (1 ch) */
    VPT_PLANE_COUNT = 44
} vpt_plane;

typedef enum vpt_dtype { VPT_DTYPE_F32 = 0, VPT_DTYPE_F16 = 1, VPT_DTYPE_U8 = 2, VPT_DTYPE_U16 = 3, VPT_DTYPE_I32 = 4 } vpt_dtype;

/* Counters filled while statistics are enabled (vpt_set_stats). */
typedef struct vpt_stats {
    uint64_t rays[6];                /* primary, sun shadow, diffuse, bounce shadow, reflection,
                                        reflection-hit shadow */
    uint64_t steps[6];               /* DDA iterations per ray kind */
} vpt_stats;

/* Per-pass device times of the last frame, from CUDA events on the
 * context stream (vpt_set_profiling). */
typedef enum vpt_pass {
    VPT_PASS_PRIMARY = 0, VPT_PASS_SHADOW = 1, VPT_PASS_DIFFUSE = 2, VPT_PASS_SPATIAL_INITIAL = 3,
    VPT_PASS_TEMPORAL = 4, VPT_PASS_VARIANCE = 5, VPT_PASS_ATROUS = 6, VPT_PASS_SHADE = 7,
    VPT_PASS_TRACE_FRAME = 8,        /* fused primary + shadow + diffuse (vpt_trace_frame) */
    VPT_PASS_LEARNED = 9,            /* features + U-Net + colour write-back (vpt_render_frame_learned) */
    VPT_PASS_REFLECTION = 10,        /* reflection trace + firefly rejection (vpt_trace_reflections) */
    VPT_PASS_GBUFFER = 11,           /* textured G-buffer (vpt_generate_gbuffer) */
    VPT_PASS_COUNT = 12
} vpt_pass;

/* Launch-shape knobs of the fused trace kernel, picked by the autotuner. */
typedef struct vpt_tuning {
    int32_t refill_threshold;        /* waiting lanes that trigger a warp refill, 1..32 (default 16) */
    int32_t trace_blocks;            /* persistent blocks of 128 threads; 0 = fill every SM once */
    int32_t fused_trace;             /* vpt_render_frame traces with vpt_trace_frame (1) or the three passes (0, default) */
    int32_t fused_prefilter;         /* SVGF runs Spatial3x3Initial inside the temporal kernel (1) or as its own
                                        launch before it (0, default: measured faster); the same planes either way */
    int32_t overlap_shadow;          /* vpt_render_frame* run the sun-shadow pass on a second stream beside the
                                        diffuse trace and SVGF, joined before the reflection and colour passes (1,
                                        default: 1.878 against 1.916 ms per 1080p frame), or in line (0) */
    int32_t split_temporal;          /* with overlap_shadow, GI on the G-buffer's grid, no block textures and the
                                        pre-filter unfused: the temporal pass's history gather runs on the second
                                        stream too, ahead of the shadow pass, and only its blend with the
                                        pre-filtered planes after the pre-filter (1), or the pass in one kernel (0,
                                        default: 1.620 against 1.647 ms per 1080p frame, the gather competing with
                                        the diffuse trace for the SMs and adding 64 bytes a texel each way) */
    int32_t reserved[2];
} vpt_tuning;

/* ------------------------------------------------------------- lifetime -- */
const char* vpt_status_string(vpt_status s);
int vpt_abi_version(void);
/* Defaults of the reference's frame loop for a 1920x1080 frame with 1 spp and 1 bounce. */
vpt_status vpt_default_config(vpt_config* cfg);
vpt_status vpt_default_frame(vpt_frame* frame);
/* Replaces MainPipeline::StartPipeline's FBO creation (Core/Pipeline.cpp:1094-1158, :1690-1735). */
vpt_status vpt_create(vpt_ctx** out, const vpt_config* cfg);
vpt_status vpt_destroy(vpt_ctx* ctx);
const char* vpt_last_error(const vpt_ctx* ctx);

/* ----------------------------------------------------------------- world -- */
/* World::Buffer -> Texture3D::CreateTexture (Core/World.h:167-171, Core/Texture3D.cpp:19-27):
 * copies X*Y*Z voxels to the device. Dimensions are runtime values (the
 * reference fixes them at compile time, Core/Macros.h:3-5). */
vpt_status vpt_upload_world(vpt_ctx* ctx, const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z);
/* BlockDataSSBO::CreateBuffers (Core/BlockDataSSBO.cpp:5-37); n <= 256. */
vpt_status vpt_set_block_table(vpt_ctx* ctx, const vpt_block* table, int32_t n);
/* World::GenerateDistanceField (Core/World.cpp:69-113). */
vpt_status vpt_build_df(vpt_ctx* ctx);

/* Block texture arrays: the four GL_TEXTURE_2D_ARRAYs of BlockDatabase
 * (Core/BlockDatabase.cpp:60-90, Core/GLClasses/TextureArray.cpp:10-78) and
 * the per-block layer indices of BlockDataSSBO (Core/BlockDataSSBO.cpp:9-35)
 * with GenerateGBuffer's grass override (u_GrassBlockProps,
 * Core/Pipeline.cpp:2086-2095). Every array is `layers` square layers of
 * `size` x `size` texels (size a power of two, 1..1024), row-major, row 0 at
 * t = 0. Mip levels are built on the device (each texel the rounded mean of
 * the 2 x 2 texels above it, per 8-bit channel). */
typedef struct vpt_block_textures {
    int32_t size;
    const uint8_t* albedo;           /* RGBA8, sRGB-encoded colour (an sRGB_ALPHA array) */
    int32_t albedo_layers;
    const uint8_t* normal;           /* RGBA8: tangent-space normal * 0.5 + 0.5 */
    int32_t normal_layers;
    const uint8_t* pbr;              /* RGBA8: roughness, metalness, displacement, AO */
    int32_t pbr_layers;
    const uint8_t* emissive;         /* R8, or NULL (no block emits through a texture) */
    int32_t emissive_layers;
    int32_t albedo_id[128];          /* layer of each block id's texture (BlockAlbedoData) */
    int32_t normal_id[128];          /* BlockNormalData */
    int32_t pbr_id[128];             /* BlockPBRData */
    int32_t emissive_id[128];        /* BlockEmissiveData; -1 = none */
    int32_t grass[10];               /* grass block id, then albedo / normal / PBR layers of
                                        its top (1-3), sides (4-6) and bottom (7-9); id -1 = none */
    int32_t transparent[128];        /* BlockTransparentData: 1 for blocks the alpha test looks through */
} vpt_block_textures;
/* Uploads the arrays and builds their mip chains; NULL removes them (flat
 * materials from the block table). Allocates the G-buffer texture planes. */
vpt_status vpt_set_block_textures(vpt_ctx* ctx, const vpt_block_textures* textures);
/* GenerateGBuffer.glsl main (:347-419; parallax mapping off, its default
 * Core/Pipeline.cpp:264, no lava block): albedo, normal-mapped normal, PBR and
 * texture AO of this frame's G-buffer hits, from the block textures sampled
 * with textureGrad at the face UV (trilinear, the LOD from the quad
 * derivatives of the UV). Needs vpt_set_block_textures and vpt_trace_primary. */
vpt_status vpt_generate_gbuffer(vpt_ctx* ctx);
/* Block edit (World::SetBlock followed by the distance-field rebuild it
 * triggers, Core/World.cpp:372-374, :458-460): writes the x-fastest voxels of
 * the box [x0,x0+w) x [y0,y0+h) x [z0,z0+d) (w*h*d bytes) into the world and,
 * when the field is built, recomputes it only within L1 distance 254 of the
 * box; the result is bit-identical to vpt_build_df of the edited world. */
vpt_status vpt_edit_world(vpt_ctx* ctx, const uint8_t* voxels, int32_t x0, int32_t y0, int32_t z0, int32_t w,
                          int32_t h, int32_t d);
vpt_status vpt_read_df(vpt_ctx* ctx, uint8_t* host_df, size_t bytes);
/* Context-free form: device pointers in and out, ordered on `stream`
 * (a cudaStream_t, 0 = legacy default stream). The device must be current. */
vpt_status vpt_df_build_device(const uint8_t* d_voxels, uint8_t* d_df, int32_t X, int32_t Y, int32_t Z, void* stream);

/* ---------------------------------------------------------------- passes -- */
/* Initial trace pass, Core/Pipeline.cpp:1959-2016 (InitialRayTraceFrag.glsl):
 * fills T, FACE, BLOCK, HIT, STEPS. Stores `cam` as this frame's camera. */
vpt_status vpt_trace_primary(vpt_ctx* ctx, const vpt_camera* cam);
/* Sun shadow pass, Core/Pipeline.cpp:2790-2850 (ShadowRayTraceFrag.glsl): fills SHADOW. */
vpt_status vpt_trace_shadow(vpt_ctx* ctx, const vpt_frame* frame);
/* Diffuse GI pass, Core/Pipeline.cpp:2169-2281 (DiffuseRayTraceFrag.glsl): fills GI_*. */
vpt_status vpt_trace_diffuse(vpt_ctx* ctx, const vpt_frame* frame);
/* SVGF, Core/Pipeline.cpp:2284-2615: Spatial3x3Initial, temporal, variance
 * and the a-trous iterations. `prev_cam` is the previous frame's camera
 * (u_PrevView / u_PrevProjection); history planes are read and written. */
vpt_status vpt_svgf(vpt_ctx* ctx, const vpt_camera* prev_cam, const vpt_frame* frame);
/* Reflection pass, Core/Pipeline.cpp:2998-3440: ReflectionTraceFrag.glsl,
 * the two bilateral passes over its hit distance, SpecularTemporalFilter
 * (firefly rejection; reprojection and accumulation when reflection_temporal)
 * and, with reflection_denoise, the x and y passes of ReflectionDenoiserNew,
 * on the GI grid, after vpt_svgf (it reads the denoised GI): fills SPEC,
 * SPEC_HIT, SPEC_MASK, SPEC_OUT, SPEC_ACC, SPEC_STABLE_HIT and SPEC_DEN. Needs
 * reflection_spp > 0; vpt_render_frame runs it when that is set. The
 * reflection planes are swapped with last frame's by vpt_end_frame. */
vpt_status vpt_trace_reflections(vpt_ctx* ctx, const vpt_frame* frame);
/* Colour pass, Core/Pipeline.cpp:3603-3821 (ColorPassFrag.glsl): fills COLOR;
 * with reflection_spp > 0 it adds the specular indirect from SPEC_OUT. */
vpt_status vpt_shade(vpt_ctx* ctx, const vpt_frame* frame);
/* The three trace passes of a frame in one persistent kernel: fills T, FACE,
 * BLOCK, HIT, STEPS, SHADOW and GI_* exactly as vpt_trace_primary,
 * vpt_trace_shadow and vpt_trace_diffuse would. Stores `cam` as this frame's
 * camera. */
vpt_status vpt_trace_frame(vpt_ctx* ctx, const vpt_camera* cam, const vpt_frame* frame);
/* Device buffers of one frame trace, owned by the caller. Every plane, the
 * GI planes included, holds cfg->width x cfg->height pixels (the fused trace
 * has no coarser GI grid: cfg->gi_divisor must be 0 or 1). Layouts as the
 * planes of vpt_plane_info: t and gi_* in cfg->storage's type (fp32 or fp16),
 * hit 3 x int32 per pixel, gi_sh 4, gi_cocg 2, gi_luma 1, gi_aosky 2 channels. */
typedef struct vpt_trace_buffers {
    const uint8_t* voxels;           /* X*Y*Z block ids, x fastest */
    const uint8_t* df;               /* their distance field (vpt_df_build_device) */
    int32_t X, Y, Z;
    const vpt_block* blocks;
    int32_t n_blocks;
    void* t;
    uint8_t* face;
    uint8_t* block;
    int32_t* hit;
    uint16_t* steps;
    uint8_t* shadow;
    void* gi_sh;
    void* gi_cocg;
    void* gi_luma;
    void* gi_aosky;
} vpt_trace_buffers;

/* No counterpart in the reference: vpt_trace_frame for callers that cannot
 * allocate device memory while rendering (engines that carve all GPU memory
 * out of a fixed start-up budget, or frame loops that cannot absorb
 * cudaMalloc's implicit device synchronisation). It allocates nothing: the
 * caller passes every input and output as device pointers, and the kernel's
 * only scratch, its work-queue counter, sits in a 256-byte static device
 * array of libvpt that every GPU using the library holds until the process
 * exits. The first call on a device looks that array's address up (with the
 * device current) and keeps it, so a device that was reset with
 * cudaDeviceReset must not be used with this call again in that process.
 * Images are limited to 16384 x 16384 and gi_divisor > 1 is rejected
 * (VPT_ERR_INVALID_ARG). All calls share the
 * array, which is reset at the start of each call: calls that overlap on the
 * GPU race, so issue them on one stream (or otherwise order them). The
 * current device and `stream` (a cudaStream_t, 0 = legacy default) are the
 * caller's; refill threshold 16 and a grid that fills every SM once. */
vpt_status vpt_trace_frame_noalloc(const vpt_trace_buffers* buffers, const vpt_config* cfg, const vpt_camera* cam,
                                   const vpt_frame* frame, void* stream);
vpt_status vpt_set_tuning(vpt_ctx* ctx, const vpt_tuning* tuning);
vpt_status vpt_get_tuning(const vpt_ctx* ctx, vpt_tuning* tuning);
/* Ping-pong swap of the G-buffer and temporal history (Core/Pipeline.cpp:1775-1788, :1970-1971). */
vpt_status vpt_end_frame(vpt_ctx* ctx);
/* Clears the history so the next frame starts without reprojection. */
vpt_status vpt_reset_history(vpt_ctx* ctx);
/* One whole frame: trace_frame, SVGF, shade, end_frame. If
 * rgb_out is not NULL the COLOR plane is copied to it as float32 RGB
 * (W*H*3 floats) and the call waits for it. prev_cam may be NULL on the
 * first frame (the camera of the previous call is used otherwise). */
vpt_status vpt_render_frame(vpt_ctx* ctx, const vpt_camera* cam, const vpt_frame* frame, float* rgb_out);
/* The same frame with a double-buffered readback: the COLOR plane is copied
 * to rgb_out (float32 RGB, W*H*3; page-locked host memory lets the copy run
 * asynchronously) on a copy stream while the next call's frame is computed.
 * The call returns once the PREVIOUS call's image is complete, so one frame
 * is in flight; vpt_readback_wait completes the last one. rgb_out must stay
 * valid until then. */
vpt_status vpt_render_frame_async(vpt_ctx* ctx, const vpt_camera* cam, const vpt_frame* frame, float* rgb_out);
/* Waits for the readback of the last vpt_render_frame_async call. */
vpt_status vpt_readback_wait(vpt_ctx* ctx);

/* The colour pass from the denoised GI (source 0, as vpt_shade), from the
 * temporally accumulated GI before any spatial filter (source 1) or from
 * this frame's raw GI (source 2). */
vpt_status vpt_shade_from(vpt_ctx* ctx, const vpt_frame* frame, int32_t source);

/* High-spp ground truth of the diffuse GI over the crop [x0, x0+w) x [y0, y0+h)
 * of the frame whose primary rays were traced last (fp32 contexts only): spp
 * samples of the diffuse path per pixel (DiffuseRayTraceFrag.glsl:535-664),
 * each on its own random stream derived from `seed`, accumulated per pixel
 * with an FP64 Welford mean and M2 of SH (4), CoCg (2) and AO (1) in that
 * channel order, in chunks of `chunk` samples merged in a fixed order.
 * mean_out and m2_out receive w*h*7 doubles each (row-major crop). No
 * counterpart in the reference (its quality reference is the screen). */
vpt_status vpt_ground_truth(vpt_ctx* ctx, const vpt_frame* frame, int32_t x0, int32_t y0, int32_t w, int32_t h,
                            int32_t spp, int32_t chunk, uint32_t seed, double* mean_out, double* m2_out);

/* Minecraft Anvil import, Core/NBT/Importer.cpp ImportWorld: every .mca region
 * file in `directory`, pre-flattening chunks (Level / xPos, zPos / Sections
 * with Y, Blocks, Data), a voxel stored only where its data value is 0,
 * mapped through mcid_to_block (the reference's BlockDatabase MinecraftIDLUT:
 * 0 must map to 0), placed at (x, y, z) - origin + (192, 0, 192) in the
 * reference's 384 x 128 x 384 world (x fastest, out_bytes >= 384*128*384).
 * Chunks in the 1.13+ palette layout are skipped. *chunks_read (optional)
 * counts the decoded chunks. No device needed. */
vpt_status vpt_import_mca_world(const char* directory, const uint8_t mcid_to_block[256], const float origin[3],
                                uint8_t* out, size_t out_bytes, int32_t* chunks_read);

/* ---------------------------------------------------------------- planes -- */
vpt_status vpt_plane_info(const vpt_ctx* ctx, int32_t plane, size_t* bytes, int32_t* channels, int32_t* dtype);
/* vpt_read_plane / vpt_write_plane of the SPEC_* planes need reflection_spp > 0
 * (VPT_ERR_STATE otherwise: they are not allocated). */
/* Width and height of a plane: the G-buffer's for the G-buffer, shadow and
 * colour planes, the GI grid's (width / gi_divisor x height / gi_divisor)
 * for the GI, temporal, variance and a-trous planes. */
vpt_status vpt_plane_dims(const vpt_ctx* ctx, int32_t plane, int32_t* width, int32_t* height);
vpt_status vpt_read_plane(vpt_ctx* ctx, int32_t plane, void* host, size_t bytes);
vpt_status vpt_write_plane(vpt_ctx* ctx, int32_t plane, const void* host, size_t bytes);
/* Device address of a plane (for callers that keep data on the GPU). */
vpt_status vpt_plane_device_ptr(vpt_ctx* ctx, int32_t plane, void** dptr);

/* ------------------------------------------------------ instrumentation -- */
vpt_status vpt_synchronize(vpt_ctx* ctx);
vpt_status vpt_set_stats(vpt_ctx* ctx, int32_t enabled);
vpt_status vpt_read_stats(vpt_ctx* ctx, vpt_stats* out);   /* synchronises, then zeroes */
vpt_status vpt_set_profiling(vpt_ctx* ctx, int32_t enabled);
vpt_status vpt_read_pass_times(vpt_ctx* ctx, float* ms, int32_t n);   /* synchronises */
/* Kernels launched by this context since it was created. */
vpt_status vpt_launch_count(const vpt_ctx* ctx, uint64_t* out);
/* The context's stream as a cudaStream_t. */
vpt_status vpt_get_stream(const vpt_ctx* ctx, void** stream);

/* Deterministic math used by every kernel (exp, exp2, log2, pow, sin, cos as
 * op 0..5), evaluated on the device (on_device = 1) or on the host; lets a
 * caller check that both give identical bits. y is read for pow and ops 6..17.
 * Ops 6..14 check the filters' packed fp32 pairs lane by lane: x * y (6, 7:
 * lanes 0 and 1), x + y (8, 9), exp(x) from the packed exponential (10, 11),
 * the weighted sum x + y * x (12) and the bilinear blends of one and two
 * channels (13, 14) of the values (x, 2x, -x, y) at weights (fract(y),
 * fract(2y)), x / 5 in the variance estimate's three-operation form (15),
 * and exp(x) from the packed exponential for non-positive arguments (16, 17;
 * x and y must be <= 0 or NaN). */
vpt_status vpt_detmath(int32_t op, const float* x, const float* y, float* out, int32_t n, int32_t on_device);

/* -------------------------------------------------------- batched worlds --
 * Many independent worlds traced together. The reference renders one World
 * per process (Core/Pipeline.cpp's frame loop over one World, Core/World.h:193-199);
 * a batch holds many such worlds, each with its own volume, distance field,
 * block table, camera and ray tile, and traces the primary, sun-shadow and
 * one diffuse bounce (with its shadow ray) of every world in one persistent
 * launch. Per world, the planes are bit-identical to vpt_trace_primary /
 * vpt_trace_shadow / vpt_trace_diffuse of a context holding that world alone.
 * All planes are float32 (no FP16 storage in a batch). */
typedef struct vpt_batch vpt_batch;

typedef struct vpt_batch_config {
    int32_t device;
    int32_t max_worlds;              /* 1..1024 */
    int32_t primary_max_steps;       /* same meaning as in vpt_config */
    int32_t shadow_max_steps;
    int32_t diffuse_max_steps;
    int32_t bounce_shadow_max_steps;
    int32_t bounces;                 /* 0..8 */
    int32_t spp;                     /* 1..32 */
    int32_t reserved[4];
} vpt_batch_config;

/* Launch shape of the persistent batch kernel (vpt_batch_autotune picks it). */
typedef struct vpt_batch_tuning {
    int32_t block_threads;           /* 64..512, a multiple of 32 */
    int32_t tiles_per_grab;          /* 8x4-pixel tile pairs (rays_per_lane 2) or tiles a warp takes per queue
                                        access, 1..16 */
    int32_t df_brick;                /* distance-field layout traced: 0 x-fastest, 4 or 8 = B^3-voxel bricks */
    int32_t blocks;                  /* persistent blocks; 0 = every SM filled to its occupancy limit */
    int32_t rays_per_lane;           /* 1: a warp traces 32 pixels at a time; 2: 64 (two tiles of one world), each
                                        lane's two primary and two shadow traversals interleaved */
    int32_t phased;                  /* 0: one persistent kernel runs the primary, shadow and diffuse passes of a
                                        tile; 1 (rays_per_lane 1): three persistent kernels, one per pass, each
                                        pass's code alone on the SMs */
    int32_t reserved[2];
} vpt_batch_tuning;

typedef struct vpt_batch_tune_record {
    vpt_batch_tuning tuning;
    float ms;                        /* median device time of one persistent launch */
    float pad;
} vpt_batch_tune_record;

typedef enum vpt_batch_mode {
    VPT_BATCH_GRAPH = 0,             /* the persistent launch, replayed from a captured CUDA graph */
    VPT_BATCH_PERSISTENT = 1,        /* the persistent launch, launched directly */
    VPT_BATCH_PER_WORLD = 2          /* three pass kernels per world (the plain path), for comparison */
} vpt_batch_mode;

/* Batch planes (vpt_batch_read_plane) reuse the vpt_plane ids T, FACE, BLOCK,
 * HIT, STEPS, SHADOW, GI_SH, GI_COCG, GI_LUMA and GI_AOSKY. */
vpt_status vpt_batch_default_config(vpt_batch_config* cfg);
vpt_status vpt_batch_create(vpt_batch** out, const vpt_batch_config* cfg);
vpt_status vpt_batch_destroy(vpt_batch* batch);
const char* vpt_batch_last_error(const vpt_batch* batch);
/* Adds a world (x-fastest voxels, each edge 1..1024) with its block table
 * (1..256 entries) and a width x height ray tile (each 1..4096); returns its
 * index in *world_id. Invalidates the distance fields of the batch. */
vpt_status vpt_batch_add_world(vpt_batch* batch, const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z,
                               const vpt_block* table, int32_t n_blocks, int32_t width, int32_t height,
                               int32_t* world_id);
vpt_status vpt_batch_set_camera(vpt_batch* batch, int32_t world, const vpt_camera* cam);
/* Distance fields of every world (World::GenerateDistanceField per world), in
 * the x-fastest layout and in the brick layout the tuning selects. */
vpt_status vpt_batch_build_df(vpt_batch* batch);
/* Copies world `world`'s x-fastest distance field out (X*Y*Z bytes). */
vpt_status vpt_batch_read_df(vpt_batch* batch, int32_t world, uint8_t* host, size_t bytes);
vpt_status vpt_batch_set_tuning(vpt_batch* batch, const vpt_batch_tuning* tuning);
vpt_status vpt_batch_get_tuning(const vpt_batch* batch, vpt_batch_tuning* tuning);
/* Traces every world with its camera. Stream-ordered; returns without waiting. */
vpt_status vpt_batch_trace(vpt_batch* batch, const vpt_frame* frame, int32_t mode);
/* No counterpart in the reference: the read bandwidth (GB/s, median of
 * `reps` reads after two warm-ups) of a `bytes`-long device buffer (1 MiB ..
 * 4 GiB) that stays in L2 when it fits, read with 128-bit L2-cached loads on
 * `device` - the memory roof of the trace kernels, whose distance-field
 * gathers hit an L2-resident volume. Allocates and frees its buffer. */
vpt_status vpt_measure_l2_read(int32_t device, uint64_t bytes, int32_t reps, float* gbs);

/* Times every candidate launch shape (one kernel with rays_per_lane 1 or 2, or
 * the phased launch; x block_threads 128/256/512 x tiles_per_grab 1/2/4 x
 * df_brick 0/4/8: 81 in all) on the batch as it stands, `reps`
 * timed launches each after one warm-up, keeps the fastest as the batch's
 * tuning and writes up to max_records records (all candidates, in the order
 * tried). Synchronises. */
vpt_status vpt_batch_autotune(vpt_batch* batch, const vpt_frame* frame, int32_t reps, vpt_batch_tune_record* records,
                              int32_t max_records, int32_t* n_records);
vpt_status vpt_batch_read_plane(vpt_batch* batch, int32_t world, int32_t plane, void* host, size_t bytes);
vpt_status vpt_batch_world_info(const vpt_batch* batch, int32_t world, int32_t dims[3], int32_t tile[2]);
vpt_status vpt_batch_count(const vpt_batch* batch, int32_t* n_worlds);
vpt_status vpt_batch_synchronize(vpt_batch* batch);
vpt_status vpt_batch_set_stats(vpt_batch* batch, int32_t enabled);
vpt_status vpt_batch_read_stats(vpt_batch* batch, vpt_stats* out);   /* synchronises, then zeroes */
vpt_status vpt_batch_launch_count(const vpt_batch* batch, uint64_t* out);
vpt_status vpt_batch_get_stream(const vpt_batch* batch, void** stream);

/* ----------------------------------------------------- learned denoiser --
 * No counterpart in the reference (its denoisers are the SVGF and a-trous
 * passes of Core/Pipeline.cpp:2284-2786). A 3-level U-Net (32/64/96
 * channels, 3x3 convolutions, ReLU, 2x2 average pooling, nearest upsampling
 * with skip concatenation) on the tcgen05 tensor cores: BF16 weights and
 * activations (NHWC, channels padded to multiples of 16), FP32 accumulation.
 * Input: 16 channels (11 features + 5 zero); output: 16 FP32 channels of
 * which 0..2 are the prediction. Image sizes must be multiples of 4. */
typedef struct vpt_unet vpt_unet;

/* Raw operators over caller device pointers, enqueued on `stream` (a
 * cudaStream_t) on the current device. conv3x3: out = act(conv(in) + bias),
 * in = channels [0,c0) of in0 (nearest-upsampled from half size when up0 = 1)
 * followed by channels [0,c1) of in1; weight [cout][9][c0+c1] BF16, tap =
 * (dy+1)*3 + (dx+1); relu 0/1; out zeroed where mask <= 0 if mask is given;
 * BF16 and/or FP32 output [n*h*w][cout]. conv3x3_dw adds
 * dW[co][tap][ci] = sum_p dy[p][co] in[p+tap][ci] to the FP32 dw.
 * vpt_nn_status synchronises `stream` and reports a timed-out tensor-core
 * wait as VPT_ERR_DEVICE_TIMEOUT. */
vpt_status vpt_nn_conv3x3(const void* in0, int32_t c0, int32_t up0, const void* in1, int32_t c1, int32_t n, int32_t h,
                          int32_t w, const void* weight, const float* bias, int32_t cout, int32_t relu,
                          const void* mask, void* out_bf16, float* out_f32, void* stream);
vpt_status vpt_nn_conv3x3_dw(const void* in0, int32_t c0, int32_t up0, const void* in1, int32_t c1, int32_t n,
                             int32_t h, int32_t w, const void* dy, int32_t cout, float* dw, void* stream);
vpt_status vpt_nn_status(void* stream);

/* Layer `layer` (0..10) of the network: padded input/output channels, real
 * ones, and the offset of its weights [cout][9][cin] (then bias [cout]) in
 * the flat FP32 parameter vector. */
vpt_status vpt_unet_layer_info(int32_t layer, int32_t* cin, int32_t* cout, int32_t* cin_real, int32_t* cout_real,
                               int64_t* offset);
/* Capacity: up to max_images images of max_height x max_width pixels. */
vpt_status vpt_unet_create(vpt_unet** out, int32_t device, int32_t max_images, int32_t max_height, int32_t max_width);
vpt_status vpt_unet_destroy(vpt_unet* unet);
const char* vpt_unet_last_error(const vpt_unet* unet);
vpt_status vpt_unet_param_count(const vpt_unet* unet, int64_t* n);
vpt_status vpt_unet_set_params(vpt_unet* unet, const float* host, int64_t n);   /* also resets Adam */
vpt_status vpt_unet_get_params(vpt_unet* unet, float* host, int64_t n);
vpt_status vpt_unet_get_grads(vpt_unet* unet, float* host, int64_t n);
/* Inference of n images (device input [n][h][w][16] BF16); the output stays
 * in the network's buffer (vpt_unet_output) and is copied to `out` (device,
 * [n][h][w][16] FP32) when not NULL. Stream-ordered on the network's stream. */
vpt_status vpt_unet_forward(vpt_unet* unet, const void* input, int32_t n, int32_t h, int32_t w, float* out);
vpt_status vpt_unet_output(vpt_unet* unet, const float** out);
/* Forward + backward of the mean squared error of output channels 0..2
 * against `target` (device [n][h][w][3] FP32); the parameter gradient is kept
 * for vpt_unet_adam / vpt_unet_get_grads. Synchronises when loss is not NULL. */
vpt_status vpt_unet_backward(vpt_unet* unet, const void* input, const float* target, int32_t n, int32_t h, int32_t w,
                             double* loss);
vpt_status vpt_unet_adam(vpt_unet* unet, float lr, float beta1, float beta2, float eps);
vpt_status vpt_unet_synchronize(vpt_unet* unet);   /* also reports timed-out waits */
vpt_status vpt_unet_get_stream(const vpt_unet* unet, void** stream);

/* The learned frame path on a context (SVGF denoiser configured):
 * vpt_learned_input traces the frame, runs the SVGF pre-filter, temporal and
 * variance passes and shades from the temporal GI (COLOR then holds the
 * network's noisy input); the frame stays open until vpt_end_frame.
 * vpt_learned_features writes the 16-channel BF16 features of a crop
 * ([h][w][16], device dst): log(1 + noisy RGB), block albedo, face normal,
 * min(hit distance, 512) / 128, log(1 + SVGF variance), log(1 + RGB shaded
 * from this frame's raw 1-spp GI), two zeros.
 * vpt_render_frame_learned renders a whole frame with the network as the
 * spatial denoiser, which predicts a log-space correction of the noisy colour
 * (COLOR = exp(log(1 + noisy) + out) - 1), and falls back to the SVGF path
 * (5 a-trous iterations) when net is NULL or the image size is not a
 * multiple of 4; *used_net tells which ran. rgb_out as in vpt_render_frame. */
vpt_status vpt_learned_input(vpt_ctx* ctx, const vpt_camera* cam, const vpt_frame* frame);
vpt_status vpt_learned_features(vpt_ctx* ctx, int32_t x0, int32_t y0, int32_t w, int32_t h, void* dst);
vpt_status vpt_render_frame_learned(vpt_ctx* ctx, vpt_unet* net, const vpt_camera* cam, const vpt_frame* frame,
                                    float* rgb_out, int32_t* used_net);

/* ---------------------------------------------------------- host helpers -- */
/* Seeded value-noise terrain (heightmap h = 40 + 16*fbm, 4 octaves, base
 * frequency 1/64, gain 0.5; grass top, three dirt layers, stone below) with
 * surface blocks 4..n_blocks-1 scattered on 1 column in 16. Host only. */
vpt_status vpt_generate_world(uint8_t* out, int32_t X, int32_t Y, int32_t Z, uint64_t seed, int32_t n_blocks);
/* Seeded flat block table: albedo, roughness, metalness uniform, 5% emissive. */
vpt_status vpt_generate_block_table(vpt_block* out, int32_t n, uint64_t seed);
/* World files (Core/WorldFileHandler.cpp:10-83). The reference's .sav is the
 * raw x-fastest volume, X*Y*Z bytes, no header (dimensions fixed at compile
 * time): header = 0 writes exactly that; header = 1 prefixes a 32-byte header
 * ("VPTWORLD", version 1, X, Y, Z, seed; little endian). vpt_load_world reads
 * either: with a header `dims` (and `seed`) are filled from it, a raw file
 * needs `dims` from the caller. Truncated, oversized or malformed files give
 * VPT_ERR_INVALID_ARG. out = NULL only checks the file and reports dims. */
vpt_status vpt_save_world(const char* path, const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z, uint64_t seed,
                          int32_t header);
vpt_status vpt_load_world(const char* path, uint8_t* out, size_t out_bytes, int32_t dims[3], uint64_t* seed);
/* Emissive voxels of a world, as LoadWorld's light list (:50-66): x, y, z per
 * voxel in x-fastest order, at most max_out written, *count = all of them. */
vpt_status vpt_emissive_voxels(const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z, const vpt_block* table,
                               int32_t n_blocks, int32_t* xyz_out, int64_t max_out, int64_t* count);
/* glm::lookAt / glm::perspective camera as Core/FpsCamera.cpp:14-24 builds it
 * (front from yaw/pitch in degrees), inverses in double precision. */
vpt_status vpt_camera_from_pose(vpt_camera* out, const float position[3], float yaw_deg, float pitch_deg,
                                float fov_deg, float aspect, float znear, float zfar);

#ifdef __cplusplus
}
#endif
#endif /* VPT_H */
