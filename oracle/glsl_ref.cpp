// Drivers for the reference's own shader functions compiled as C++
// (oracle/build_glsl_ref.py writes them, rewritten mechanically, into
// oracle/_ref/glsl_ref_gen.inc). TEST INFRASTRUCTURE ONLY: they stand in for
// the dispatches and draws of the reference's frame loop, one invocation or
// fragment at a time, so tests/test_oracle_glsl_ref.py can compare the
// reference's code with the oracle on the same inputs. Volumes are x fastest.
#include <cstdint>
#include <cstring>

#include "glsl_compat.h"

namespace glsl {
#include "glsl_ref_gen.inc"
}  // namespace glsl

using namespace glsl;

namespace {
mat4 mat_from(const float* m) {
    mat4 r;
    for (int c = 0; c < 4; c++) r[c] = vec4(m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]);
    return r;
}
}  // namespace

extern "C" {

// World::GenerateDistanceField (Core/World.cpp:69-113): the X, Y and Z
// passes of ManhattanDistance{X,Y,Z}.comp over an R8 image, each invocation
// one line (invocations of a pass are independent, so their order is free).
// vox: X*Y*Z block ids; df: the X*Y*Z distances out.
void glslref_build_df(const uint8_t* vox, int X, int Y, int Z, uint8_t* df) {
    std::memset(df, 0, (size_t)X * Y * Z);
    df_x::WORLD_SIZE_X = X; df_x::WORLD_SIZE_Y = Y; df_x::WORLD_SIZE_Z = Z;
    df_y::WORLD_SIZE_X = X; df_y::WORLD_SIZE_Y = Y; df_y::WORLD_SIZE_Z = Z;
    df_z::WORLD_SIZE_X = X; df_z::WORLD_SIZE_Y = Y; df_z::WORLD_SIZE_Z = Z;
    df_x::u_BlockData = sampler3D{vox, X, Y, Z};
    df_x::o_DistanceBuffer = image3D{df, X, Y, Z};
    df_y::o_DistanceBuffer = image3D{df, X, Y, Z};
    df_z::o_DistanceBuffer = image3D{df, X, Y, Z};
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++) {
            df_x::gl_GlobalInvocationID = uvec3{0u, (unsigned)y, (unsigned)z};
            df_x::main();
        }
    for (int z = 0; z < Z; z++)
        for (int x = 0; x < X; x++) {
            df_y::gl_GlobalInvocationID = uvec3{(unsigned)x, 0u, (unsigned)z};
            df_y::main();
        }
    for (int y = 0; y < Y; y++)
        for (int x = 0; x < X; x++) {
            df_z::gl_GlobalInvocationID = uvec3{(unsigned)x, (unsigned)y, 0u};
            df_z::main();
        }
}

// The initial ray trace (Core/Pipeline.cpp:1977-2000, InitialRayTraceFrag.glsl
// main) over a W x H target, without TAA jitter or alpha testing. The
// fragment's v_TexCoords is the texel centre ((i + 0.5) / W, (j + 0.5) / H),
// what the full-screen quad's interpolation gives there. inv_view / inv_proj:
// column-major 4x4. Out: o_HitDistance, o_Normal and o_BlockID per texel.
void glslref_trace_primary(const uint8_t* vox, const uint8_t* df, int X, int Y, int Z, const float* inv_view,
                           const float* inv_proj, int W, int H, int render_distance, float fov_deg, float* o_t,
                           float* o_normal, float* o_block) {
    primary::WORLD_SIZE_X = X; primary::WORLD_SIZE_Y = Y; primary::WORLD_SIZE_Z = Z;
    primary::u_VoxelDataTexture = sampler3D{vox, X, Y, Z};
    primary::u_DistanceFieldTexture = sampler3D{df, X, Y, Z};
    primary::u_InverseView = mat_from(inv_view);
    primary::u_InverseProjection = mat_from(inv_proj);
    primary::u_Dimensions = vec2((float)W, (float)H);
    primary::u_RenderDistance = render_distance;
    primary::u_ShouldAlphaTest = false;
    primary::u_JitterSceneForTAA = false;
    primary::u_FOV = fov_deg;
    primary::u_Time = 0.0f;
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            primary::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            primary::main();
            const size_t px = (size_t)j * W + i;
            o_t[px] = primary::o_HitDistance;
            o_normal[px] = primary::o_Normal;
            o_block[px] = primary::o_BlockID;
        }
}

// The sun-shadow trace (Core/Pipeline.cpp:2796-2830, ShadowRayTraceFrag.glsl
// main) over a W x H target at full resolution (no Halton offset), hard
// shadows (no contact-hardening cone), no alpha test. hit_t: the G-buffer's
// hit distance plane (u_PositionTexture); normal: its face plane as the
// initial trace writes it (u_NormalTexture, face id / 10, GL_NEAREST as the
// G-buffer's face plane is, Core/Pipeline.cpp:1094). v_RayOrigin is the
// camera position the vertex stage passes, gl_FragCoord the texel centre.
// Out: o_Shadow per texel.
void glslref_trace_shadow(const uint8_t* vox, const uint8_t* df, int X, int Y, int Z, const float* inv_view,
                          const float* inv_proj, int W, int H, const float* hit_t, const float* normal,
                          const float* light_dir, float* o_shadow) {
    static const float no_noise[1] = {0.0f};
    shadow::WORLD_SIZE_X = X; shadow::WORLD_SIZE_Y = Y; shadow::WORLD_SIZE_Z = Z;
    shadow::u_VoxelData = sampler3D{vox, X, Y, Z};
    shadow::u_DistanceFieldTexture = sampler3D{df, X, Y, Z};
    shadow::u_PositionTexture = sampler2D{hit_t, W, H};
    shadow::u_NormalTexture = sampler2D{normal, W, H, 1, true};
    shadow::u_BlueNoiseTexture = sampler2D{no_noise, 1, 1};
    shadow::u_InverseView = mat_from(inv_view);
    shadow::u_InverseProjection = mat_from(inv_proj);
    shadow::u_Dimensions = vec2((float)W, (float)H);
    shadow::u_Halton = vec2(0.0f, 0.0f);
    shadow::u_LightDirection = vec3(light_dir[0], light_dir[1], light_dir[2]);
    shadow::u_ContactHardeningShadows = false;
    shadow::u_ShouldAlphaTest = false;
    shadow::u_FOV = 90.0f;
    shadow::u_Time = 0.0f;
    shadow::u_CurrentFrame = 0;
    shadow::v_RayOrigin = vec3(inv_view[12], inv_view[13], inv_view[14]);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            shadow::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            shadow::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            shadow::main();
            o_shadow[(size_t)j * W + i] = shadow::o_Shadow;
        }
}

// The pre-temporal 3x3 filter (Core/Pipeline.cpp:2288-2330,
// Spatial3x3Initial.glsl main) over a W x H grid. t: hit distance, normal:
// face id / 10; sh (4 channels), cocg (2), aosky (2), luma (1): the diffuse
// trace's planes. Out: o_SH, o_CoCg, o_AOSky, o_Utility per texel.
void glslref_spatial_initial(const float* inv_view, const float* inv_proj, int W, int H, const float* t,
                             const float* normal, const float* sh, const float* cocg, const float* aosky,
                             const float* luma, float* o_sh, float* o_cocg, float* o_aosky, float* o_luma) {
    pre3x3::u_PositionTexture = sampler2D{t, W, H, 1};
    pre3x3::u_NormalTexture = sampler2D{normal, W, H, 1, true};
    pre3x3::u_SH = sampler2D{sh, W, H, 4};
    pre3x3::u_CoCg = sampler2D{cocg, W, H, 2};
    pre3x3::u_AO = sampler2D{aosky, W, H, 2};
    pre3x3::u_Utility = sampler2D{luma, W, H, 1};
    pre3x3::u_InverseView = mat_from(inv_view);
    pre3x3::u_InverseProjection = mat_from(inv_proj);
    pre3x3::u_Dimensions = vec2((float)W, (float)H);
    pre3x3::u_Time = 0.0f;
    pre3x3::v_RayOrigin = vec3(inv_view[12], inv_view[13], inv_view[14]);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            pre3x3::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            pre3x3::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            pre3x3::main();
            const size_t px = (size_t)j * W + i;
            for (int c = 0; c < 4; c++) o_sh[px * 4 + c] = pre3x3::o_SH[c];
            o_cocg[px * 2] = pre3x3::o_CoCg.x;
            o_cocg[px * 2 + 1] = pre3x3::o_CoCg.y;
            o_aosky[px * 2] = pre3x3::o_AOSky.x;
            o_aosky[px * 2 + 1] = pre3x3::o_AOSky.y;
            o_luma[px] = pre3x3::o_Utility;
        }
}

// The SVGF variance estimate (Core/Pipeline.cpp:2440-2475,
// SVGF/VarianceEstimate.glsl main) over a W x H grid. t / normal as above;
// sh (4 channels), cocg (2), util (4: accumulated frames, moment, luminance):
// the temporal pass's planes. Out: o_SH, o_CoCg, o_Variance per texel.
void glslref_variance(const float* inv_view, const float* inv_proj, int W, int H, const float* t,
                      const float* normal, const float* sh, const float* cocg, const float* util, float* o_sh,
                      float* o_cocg, float* o_var) {
    variance::u_PositionTexture = sampler2D{t, W, H, 1};
    variance::u_NormalTexture = sampler2D{normal, W, H, 1, true};
    variance::u_SH = sampler2D{sh, W, H, 4};
    variance::u_CoCg = sampler2D{cocg, W, H, 2};
    variance::u_Utility = sampler2D{util, W, H, 4};
    variance::u_InverseView = mat_from(inv_view);
    variance::u_InverseProjection = mat_from(inv_proj);
    variance::v_RayOrigin = vec3(inv_view[12], inv_view[13], inv_view[14]);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            variance::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            variance::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            variance::main();
            const size_t px = (size_t)j * W + i;
            for (int c = 0; c < 4; c++) o_sh[px * 4 + c] = variance::o_SH[c];
            o_cocg[px * 2] = variance::o_CoCg.x;
            o_cocg[px * 2 + 1] = variance::o_CoCg.y;
            o_var[px] = variance::o_Variance;
        }
}

// One SVGF a-trous iteration (Core/Pipeline.cpp:2481-2610,
// SVGF/SpatialFilter.glsl main) of step `step` over a W x H grid, with the
// pipeline's settings (3x3 taps, aggressive disocclusion handling, spatial
// filter on). sh (4 channels), cocg (2), variance (1), aosky (2): the
// iteration's input planes; util (4): the temporal pass's (accumulated
// frames first). Out: o_SH, o_CoCg, o_Variance, o_AOAndSkylighting.
void glslref_atrous(int W, int H, int step, float resolution_scale,
                    float color_phi_bias, float time, const float* t, const float* normal, const float* util,
                    const float* sh, const float* cocg, const float* var, const float* aosky, float* o_sh,
                    float* o_cocg, float* o_var, float* o_aosky) {
    atrous::u_PositionTexture = sampler2D{t, W, H, 1};
    atrous::u_NormalTexture = sampler2D{normal, W, H, 1, true};
    atrous::u_Utility = sampler2D{util, W, H, 4};
    atrous::u_TemporalMoment = sampler2D{util, W, H, 4};
    atrous::u_SH = sampler2D{sh, W, H, 4};
    atrous::u_CoCg = sampler2D{cocg, W, H, 2};
    atrous::u_VarianceTexture = sampler2D{var, W, H, 1};
    atrous::u_AO = sampler2D{aosky, W, H, 2};
    atrous::u_Dimensions = vec2((float)W, (float)H);
    atrous::u_Step = step;
    atrous::u_LargeKernel = false;
    atrous::AGGRESSIVE_DISOCCLUSION_HANDLING = true;
    atrous::DO_SPATIAL = true;
    atrous::u_ColorPhiBias = color_phi_bias;
    atrous::u_ResolutionScale = resolution_scale;
    atrous::u_Time = time;
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            atrous::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            atrous::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            atrous::main();
            const size_t px = (size_t)j * W + i;
            for (int c = 0; c < 4; c++) o_sh[px * 4 + c] = atrous::o_SH[c];
            o_cocg[px * 2] = atrous::o_CoCg.x;
            o_cocg[px * 2 + 1] = atrous::o_CoCg.y;
            o_var[px] = atrous::o_Variance;
            o_aosky[px * 2] = atrous::o_AOAndSkylighting.x;
            o_aosky[px * 2 + 1] = atrous::o_AOAndSkylighting.y;
        }
}

// The SVGF temporal pass (Core/Pipeline.cpp:2336-2436,
// SVGF/TemporalFilter.glsl main) over a W x H grid. The current frame: t,
// normal (face id / 10), block (id / 255), the pre-filtered sh (4 channels),
// cocg (2), luma (1) and aosky (2); the previous frame: its G-buffer (prev_t,
// prev_normal, prev_block) and history (prev_sh, prev_cocg, prev_util (4),
// prev_aosky), sampled at the reprojected coordinates (bilinear, the face and
// block planes nearest). view / proj: the previous camera's. Out: o_SH,
// o_CoCg, o_Utility (3), o_AOAndSkyLighting.
void glslref_temporal(const float* inv_view, const float* inv_proj, const float* prev_view, const float* prev_proj,
                      int W, int H, int be_useful, const float* t, const float* normal, const float* block,
                      const float* sh, const float* cocg, const float* luma, const float* aosky, const float* prev_t,
                      const float* prev_normal, const float* prev_block, const float* prev_sh,
                      const float* prev_cocg, const float* prev_util, const float* prev_aosky, float* o_sh,
                      float* o_cocg, float* o_util, float* o_aosky) {
    temporal::u_CurrentPositionTexture = sampler2D{t, W, H, 1};
    temporal::u_CurrentNormalTexture = sampler2D{normal, W, H, 1, true};
    temporal::u_CurrentBlockIDTexture = sampler2D{block, W, H, 1, true};
    temporal::u_CurrentSH = sampler2D{sh, W, H, 4};
    temporal::u_CurrentCoCg = sampler2D{cocg, W, H, 2};
    temporal::u_NoisyLuminosity = sampler2D{luma, W, H, 1};
    temporal::u_CurrentAO = sampler2D{aosky, W, H, 2};
    temporal::u_PreviousPositionTexture = sampler2D{prev_t, W, H, 1, false, false};
    temporal::u_PreviousNormalTexture = sampler2D{prev_normal, W, H, 1, true};
    temporal::u_PrevBlockIDTexture = sampler2D{prev_block, W, H, 1, true};
    temporal::u_PreviousSH = sampler2D{prev_sh, W, H, 4, false, false};
    temporal::u_PrevCoCg = sampler2D{prev_cocg, W, H, 2, false, false};
    temporal::u_PreviousUtility = sampler2D{prev_util, W, H, 4, false, false};
    temporal::u_PreviousAO = sampler2D{prev_aosky, W, H, 2, false, false};
    temporal::u_InverseView = mat_from(inv_view);
    temporal::u_InverseProjection = mat_from(inv_proj);
    temporal::u_PrevView = mat_from(prev_view);
    temporal::u_PrevProjection = mat_from(prev_proj);
    temporal::u_BeUseful = be_useful != 0;
    temporal::u_Time = 0.0f;
    temporal::v_RayOrigin = vec3(inv_view[12], inv_view[13], inv_view[14]);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            temporal::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            temporal::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            temporal::main();
            const size_t px = (size_t)j * W + i;
            for (int c = 0; c < 4; c++) o_sh[px * 4 + c] = temporal::o_SH[c];
            o_cocg[px * 2] = temporal::o_CoCg.x;
            o_cocg[px * 2 + 1] = temporal::o_CoCg.y;
            for (int c = 0; c < 3; c++) o_util[px * 3 + c] = temporal::o_Utility[c];
            o_aosky[px * 2] = temporal::o_AOAndSkyLighting.x;
            o_aosky[px * 2 + 1] = temporal::o_AOAndSkyLighting.y;
        }
}

// One a-trous iteration of the non-SVGF denoiser (Core/Pipeline.cpp:2720-2786,
// AtrousSpatialFilter.glsl main) of step `step` over a W x H grid. t,
// normal (face id / 10), block (id / 255), var: the G-buffer and the
// variance estimate; sh (4 channels) and cocg (2): the iteration's input.
// Out: o_SpatialResult (SH) and o_SpatialResult2 (CoCg) per texel.
void glslref_plain_atrous(const float* inv_view, const float* inv_proj, int W, int H, int step, const float* t,
                          const float* normal, const float* block, const float* var, const float* sh,
                          const float* cocg, float* o_sh, float* o_cocg) {
    plain_atrous::u_PositionTexture = sampler2D{t, W, H, 1};
    plain_atrous::u_NormalTexture = sampler2D{normal, W, H, 1, true};
    plain_atrous::u_BlockIDTexture = sampler2D{block, W, H, 1, true};
    plain_atrous::u_VarianceTexture = sampler2D{var, W, H, 1};
    plain_atrous::u_InputTexture = sampler2D{sh, W, H, 4};
    plain_atrous::u_InputTexture2 = sampler2D{cocg, W, H, 2};
    plain_atrous::u_InverseView = mat_from(inv_view);
    plain_atrous::u_InverseProjection = mat_from(inv_proj);
    plain_atrous::u_Dimensions = vec2((float)W, (float)H);
    plain_atrous::u_Step = step;
    plain_atrous::v_RayOrigin = vec3(inv_view[12], inv_view[13], inv_view[14]);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            plain_atrous::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            plain_atrous::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            plain_atrous::main();
            const size_t px = (size_t)j * W + i;
            for (int c = 0; c < 4; c++) o_sh[px * 4 + c] = plain_atrous::o_SpatialResult[c];
            o_cocg[px * 2] = plain_atrous::o_SpatialResult2.x;
            o_cocg[px * 2 + 1] = plain_atrous::o_SpatialResult2.y;
        }
}

// The non-SVGF temporal pass (Core/Pipeline.cpp:2618-2680, TemporalFilter.glsl
// main in its diffuse mode: u_DiffuseTemporal on, u_ShadowTemporal off,
// u_MinimumMix 0, u_MaximumMix 0.96) over a W x H grid. t / prev_t: the
// current and previous hit distances; sh (4 channels) / cocg (2): this
// frame's GI, prev_sh / prev_cocg the previous output, sampled at the
// reprojected coordinates. Out: o_Color (SH) and o_CoCg per texel.
void glslref_plain_temporal(const float* inv_view, const float* inv_proj, const float* prev_view,
                            const float* prev_proj, int W, int H, const float* t, const float* prev_t,
                            const float* sh, const float* cocg, const float* prev_sh, const float* prev_cocg,
                            float* o_sh, float* o_cocg) {
    static const float zero[1] = {0.0f};
    plain_temporal::u_CurrentColorTexture = sampler2D{sh, W, H, 4};
    plain_temporal::u_CurrentPositionTexture = sampler2D{t, W, H, 1};
    plain_temporal::u_PreviousColorTexture = sampler2D{prev_sh, W, H, 4, false, false};
    plain_temporal::u_PreviousFramePositionTexture = sampler2D{prev_t, W, H, 1, false, false};
    plain_temporal::u_CurrentSH = sampler2D{cocg, W, H, 2};
    plain_temporal::u_PreviousSH = sampler2D{prev_cocg, W, H, 2, false, false};
    plain_temporal::u_ShadowTransversals = sampler2D{zero, 1, 1, 1};
    plain_temporal::u_InverseView = mat_from(inv_view);
    plain_temporal::u_InverseProjection = mat_from(inv_proj);
    plain_temporal::u_PrevView = mat_from(prev_view);
    plain_temporal::u_PrevProjection = mat_from(prev_proj);
    plain_temporal::u_MinimumMix = 0.0f;
    plain_temporal::u_MaximumMix = 0.96f;
    plain_temporal::u_DiffuseTemporal = true;
    plain_temporal::u_ShadowTemporal = false;
    plain_temporal::u_ShouldFilterShadows = false;
    plain_temporal::v_RayOrigin = vec3(inv_view[12], inv_view[13], inv_view[14]);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            plain_temporal::v_TexCoords = vec2(((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H);
            plain_temporal::gl_FragCoord = vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            plain_temporal::main();
            const size_t px = (size_t)j * W + i;
            for (int c = 0; c < 4; c++) o_sh[px * 4 + c] = plain_temporal::o_Color[c];
            o_cocg[px * 2] = plain_temporal::o_CoCg.x;
            o_cocg[px * 2 + 1] = plain_temporal::o_CoCg.y;
        }
}

// The diffuse trace's IrridianceToSH (DiffuseRayTraceFrag.glsl:766-784) and
// the colour pass's SHToIrridiance (ColorPassFrag.glsl:357-368) over n items.
// op 0: in = radiance (3) and direction (3) per item, out = SH (4) and CoCg
// (2); op 1: in = SH (4), CoCg (2) and normal (3), out = irradiance (3).
void glslref_sh_codec(int op, int n, const float* in, float* out) {
    for (int k = 0; k < n; k++) {
        if (op == 0) {
            const float* a = in + 6 * k;
            const arr_float_6 r = sh_encode::IrridianceToSH(vec3(a[0], a[1], a[2]), vec3(a[3], a[4], a[5]));
            for (int i = 0; i < 6; i++) out[6 * k + i] = r[i];
        } else {
            const float* a = in + 9 * k;
            const vec3 r = sh_decode::SHToIrridiance(vec4(a[0], a[1], a[2], a[3]), vec2(a[4], a[5]),
                                                     vec3(a[6], a[7], a[8]));
            out[3 * k] = r.x;
            out[3 * k + 1] = r.y;
            out[3 * k + 2] = r.z;
        }
    }
}

// DiffuseRayBRDF (DiffuseRayTraceFrag.glsl:527-531, DiffuseHammon :1311-1332)
// over n items: in = normal (3), incident (3), direction (3), roughness per
// item; out = the BRDF's first component.
void glslref_diffuse_brdf(int n, const float* in, float* out) {
    for (int k = 0; k < n; k++) {
        const float* a = in + 10 * k;
        out[k] = brdf::DiffuseRayBRDF(vec3(a[0], a[1], a[2]), vec3(a[3], a[4], a[5]), vec3(a[6], a[7], a[8]), a[9]).x;
    }
}

}  // extern "C"
