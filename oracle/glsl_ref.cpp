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

}  // extern "C"
