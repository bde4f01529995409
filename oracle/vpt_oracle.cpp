// CPU oracle for the VoxelPathTracer hot path.
//
// TEST INFRASTRUCTURE ONLY (see vpt_oracle.h): a C++17 restatement of the
// reference shaders, used by the parity tests as the checker and by bench.py
// as the timed CPU baseline. Build: g++ -O2 -fopenmp -ffp-contract=off.
//
// Conventions that the reference leaves to the OpenGL implementation are
// fixed here and in the CUDA kernels alike:
//   * pixel (i, j) has texture coordinate ((i+0.5)/W, (j+0.5)/H), row 0 at the
//     bottom, exactly like gl_FragCoord / v_TexCoords of a full-screen quad;
//   * texture() at a texel centre returns that texel (what the hardware's
//     fixed-point addressing does); at other coordinates it is bilinear with
//     REPEAT wrap (Core/GLClasses/Framebuffer.cpp:64-70) and fp32 weights;
//     the R8 face and block planes are nearest-filtered
//     (Core/Pipeline.cpp:1094);
//   * int(NaN) = 0 and out-of-range conversions saturate (omath.h f2i);
//   * normalize(v) = v * (1 / sqrt(dot(v, v))), dot sums left to right;
//   * transcendental functions come from omath.h.
// Documented substitutions (the reference's versions need textures):
//   * block table: flat albedo RGB8, roughness u8, metalness u8, emissive flag;
//   * sky: an analytic gradient instead of the atmosphere cubemap;
//   * random numbers: PCG (Jarzynski & Olano 2020, "Hash Functions for GPU
//     Rendering") seeded per pixel instead of fract(sin()) / blue noise;
//   * no TAA jitter, no alpha testing, no checkerboard SPP, no player shadow,
//     no specular/reflection input (its floor 0.0001 is kept).
#include "vpt_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "omath.h"

using namespace vpto;

namespace {

const float PI = 3.14159265359f;   // DiffuseRayTraceFrag.glsl:11, ColorPassFrag.glsl:6

// Optional ray / DDA-step counters (primary, shadow, diffuse, bounce shadow),
// same layout as vpt_stats; used by the CPU baseline to count its work.
uint64_t* g_counters = nullptr;
struct RowCount {
    uint64_t rays[6] = {0, 0, 0, 0, 0, 0};
    uint64_t steps[6] = {0, 0, 0, 0, 0, 0};
    void add(int kind, int nsteps) { rays[kind] += 1; steps[kind] += (uint64_t)nsteps; }
    void flush() {
        if (!g_counters) return;
        for (int k = 0; k < 6; k++) {
#pragma omp atomic
            g_counters[k] += rays[k];
#pragma omp atomic
            g_counters[6 + k] += steps[k];
        }
    }
};

inline size_t vidx(const vpto_world* w, int x, int y, int z) {
    return (size_t)x + (size_t)w->X * ((size_t)y + (size_t)w->Y * (size_t)z);
}

// IsInVolume (InitialRayTraceFrag.glsl:68-77) on integer coordinates.
inline bool in_volume(const vpto_world* w, int x, int y, int z) {
    return !(x < 0 || y < 0 || z < 0 || x > w->X - 1 || y > w->Y - 1 || z > w->Z - 1);
}

// GetVoxel (InitialRayTraceFrag.glsl:79-87): block id, 0 outside.
inline int get_voxel(const vpto_world* w, int x, int y, int z) {
    return in_volume(w, x, y, z) ? (int)w->vox[vidx(w, x, y, z)] : 0;
}

// int(floor(ToConservativeEuclidean(Dist))) (InitialRayTraceFrag.glsl:89-92, :328-330).
// texelFetch(R8)*255 returns the stored integer exactly for every byte value.
inline int euclid_steps(int dist) {
    float D = (float)dist;
    float e = (D == 1.0f) ? 1.0f : D * 0.57735026918f;
    return f2i(std::floor(e));
}

struct TraceResult {
    float t;          // distance(origin, initial_origin) or -1
    v3 normal;        // -RaySign[MinIdx] on MinIdx (valid when hit)
    int block;        // GetVoxel at the end point (0 on miss)
    int32_t cell[3];  // ivec3(floor(origin)) at loop exit
    int steps;        // itr at loop exit
};

// VoxelTraversalDF: InitialRayTraceFrag.glsl:307-374 (identical copies at
// ShadowRayTraceFrag.glsl:222-289 and DiffuseRayTraceFrag.glsl:1043-1110, the
// latter with the step cap as a parameter).
TraceResult traverse(const vpto_world* w, v3 origin, v3 direction, int max_steps) {
    const v3 initial = origin;
    bool intersection = false;
    int min_idx = 0;
    const int sgn[3] = {isign(direction.x), isign(direction.y), isign(direction.z)};
    const int half[3] = {(1 + sgn[0]) >> 1, (1 + sgn[1]) >> 1, (1 + sgn[2]) >> 1};
    const v3 inv = mk3(1.0f / direction.x, 1.0f / direction.y, 1.0f / direction.z);
    int itr = 0;
    for (itr = 0; itr < max_steps; itr++) {
        int lx = f2i(std::floor(origin.x));
        int ly = f2i(std::floor(origin.y));
        int lz = f2i(std::floor(origin.z));
        if (!in_volume(w, lx, ly, lz)) {
            intersection = false;
            break;
        }
        int e = euclid_steps((int)w->df[vidx(w, lx, ly, lz)]);
        if (e == 0) break;
        if (e == 1) {
            // one exact DDA face step (:341-356)
            int g[3] = {f2i(origin.x), f2i(origin.y), f2i(origin.z)};
            v3 wv = mk3(origin.x - (float)g[0], origin.y - (float)g[1], origin.z - (float)g[2]);
            v3 df = mk3(((float)half[0] - wv.x) * inv.x, ((float)half[1] - wv.y) * inv.y,
                        ((float)half[2] - wv.z) * inv.z);
            min_idx = (df.x < df.y && sgn[0] != 0) ? ((df.x < df.z || sgn[2] == 0) ? 0 : 2)
                                                   : ((df.y < df.z || sgn[2] == 0) ? 1 : 2);
            g[min_idx] += sgn[min_idx];
            float dm = comp(df, min_idx);
            wv = mk3(wv.x + direction.x * dm, wv.y + direction.y * dm, wv.z + direction.z * dm);
            set_comp(&wv, min_idx, (float)(1 - half[min_idx]));
            origin = mk3((float)g[0] + wv.x, (float)g[1] + wv.y, (float)g[2] + wv.z);
            set_comp(&origin, min_idx, comp(origin, min_idx) + (float)sgn[min_idx] * 0.0001f);
            intersection = true;
        } else {
            // jump by the conservative Euclidean radius (:361)
            float k = (float)(e - 1);
            origin = mk3(origin.x + k * direction.x, origin.y + k * direction.y,
                         origin.z + k * direction.z);
        }
    }
    TraceResult r;
    r.cell[0] = f2i(std::floor(origin.x));
    r.cell[1] = f2i(std::floor(origin.y));
    r.cell[2] = f2i(std::floor(origin.z));
    r.steps = itr;
    r.normal = mk3(0.0f, 0.0f, 0.0f);
    r.block = 0;
    r.t = -1.0f;
    if (intersection) {   // :365-371
        set_comp(&r.normal, min_idx, (float)(-sgn[min_idx]));
        r.block = get_voxel(w, r.cell[0], r.cell[1], r.cell[2]);
        r.t = r.block > 0 ? length(sub(origin, initial)) : -1.0f;
    }
    return r;
}

int normal_id(v3 n);
bool alpha_active(const vpto_params* p);
bool alpha_active_shadows(const vpto_params* p);

// K of StopRay (InitialRayTraceFrag.glsl:421): 1 / (2 tan(fov / (2 W))),
// the vertical fov 2 atan(1 / proj[1][1]), in double precision.
inline float alpha_k(float proj11, int width) {
    const double fov = 2.0 * std::atan(1.0 / (double)proj11);
    return (float)(1.0 / (std::tan(fov / (2.0 * (double)width)) * 2.0));
}

// StopRay (InitialRayTraceFrag.glsl:189-202) with the block textures set by
// vpto_set_block_textures (true for every block without them).
// flip_x / lod_bias: 1 / 0 for the primary rays, 0 / -2 for the shadow rays
// (ShadowRayTraceFrag.glsl:105-117).
bool alpha_stop(v3 p, v3 n, int type, v3 cam, float k, int flip_x, int lod_bias);

// VoxelTraversalDF_AlphaTest (InitialRayTraceFrag.glsl:204-305): at a solid
// voxel (E == 0) StopRay decides; if the ray goes on, up to four exact face
// steps look for a voxel that stops it, then the loop continues from one
// direction length back (origin += (E - 1) * direction).
TraceResult traverse_alpha(const vpto_world* w, v3 origin, v3 direction, int max_steps, v3 cam, float k,
                           int flip_x = 1, int lod_bias = 0) {
    const v3 initial = origin;
    bool intersection = false;
    int min_idx = 0;
    const int sgn[3] = {isign(direction.x), isign(direction.y), isign(direction.z)};
    const int half[3] = {(1 + sgn[0]) >> 1, (1 + sgn[1]) >> 1, (1 + sgn[2]) >> 1};
    const v3 inv = mk3(1.0f / direction.x, 1.0f / direction.y, 1.0f / direction.z);
    auto face_step = [&]() {
        int g[3] = {f2i(origin.x), f2i(origin.y), f2i(origin.z)};
        v3 wv = mk3(origin.x - (float)g[0], origin.y - (float)g[1], origin.z - (float)g[2]);
        v3 df = mk3(((float)half[0] - wv.x) * inv.x, ((float)half[1] - wv.y) * inv.y, ((float)half[2] - wv.z) * inv.z);
        min_idx = (df.x < df.y && sgn[0] != 0) ? ((df.x < df.z || sgn[2] == 0) ? 0 : 2)
                                               : ((df.y < df.z || sgn[2] == 0) ? 1 : 2);
        g[min_idx] += sgn[min_idx];
        float dm = comp(df, min_idx);
        wv = mk3(wv.x + direction.x * dm, wv.y + direction.y * dm, wv.z + direction.z * dm);
        set_comp(&wv, min_idx, (float)(1 - half[min_idx]));
        origin = mk3((float)g[0] + wv.x, (float)g[1] + wv.y, (float)g[2] + wv.z);
        set_comp(&origin, min_idx, comp(origin, min_idx) + (float)sgn[min_idx] * 0.0001f);
    };
    auto step_normal = [&]() {
        v3 n = mk3(0.0f, 0.0f, 0.0f);
        set_comp(&n, min_idx, (float)(-sgn[min_idx]));
        return n;
    };
    int itr = 0;
    for (itr = 0; itr < max_steps; itr++) {
        int lx = f2i(std::floor(origin.x)), ly = f2i(std::floor(origin.y)), lz = f2i(std::floor(origin.z));
        if (!in_volume(w, lx, ly, lz)) {
            intersection = false;
            break;
        }
        int e = euclid_steps((int)w->df[vidx(w, lx, ly, lz)]);
        if (e == 0) {
            if (alpha_stop(origin, step_normal(), get_voxel(w, lx, ly, lz), cam, k, flip_x, lod_bias)) break;
            for (int s = 0; s < 4; s++) {
                face_step();
                const int cx = f2i(std::floor(origin.x)), cy = f2i(std::floor(origin.y)), cz = f2i(std::floor(origin.z));
                const int bt = get_voxel(w, cx, cy, cz);
                if (bt > 0 && alpha_stop(origin, step_normal(), bt, cam, k, flip_x, lod_bias)) {
                    TraceResult r;
                    r.cell[0] = cx;
                    r.cell[1] = cy;
                    r.cell[2] = cz;
                    r.steps = itr;
                    r.normal = step_normal();
                    r.block = bt;
                    r.t = length(sub(origin, initial));
                    return r;
                }
            }
        }
        if (e == 1) {
            face_step();
            intersection = true;
        } else {
            float kk = (float)(e - 1);
            origin = mk3(origin.x + kk * direction.x, origin.y + kk * direction.y, origin.z + kk * direction.z);
        }
    }
    TraceResult r;
    r.cell[0] = f2i(std::floor(origin.x));
    r.cell[1] = f2i(std::floor(origin.y));
    r.cell[2] = f2i(std::floor(origin.z));
    r.steps = itr;
    r.normal = mk3(0.0f, 0.0f, 0.0f);
    r.block = 0;
    r.t = -1.0f;
    if (intersection) {
        set_comp(&r.normal, min_idx, (float)(-sgn[min_idx]));
        r.block = get_voxel(w, r.cell[0], r.cell[1], r.cell[2]);
        r.t = r.block > 0 ? length(sub(origin, initial)) : -1.0f;
    }
    return r;
}

// GetNormalID (InitialRayTraceFrag.glsl:143-185): exact compares, 0 when none match.
int normal_id(v3 n) {
    static const v3 N[6] = {{0, 0, 1}, {0, 0, -1}, {0, 1, 0}, {0, -1, 0}, {-1, 0, 0}, {1, 0, 0}};
    for (int i = 0; i < 6; i++)
        if (n.x == N[i].x && n.y == N[i].y && n.z == N[i].z) return i;
    return 0;
}

// GetNormalFromID (e.g. SVGF/TemporalFilter.glsl:108-119); `miss` is what
// ids > 5 decode to (vec3(1) in most shaders, vec3(0.5) in the diffuse pass).
v3 normal_from_id(int id, float miss) {
    static const v3 N[6] = {{0, 0, 1}, {0, 0, -1}, {0, 1, 0}, {0, -1, 0}, {-1, 0, 0}, {1, 0, 0}};
    if (id > 5 || id < 0) return mk3(miss, miss, miss);
    return N[id];
}

// ------------------------------------------------------------ camera rays --
inline v2 texcoord(int i, int j, int W, int H) {
    return v2{((float)i + 0.5f) / (float)W, ((float)j + 0.5f) / (float)H};
}

// GetRayDirectionAt (e.g. ShadowRayTraceFrag.glsl:303-308) / GetRayStuff
// (InitialRayTraceFrag.glsl:398-414 without TAA jitter).
inline v3 ray_dir_at(const vpto_camera* c, v2 uv) {
    float cx = uv.x * 2.0f - 1.0f;
    float cy = uv.y * 2.0f - 1.0f;
    v4 e = mat_mul4(c->inv_proj, cx, cy, -1.0f, 1.0f);
    v4 d = mat_mul4(c->inv_view, e.x, e.y, -1.0f, 0.0f);
    return mk3(d.x, d.y, d.z);
}

inline v3 ray_origin(const vpto_camera* c) { return mk3(c->inv_view[12], c->inv_view[13], c->inv_view[14]); }

// ------------------------------------------------------------- sampling --
inline int wrapi(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

struct Plane {
    const float* p;
    int W, H, C;
    float at(int i, int j, int c) const {
        return p[((size_t)wrapi(j, H) * W + wrapi(i, W)) * C + c];
    }
    // texture() with GL_LINEAR + GL_REPEAT, fp32 weights.
    void linear(v2 uv, float* out) const {
        float x = uv.x * (float)W - 0.5f;
        float y = uv.y * (float)H - 0.5f;
        float x0 = std::floor(x), y0 = std::floor(y);
        float ax = x - x0, ay = y - y0;
        int i0 = f2i(x0), j0 = f2i(y0);
        for (int c = 0; c < C; c++) {
            float v00 = at(i0, j0, c), v10 = at(i0 + 1, j0, c);
            float v01 = at(i0, j0 + 1, c), v11 = at(i0 + 1, j0 + 1, c);
            float b = v00 * (1.0f - ax) + v10 * ax;
            float t = v01 * (1.0f - ax) + v11 * ax;
            out[c] = b * (1.0f - ay) + t * ay;
        }
    }
};

struct Plane8 {
    const uint8_t* p;
    int W, H;
    int at(int i, int j) const { return p[(size_t)wrapi(j, H) * W + wrapi(i, W)]; }
    // texture() with GL_NEAREST + GL_REPEAT
    int nearest(v2 uv) const {
        return at(f2i(std::floor(uv.x * (float)W)), f2i(std::floor(uv.y * (float)H)));
    }
    // texture() with GL_LINEAR + GL_REPEAT of a 0/1 plane read as UNORM8
    // (the sun-shadow FBO, Core/Pipeline.cpp:1152), fp32 weights.
    float linearf(v2 uv) const {
        float x = uv.x * (float)W - 0.5f;
        float y = uv.y * (float)H - 0.5f;
        float x0 = std::floor(x), y0 = std::floor(y);
        float ax = x - x0, ay = y - y0;
        int i0 = f2i(x0), j0 = f2i(y0);
        float v00 = (float)at(i0, j0), v10 = (float)at(i0 + 1, j0);
        float v01 = (float)at(i0, j0 + 1), v11 = (float)at(i0 + 1, j0 + 1);
        float b = v00 * (1.0f - ax) + v10 * ax;
        float t = v01 * (1.0f - ax) + v11 * ax;
        return b * (1.0f - ay) + t * ay;
    }
};

inline float storage(float v, int fp16) { return fp16 ? half_round(v) : v; }

// GetPositionAt at a texel centre (fetch) or at an arbitrary coordinate (linear).
inline v4 position_fetch(const vpto_camera* c, const Plane& t, int i, int j, v2 txc) {
    float d = t.at(i, j, 0);
    v3 p = add(ray_origin(c), muls(normalize(ray_dir_at(c, txc)), d));
    return v4{p.x, p.y, p.z, d};
}
inline v4 position_linear(const vpto_camera* c, const Plane& t, v2 txc) {
    float d;
    t.linear(txc, &d);
    v3 p = add(ray_origin(c), muls(normalize(ray_dir_at(c, txc)), d));
    return v4{p.x, p.y, p.z, d};
}

// ---------------------------------------------------------------- shading --
inline float luminance(v3 c) { return dot(c, mk3(0.299f, 0.587f, 0.114f)); }   // GetLuminance
inline float sh_to_y(const float* sh) { return fmaxg(0.0f, 3.544905f * sh[3]); }  // SHToY

// Analytic sky standing in for the atmosphere cubemap: direction-only like a
// cubemap lookup, horizon-to-zenith gradient.
inline v3 sky_radiance(v3 d) {
    v3 n = normalize(d);
    float a = clampf(n.y, 0.0f, 1.0f);
    return vmix(mk3(0.62f, 0.74f, 0.92f), mk3(0.20f, 0.38f, 0.85f), a);
}

// GetSkyColorAt (DiffuseRayTraceFrag.glsl:984-988)
inline v3 sky_color_at(v3 rd) {
    rd.y = clampf(rd.y, 0.125f, 1.5f);
    return sky_radiance(rd);
}

// IrridianceToSH (DiffuseRayTraceFrag.glsl:766-784)
inline void irradiance_to_sh(v3 r, v3 d, float* sh, float* cocg) {
    float co = r.x - r.z;
    float t = r.z + co * 0.5f;
    float cg = r.y - t;
    float y = fmaxg(t + cg * 0.5f, 0.0f);
    float l00 = 0.282095f;
    float l1_1 = 0.488603f * d.y;
    float l10 = 0.488603f * d.z;
    float l11 = 0.488603f * d.x;
    sh[0] = fmaxg(l11 * y, -100.0f);
    sh[1] = fmaxg(l1_1 * y, -100.0f);
    sh[2] = fmaxg(l10 * y, -100.0f);
    sh[3] = fmaxg(l00 * y, -100.0f);
    cocg[0] = co;
    cocg[1] = cg;
}

// SHToIrridiance (ColorPassFrag.glsl:357-368)
inline v3 sh_to_irradiance(const float* sh, const float* cocg_in, v3 v) {
    float x = dot(mk3(sh[0], sh[1], sh[2]), v);
    float y = 2.0f * (1.023326f * x + 0.886226f * sh[3]);
    y = fmaxg(y, 0.0f);
    float s = (y * 0.282095f) / (sh[3] + 1e-6f);
    float co = cocg_in[0] * s, cg = cocg_in[1] * s;
    float t = y - cg * 0.5f;
    float g = cg + t;
    float b = t - co * 0.5f;
    float r = b + co;
    return vmax(mk3(r, g, b), 0.0f);
}

// InverseSchlick (DiffuseRayTraceFrag.glsl:1305-1308)
inline float inverse_schlick(float f0, float voh) {
    return 1.0f - clampf(f0 + (1.0f - f0) * dm_pow(1.0f - voh, 5.0f), 0.0f, 1.0f);
}

// DiffuseHammon (DiffuseRayTraceFrag.glsl:1311-1332); rcp(x) = 1/x.
inline float diffuse_hammon(v3 n, v3 v, v3 l, float rough) {
    float ndl = fmaxg(dot(n, l), 0.0f);
    if (ndl <= 0.0f) return 0.0f;
    float ndv = fmaxg(dot(n, v), 0.0f);
    float ldv = fmaxg(dot(l, v), 0.0f);
    v3 h = normalize(add(v, l));
    float ndh = fmaxg(dot(n, h), 0.0f);
    float facing = ldv * 0.5f + 0.5f;
    float single_rough = facing * (0.9f - 0.4f * facing) * ((0.5f + ndh) * (1.0f / fmaxg(ndh, 0.02f)));
    float single_smooth = 1.05f * inverse_schlick(0.0f, ndl) * inverse_schlick(0.0f, fmaxg(ndv, 0.0f));
    float single = clampf(mixf(single_smooth, single_rough, rough) * (1.0f / PI), 0.0f, 1.0f);
    float multi = 0.1159f * rough;
    return clampf((multi + single) * ndl, 0.0f, 1.0f);
}

// ------------------------------------------------------------------- RNG --
inline uint32_t pcg_step(uint32_t* s) {
    *s = *s * 747796405u + 2891336453u;
    uint32_t w = ((*s >> ((*s >> 28u) + 4u)) ^ *s) * 277803737u;
    return (w >> 22u) ^ w;
}
inline uint32_t pcg_hash(uint32_t v) {
    uint32_t s = v;
    return pcg_step(&s);
}
inline float rand01(uint32_t* s) { return (float)(pcg_step(s) >> 8) * (1.0f / 16777216.0f); }
inline uint32_t pixel_seed(const vpto_frame* f, uint32_t pixel) {
    return pcg_hash(pixel + pcg_hash(f->frame_index + pcg_hash(f->seed)));
}

// cosWeightedRandomHemisphereDirection (DiffuseRayTraceFrag.glsl:945-967)
inline v3 cos_hemisphere(v3 n, uint32_t* rng) {
    float rx_ = rand01(rng);
    float ry_ = rand01(rng);
    float pi2 = 2.0f * PI;
    v3 uu = normalize(cross(n, mk3(0.0f, 1.0f, 1.0f)));
    v3 vv = cross(uu, n);
    float ra = std::sqrt(ry_);
    float rx = ra * dm_cos(pi2 * rx_);
    float ry = ra * dm_sin(pi2 * rx_);
    float rz = std::sqrt(1.0f - ry_);
    v3 rr = mk3((rx * uu.x + ry * vv.x) + rz * n.x, (rx * uu.y + ry * vv.y) + rz * n.y,
                (rx * uu.z + ry * vv.z) + rz * n.z);
    return normalize(rr);
}

struct Material {
    v3 albedo;
    float rough, metal;
    int emissive;
};
inline Material material(const vpto_world* w, int id) {
    if (id < 0 || id >= w->n_blocks) id = 0;
    const vpto_block& b = w->blocks[id];
    Material m;
    m.albedo = mk3((float)b.albedo[0] / 255.0f, (float)b.albedo[1] / 255.0f, (float)b.albedo[2] / 255.0f);
    m.rough = (float)b.roughness / 255.0f;
    m.metal = (float)b.metalness / 255.0f;
    m.emissive = b.emissive ? 1 : 0;
    return m;
}

struct Lighting {       // per-frame constants of DiffuseRayTraceFrag main (:832-839)
    v3 light_color, light_dir;
    bool moon_stronger;
    float emissivity_multiplier;
    float sun_visibility;   // Core/Pipeline.cpp:1828
};

inline v3 moon_dir_of(v3 s) { return normalize(mk3(-s.x, -s.y, s.z)); }   // Core/Pipeline.cpp:1663

Lighting frame_lighting(const vpto_frame* f) {
    const v3 SUN_COLOR = muls(divs(mk3(192.0f, 216.0f, 255.0f), 255.0f), 16.0f);   // :184
    const v3 NIGHT_COLOR = muls(divs(mk3(96.0f, 192.0f, 255.0f), 255.0f), 1.5f);   // :185
    const v3 DUSK_COLOR = muls(divs(mk3(96.0f, 192.0f, 255.0f), 255.0f), 0.9f);    // :186
    v3 sun = mk3(f->sun_dir[0], f->sun_dir[1], f->sun_dir[2]);
    Lighting L;
    bool sun_stronger = -sun.y < 0.01f;
    float dusk = clampf(dm_pow(std::fabs(sun.y - 1.0f), 2.9f), 0.0f, 1.0f);
    v3 sun_color = vmix(SUN_COLOR, DUSK_COLOR, dusk);
    L.light_color = sun_stronger ? sun_color : NIGHT_COLOR;
    L.light_color = muls(L.light_color, 0.4f * f->gi_sun_strength);
    L.light_dir = sun_stronger ? sun : moon_dir_of(sun);
    L.moon_stronger = !sun_stronger;
    L.emissivity_multiplier = L.moon_stronger ? 13.0f : 12.0f;
    L.sun_visibility = clampf(dot(sun, mk3(0.0f, 1.0f, 0.0f)) + 0.05f, 0.0f, 0.1f) * 12.0f;
    return L;
}

// The block textures' material at a bounce hit (set by vpto_set_block_textures;
// false without textures): textureLod of the albedo array at level 3 and of
// the PBR array at level 2 at the block's albedo layer (DiffuseRayTraceFrag.glsl
// :569-584), at CalculateUV's coordinates (:1235-1273), and the emissive
// texel at level 0 (has_emis false when the block has no emissive layer).
bool tex_bounce_material(int bid, v3 ip, v3 hn, v3* albedo, float* rough, float* emis, bool* has_emis);

// CalculateDiffuse (DiffuseRayTraceFrag.glsl:535-664) with `bounces` = MAX_BOUNCE_LIMIT.
v4 calculate_diffuse(const vpto_world* w, const vpto_params* p, const vpto_frame* f, const Lighting& L,
                     v3 initial_origin, v3 input_normal, uint32_t* rng, v3* odir, bool* skyhit, RowCount* cnt) {
    *skyhit = false;
    const float bias = 0.06f;
    v3 ro = add(initial_origin, muls(input_normal, bias));
    v3 rd = cos_hemisphere(input_normal, rng);
    float ao = 1.0f;
    v3 contribution = mk3(0, 0, 0);
    v3 throughput = mk3(1, 1, 1);
    for (int i = 0; i < p->bounces; i++) {
        if (i == 0) *odir = rd;
        TraceResult tr = traverse(w, ro, rd, p->diffuse_max_steps);
        cnt->add(2, tr.steps);
        float T = tr.t;
        bool intersect = T > 0.0f;
        v3 ip = add(ro, muls(rd, T));
        if (intersect && tr.block > 0) {
            const int bid = std::min(std::max(tr.block, 0), 127);
            Material m = material(w, bid);
            v3 hn = tr.normal;
            float emissivity = 0.0f;
            v3 t_albedo;
            float t_rough, t_emis;
            bool t_has;
            if (tex_bounce_material(bid, ip, hn, &t_albedo, &t_rough, &t_emis, &t_has)) {
                m.albedo = t_albedo;
                m.rough = t_rough;
                if (t_has) emissivity = t_emis * L.emissivity_multiplier * f->diffuse_light_intensity;
            } else if (m.emissive) {
                emissivity = 1.0f * L.emissivity_multiplier * f->diffuse_light_intensity;
            }
            float ndl = fmaxg(dot(hn, L.light_dir), 0.0f);
            v3 bias_shadow = muls(hn, 0.045f);
            float shadow_at;
            if (L.moon_stronger) {
                shadow_at = 1.0f;
            } else {
                // GetShadowAt (:1202-1222)
                if (ndl < 0.001f) {
                    shadow_at = 0.0f;
                } else {
                    TraceResult sr = traverse(w, add(ip, bias_shadow), L.light_dir, p->bounce_shadow_max_steps);
                    cnt->add(3, sr.steps);
                    shadow_at = sr.t > 0.0f ? 1.0f : 0.0f;
                }
            }
            v3 emissive_color = muls(m.albedo, emissivity * mixf(1.0f, 1.0f, L.sun_visibility));
            // SunBRDF (:499-508)
            float hs = diffuse_hammon(hn, neg(rd), L.light_dir, m.rough);
            v3 sun_brdf = muls(muls(mul(muls(m.albedo, hs), muls(L.light_color, 3.5f)), 1.0f - shadow_at), PI);
            v3 new_dir = cos_hemisphere(hn, rng);
            float cos_theta = clampf(dot(hn, new_dir), 0.0f, 1.0f);
            float pdf = fmaxg(cos_theta / PI, 0.00001f);
            float att = diffuse_hammon(hn, neg(rd), new_dir, m.rough);   // DiffuseRayBRDF (:527-531)
            contribution = add(contribution, mul(throughput, sun_brdf));
            contribution = add(contribution, mul(emissive_color, throughput));
            throughput = mul(throughput, divs(muls(m.albedo, att), pdf));
            rd = new_dir;
            ro = add(ip, muls(hn, bias));
        } else {
            float x = mixf(1.0f, 1.05f, L.sun_visibility);
            x = clampf(x * 1.0f * f->gi_sky_strength, 0.0f, 5.0f);
            v3 sky = muls(sky_color_at(rd), x);
            contribution = add(contribution, mul(sky, throughput));
            *skyhit = true;
            break;
        }
        if (i == 0) {
            const float dao = 2.0f;
            if (T < dao && T > 0.0f) ao = fmaxg(T / dao, 0.0f);
        }
    }
    return v4{contribution.x, contribution.y, contribution.z, ao};
}

// CalculateDirectionalLight (ColorPassFrag.glsl:419-451) with
// FresnelSchlickRoughness (:1205-1209), ndfGGX (:394-400), gaSchlickGGX (:402-412).
v3 fresnel_schlick_roughness(v3 eye, v3 n, v3 f0, float rough) {
    float cos_theta = clampf(dot(eye, n), 0.00001f, 1.0f);
    float k = dm_pow(1.0f - cos_theta, 5.0f);
    v3 m = mk3(fmaxg(1.0f - rough, f0.x), fmaxg(1.0f - rough, f0.y), fmaxg(1.0f - rough, f0.z));
    return add(f0, muls(sub(m, f0), k));
}

v3 directional_light(v3 viewer, v3 wp, v3 light_dir, v3 radiance, v3 radiance_s, v3 albedo, v3 n,
                     float rough, float metal, float shadow) {
    const float DIELECTRIC = 0.04f, Epsilon = 0.00001f;
    float sh = fming(shadow, 1.0f);
    v3 lo = normalize(sub(viewer, wp));
    float cos_lo = fmaxg(0.0f, dot(n, lo));
    v3 f0 = vmix(mk3(DIELECTRIC, DIELECTRIC, DIELECTRIC), albedo, metal);
    v3 li = light_dir;
    v3 lh = normalize(add(li, lo));
    float cos_li = fmaxg(0.0f, dot(n, li));
    float cos_lh = fmaxg(0.0f, dot(n, lh));
    v3 F = fresnel_schlick_roughness(lo, n, f0, rough);
    float alpha = rough * rough;
    float alpha_sq = alpha * alpha;
    float denom = (cos_lh * cos_lh) * (alpha_sq - 1.0f) + 1.0f;
    float D = alpha_sq / ((PI * denom) * denom);
    float r1 = rough + 1.0f;
    float k = (r1 * r1) / 8.0f;
    float G = (cos_li / (cos_li * (1.0f - k) + k)) * (cos_lo / (cos_lo * (1.0f - k) + k));
    v3 kd = vmix(sub(mk3(1, 1, 1), F), mk3(0, 0, 0), metal);
    v3 diffuse_brdf = mul(kd, albedo);
    v3 spec = divs(muls(muls(F, D), G), fmaxg(Epsilon, (4.0f * cos_li) * cos_lo));
    spec = vclamp(spec, 0.0f, 2.0f);
    v3 result = add(muls(mul(diffuse_brdf, radiance), cos_li), muls(mul(spec, radiance_s), cos_li));
    return muls(vclamp(result, 0.0f, 2.5f), clampf(1.0f - sh, 0.0f, 1.0f));
}

// BasicSaturation (ColorPassFrag.glsl:1227-1232)
inline v3 basic_saturation(v3 c, float adj) {
    float l = dot(c, mk3(0.2125f, 0.7154f, 0.0721f));
    return vmix(mk3(l, l, l), c, adj);
}

// KarisEnvBRDFApprox (ColorPassFrag.glsl:384-391)
inline v2 karis_env_brdf(float ndv, float rough) {
    float rx = rough * -1.0f + 1.0f;
    float ry = rough * -0.0275f + 0.0425f;
    float rz = rough * -0.572f + 1.040f;
    float rw = rough * 0.022f + -0.040f;
    float a004 = fming(rx * rx, dm_exp2(-9.28f * ndv)) * rx + ry;
    return v2{-1.04f * a004 + rz, 1.04f * a004 + rw};
}

}  // namespace

extern "C" {

void vpto_set_counters(uint64_t* counters) { g_counters = counters; }

int vpto_omp_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

float vpto_exp(float x) { return dm_exp(x); }
float vpto_exp2(float x) { return dm_exp2(x); }
float vpto_log2(float x) { return dm_log2(x); }
float vpto_pow(float x, float y) { return dm_pow(x, y); }
float vpto_sin(float x) { return dm_sin(x); }
float vpto_cos(float x) { return dm_cos(x); }
float vpto_half_round(float x) { return half_round(x); }

// World::GenerateDistanceField (Core/World.cpp:69-113): X, Y, Z passes in
// sequence, each a forward then a backward sweep along one axis.
void vpto_build_df(const uint8_t* vox, int X, int Y, int Z, uint8_t* df) {
    const int max_d = std::min(254, X + Y + Z);   // ManhattanDistanceX.comp:51
    const size_t sx = 1, sy = (size_t)X, sz = (size_t)X * Y;
    // ManhattanDistanceX.comp:45-68
#pragma omp parallel for schedule(static)
    for (int zy = 0; zy < Y * Z; zy++) {
        int y = zy % Y, z = zy / Y;
        uint8_t* d = df + y * sy + z * sz;
        const uint8_t* v = vox + y * sy + z * sz;
        d[0] = v[0] > 0 ? 0 : (uint8_t)max_d;
        for (int x = 1; x < X; x++)
            d[x * sx] = v[x * sx] > 0 ? 0 : (uint8_t)std::min(max_d, 1 + (int)d[(x - 1) * sx]);
        for (int x = X - 2; x >= 0; x--)
            if (d[(x + 1) * sx] < d[x * sx]) d[x * sx] = (uint8_t)(1 + d[(x + 1) * sx]);
    }
    // ManhattanDistanceY.comp:94-119
#pragma omp parallel for schedule(static)
    for (int zx = 0; zx < X * Z; zx++) {
        int x = zx % X, z = zx / X;
        uint8_t* d = df + x * sx + z * sz;
        for (int y = 1; y < Y; y++)
            if (d[(y - 1) * sy] < d[y * sy]) d[y * sy] = (uint8_t)(1 + d[(y - 1) * sy]);
        for (int y = Y - 2; y >= 0; y--)
            if (d[(y + 1) * sy] < d[y * sy]) d[y * sy] = (uint8_t)(1 + d[(y + 1) * sy]);
    }
    // ManhattanDistanceZ.comp:142-166
#pragma omp parallel for schedule(static)
    for (int yx = 0; yx < X * Y; yx++) {
        int x = yx % X, y = yx / X;
        uint8_t* d = df + x * sx + y * sy;
        for (int z = 1; z < Z; z++)
            if (d[(z - 1) * sz] < d[z * sz]) d[z * sz] = (uint8_t)(1 + d[(z - 1) * sz]);
        for (int z = Z - 2; z >= 0; z--)
            if (d[(z + 1) * sz] < d[z * sz]) d[z * sz] = (uint8_t)(1 + d[(z + 1) * sz]);
    }
}

// InitialRayTraceFrag.glsl main (:417-468)
void vpto_trace_primary(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                        int row0, int row1, vpto_gbuffer* out) {
    const int W = p->width, H = p->height;
    const v3 r0 = ray_origin(cam);
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = row0; j < row1; j++) {
        RowCount cnt;
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v3 dir = normalize(ray_dir_at(cam, texcoord(i, j, W, H)));
            TraceResult r = alpha_active(p) ? traverse_alpha(w, r0, dir, p->primary_max_steps, r0, alpha_k(cam->proj[5], W))
                                           : traverse(w, r0, dir, p->primary_max_steps);
            cnt.add(0, r.steps);
            bool intersect = r.t > 0.0f && r.block > 0;
            out->t[px] = storage(r.t, p->storage);
            out->face[px] = (uint8_t)(intersect ? normal_id(r.normal) : 10);
            out->block[px] = (uint8_t)(intersect ? r.block : 0);
            out->hit[px * 3 + 0] = r.cell[0];
            out->hit[px * 3 + 1] = r.cell[1];
            out->hit[px * 3 + 2] = r.cell[2];
            out->steps[px] = (uint16_t)r.steps;
        }
        cnt.flush();
    }
}

// ShadowRayTraceFrag.glsl main (:414-513): hard sun shadow, no cone jitter.
void vpto_trace_shadow(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                       const vpto_frame* f, const float* t, const uint8_t* face,
                       int row0, int row1, uint8_t* shadow) {
    const int W = p->width, H = p->height;
    const v3 r0 = ray_origin(cam);
    const v3 L = mk3(f->sun_dir[0], f->sun_dir[1], f->sun_dir[2]);
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = row0; j < row1; j++) {
        RowCount cnt;
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            float d = t[px];
            if (d < 0.0f) { shadow[px] = 0; continue; }
            v3 pos = add(r0, muls(normalize(ray_dir_at(cam, texcoord(i, j, W, H))), d));
            v3 n = normal_from_id(face[px], 1.0f);
            float ndl = dot(n, L);
            if (ndl <= 0.01f) { shadow[px] = 1; continue; }
            v3 o = add(pos, mul(n, mk3(0.06f, 0.06f, 0.06f)));
            int block_at = get_voxel(w, f2i(std::floor(o.x)), f2i(std::floor(o.y)), f2i(std::floor(o.z)));
            float T = -1.0f;
            if (d > 0.0f) {
                TraceResult r = alpha_active_shadows(p)
                                    ? traverse_alpha(w, o, L, p->shadow_max_steps, ray_origin(cam),
                                                     alpha_k(cam->proj[5], W), 0, -2)
                                    : traverse(w, o, L, p->shadow_max_steps);
                cnt.add(1, r.steps);
                T = r.t;
            }
            shadow[px] = (uint8_t)((T > 0.0f || block_at > 0) ? 1 : 0);
        }
        cnt.flush();
    }
}

// DiffuseRayTraceFrag.glsl main (:822-935)
// The diffuse GI and its filters run on a grid gi_divisor times coarser than
// the G-buffer: DiffuseTraceResolution = DiffuseIndirectSuperSampleRes = 1/d
// (Core/Pipeline.cpp:72, :79, :1702-1710; 1/4 by default, 1/2 in the higher
// presets :1256-1282). Every such pass sets its offsets in GI texels
// (u_Dimensions / textureSize of a GI plane, e.g. :2303, :2568).
inline int gi_div(const vpto_params* p) { return p->gi_divisor > 1 ? p->gi_divisor : 1; }

void vpto_gi_view(const vpto_params* p, const float* t, const uint8_t* face, const uint8_t* block,
                  float* t_view, uint8_t* face_view, uint8_t* block_view) {
    const int d = gi_div(p), W = p->width, H = p->height, Wg = W / d, Hg = H / d;
    const Plane T{t, W, H, 1};
    const Plane8 F{face, W, H}, B{block, W, H};
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Hg; j++) {
        for (int i = 0; i < Wg; i++) {
            const size_t q = (size_t)j * Wg + i;
            if (d == 1) {
                t_view[q] = t[q];
                face_view[q] = face[q];
                block_view[q] = block[q];
                continue;
            }
            const v2 uv = texcoord(i, j, Wg, Hg);
            float v;
            T.linear(uv, &v);
            t_view[q] = storage(v, p->storage);
            face_view[q] = (uint8_t)F.nearest(uv);
            block_view[q] = (uint8_t)B.nearest(uv);
        }
    }
}

void vpto_trace_diffuse(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                        const vpto_frame* f, const float* t, const uint8_t* face,
                        int row0, int row1, vpto_gi* out) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const v3 r0 = ray_origin(cam);
    const Lighting L = frame_lighting(f);
    const int fp16 = p->storage;
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = row0; j < row1; j++) {
        RowCount cnt;
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v2 uv = texcoord(i, j, W, H);
            v3 dir = normalize(ray_dir_at(cam, uv));
            float d = t[px];
            v3 pos = add(r0, muls(dir, d));
            v3 n = normal_from_id(face[px], 0.5f);
            float sh[4], cocg[2];
            if (d < 0.0f) {
                irradiance_to_sh(muls(sky_radiance(dir), 2.66f), n, sh, cocg);
                for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(sh[c], fp16);
                out->cocg[px * 2 + 0] = storage(cocg[0], fp16);
                out->cocg[px * 2 + 1] = storage(cocg[1], fp16);
                out->luma[px] = storage(luminance(mk3(0, 0, 0)), fp16);
                out->aosky[px * 2 + 0] = storage(1.0f, fp16);
                out->aosky[px * 2 + 1] = storage(0.0f, fp16);
                continue;
            }
            uint32_t rng = pixel_seed(f, (uint32_t)px);
            int spp = std::min(std::max(p->spp, 1), 32);
            if (L.moon_stronger) spp *= 2;
            float tot_sh[4] = {0, 0, 0, 0}, tot_cocg[2] = {0, 0};
            v3 radiance = mk3(0, 0, 0);
            float acc_ao = 0.0f, skyhits = 0.0f;
            for (int s = 0; s < spp; s++) {
                v3 odir = mk3(0, 0, 0);
                bool ss = false;
                v4 x = calculate_diffuse(w, p, f, L, pos, n, &rng, &odir, &ss, &cnt);
                v3 xc = vclamp(mk3(x.x, x.y, x.z), 0.0f, 8.0f);
                radiance = add(radiance, xc);
                acc_ao += x.w;
                irradiance_to_sh(xc, odir, sh, cocg);
                for (int c = 0; c < 4; c++) tot_sh[c] += sh[c];
                tot_cocg[0] += cocg[0];
                tot_cocg[1] += cocg[1];
                skyhits += ss ? 1.0f : 0.0f;
            }
            float fs = (float)spp;
            acc_ao /= fs;
            for (int c = 0; c < 4; c++) tot_sh[c] /= fs;
            tot_cocg[0] /= fs;
            tot_cocg[1] /= fs;
            radiance = divs(radiance, fs);
            skyhits /= fs;
            for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(clampf(tot_sh[c], -100.0f, 100.0f), fp16);
            out->cocg[px * 2 + 0] = storage(clampf(tot_cocg[0], -100.0f, 100.0f), fp16);
            out->cocg[px * 2 + 1] = storage(clampf(tot_cocg[1], -100.0f, 100.0f), fp16);
            out->luma[px] = storage(clampf(fmaxg(luminance(radiance), 0.01f), 0.001f, 64.0f), fp16);
            out->aosky[px * 2 + 0] = storage(clampf(acc_ao, 0.0f, 1.0f), fp16);
            out->aosky[px * 2 + 1] = storage(clampf(skyhits, 0.0f, 1.0f), fp16);
        }
        cnt.flush();
    }
}

// Spatial3x3Initial.glsl main (:96-176)
void vpto_spatial_initial(const vpto_camera* cam, const vpto_params* p,
                          const float* t, const uint8_t* face, const vpto_gi* in, vpto_gi* out) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const int fp16 = p->storage;
    const Plane T{t, W, H, 1}, SH{in->sh, W, H, 4}, CC{in->cocg, W, H, 2}, AO{in->aosky, W, H, 2};
    const Plane8 F{face, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float atrous_w[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v2 uv = texcoord(i, j, W, H);
            v4 bp = position_fetch(cam, T, i, j, uv);
            v3 bn = normal_from_id(F.at(i, j), 1.0f);
            float bsh[4], bcc[2], bao[2];
            for (int c = 0; c < 4; c++) bsh[c] = SH.at(i, j, c);
            for (int c = 0; c < 2; c++) { bcc[c] = CC.at(i, j, c); bao[c] = AO.at(i, j, c); }
            float bl = sh_to_y(bsh);
            float butil = in->luma[px];
            float tsh[4] = {bsh[0], bsh[1], bsh[2], bsh[3]}, tcc[2] = {bcc[0], bcc[1]};
            float tao[2] = {bao[0], bao[1]};
            float tw = 1.0f, taow = 1.0f;
            const float phi = 4.0f;
            for (int x = -1; x <= 1; x++) {
                for (int y = -1; y <= 1; y++) {
                    if (x == 0 && y == 0) continue;
                    int si = i + x, sj = j + y;
                    if (si < 0 || si >= W || sj < 0 || sj >= H) continue;   // InScreenSpace
                    v2 sc = v2{uv.x + (float)x * texel_x, uv.y + (float)y * texel_y};
                    v4 sp = position_fetch(cam, T, si, sj, sc);
                    v3 pd = mk3(std::fabs(sp.x - bp.x), std::fabs(sp.y - bp.y), std::fabs(sp.z - bp.z));
                    float dist_sqr = dot(pd, pd);
                    if (dist_sqr < 1.0f) {
                        float ssh[4], scc[2];
                        for (int c = 0; c < 4; c++) ssh[c] = SH.at(si, sj, c);
                        for (int c = 0; c < 2; c++) scc[c] = CC.at(si, sj, c);
                        v3 sn = normal_from_id(F.at(si, sj), 1.0f);
                        float sl = sh_to_y(ssh);
                        float nw = dm_pow(fmaxg(dot(bn, sn), 0.0f), 16.0f);
                        float lw = std::fabs(sl - bl) / phi;
                        float wgt = dm_exp(-lw - nw);
                        wgt = fmaxg(wgt, 0.01f);
                        wgt = (atrous_w[std::abs(x)] * atrous_w[std::abs(y)]) * wgt;
                        wgt = fmaxg(wgt, 0.01f);
                        wgt = clampf(wgt, 0.0f, 1.0f);
                        for (int c = 0; c < 4; c++) tsh[c] += ssh[c] * wgt;
                        for (int c = 0; c < 2; c++) tcc[c] += scc[c] * wgt;
                        tw += wgt;
                        for (int c = 0; c < 2; c++) tao[c] += AO.at(si, sj, c) * wgt;
                        taow += wgt;
                    }
                }
            }
            tw = fmaxg(tw, 0.01f);
            for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(tsh[c] / tw, fp16);
            for (int c = 0; c < 2; c++) out->cocg[px * 2 + c] = storage(tcc[c] / tw, fp16);
            float aw = fmaxg(taow, 0.01f);
            for (int c = 0; c < 2; c++) out->aosky[px * 2 + c] = storage(tao[c] / aw, fp16);
            out->luma[px] = storage(butil, fp16);
        }
    }
}

// How many x with bit patterns in [lo, hi) give a division x / c different
// from the three-operation form the device uses for a constant divisor:
// q = x * RN(1/c), then one correction with the exact remainder,
// q + fma(-q, c, x) * RN(1/c) (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990). An exhaustive run over every non-negative finite float is what
// allows the form for a given c.
uint64_t vpto_check_div_const(float c, uint32_t lo, uint32_t hi) {
    const float y = 1.0f / c;
    uint64_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
    for (int64_t u = (int64_t)lo; u < (int64_t)hi; u++) {
        uint32_t b = (uint32_t)u;
        float x;
        std::memcpy(&x, &b, 4);
        const float q = x * y;
        const float r = std::fma(-q, c, x);
        const float d = std::fma(r, y, q);
        const float e = x / c;
        uint32_t bd, be;
        std::memcpy(&bd, &d, 4);
        std::memcpy(&be, &e, 4);
        bad += bd != be;
    }
    return bad;
}

// The oracle's vector builtins over n inputs, for the comparison with glm:
// op 0 dot, 1 cross, 2 length, 3 normalize, 4 mix (scalar), 5 mat4 * vec4.
void vpto_vecmath(int op, const float* a, const float* b, const float* c, float* out, int n) {
    for (int k = 0; k < n; k++) {
        if (op == 5) {
            const v4 r = mat_mul4(a + 16 * k, b[4 * k], b[4 * k + 1], b[4 * k + 2], b[4 * k + 3]);
            out[4 * k] = r.x;
            out[4 * k + 1] = r.y;
            out[4 * k + 2] = r.z;
            out[4 * k + 3] = r.w;
            continue;
        }
        const v3 x = mk3(a[3 * k], a[3 * k + 1], a[3 * k + 2]), y = mk3(b[3 * k], b[3 * k + 1], b[3 * k + 2]);
        v3 r = mk3(0.0f, 0.0f, 0.0f);
        switch (op) {
            case 0: r.x = dot(x, y); break;
            case 1: r = cross(x, y); break;
            case 2: r.x = length(x); break;
            case 3: r = normalize(x); break;
            case 4: r.x = mixf(x.x, y.x, c[3 * k]); break;
            default: break;
        }
        out[3 * k] = r.x;
        out[3 * k + 1] = r.y;
        out[3 * k + 2] = r.z;
    }
}

// u_PrevProjection * u_PrevView (SVGF/TemporalFilter.glsl:61-68), a 4x4
// product evaluated left to right.
static void prev_view_proj(const vpto_camera* prev_cam, float* m) {
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            m[c * 4 + r] = ((prev_cam->proj[0 * 4 + r] * prev_cam->view[c * 4 + 0] +
                             prev_cam->proj[1 * 4 + r] * prev_cam->view[c * 4 + 1]) +
                            prev_cam->proj[2 * 4 + r] * prev_cam->view[c * 4 + 2]) +
                           prev_cam->proj[3 * 4 + r] * prev_cam->view[c * 4 + 3];
}

// Reprojection(ProjectPositionPrevious(pos)) (SVGF/TemporalFilter.glsl:61-73):
// the previous frame's texture coordinate of world position pos.
static inline v2 reproject(const float* m, v4 pos) {
    v4 pr = mat_mul4(m, pos.x, pos.y, pos.z, 1.0f);
    return v2{(pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f};
}

// The world position GetPositionAt gives each texel of the hit-distance plane
// t and its reprojected coordinate, as the temporal pass computes them.
void vpto_reproject(const vpto_camera* cam, const vpto_camera* prev_cam, int W, int H, const float* t, float* pos,
                    float* uv_prev) {
    const Plane T{t, W, H, 1};
    float m[16];
    prev_view_proj(prev_cam, m);
    for (int j = 0; j < H; j++)
        for (int i = 0; i < W; i++) {
            const size_t px = (size_t)j * W + i;
            const v4 bp = position_fetch(cam, T, i, j, texcoord(i, j, W, H));
            const v2 rc = reproject(m, bp);
            pos[px * 3 + 0] = bp.x;
            pos[px * 3 + 1] = bp.y;
            pos[px * 3 + 2] = bp.z;
            uv_prev[px * 2 + 0] = rc.x;
            uv_prev[px * 2 + 1] = rc.y;
        }
}

// SVGF/TemporalFilter.glsl main (:132-360)
void vpto_temporal(const vpto_camera* cam, const vpto_camera* prev_cam, const vpto_params* p,
                   const vpto_frame* f,
                   const float* t, const uint8_t* face, const uint8_t* block,
                   const float* prev_t, const uint8_t* prev_face, const uint8_t* prev_block,
                   const vpto_gi* cur, const vpto_history* prev, vpto_history* out) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const int fp16 = p->storage;
    const Plane T{t, W, H, 1}, PT{prev_t, p->width, p->height, 1};
    const Plane8 F{face, W, H}, B{block, W, H}, PF{prev_face, p->width, p->height}, PB{prev_block, p->width, p->height};
    const Plane PSH{prev->sh, W, H, 4}, PCC{prev->cocg, W, H, 2}, PU{prev->util, W, H, 4}, PAO{prev->aosky, W, H, 2};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    float m[16];
    prev_view_proj(prev_cam, m);
    const float weights[5] = {3.0f / 32.0f, 3.0f / 32.0f, 9.0f / 64.0f, 3.0f / 32.0f, 3.0f / 32.0f};
    const int offs[5][2] = {{1, 0}, {0, 1}, {0, 0}, {-1, 0}, {0, -1}};
    const bool be_useful = f->temporal != 0;
    const v3 viewer = ray_origin(cam);
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v2 uv = texcoord(i, j, W, H);
            v4 bp = position_fetch(cam, T, i, j, uv);
            v3 bn = normal_from_id(F.at(i, j), 1.0f);
            float bsh[4], bcc[2], bao[2];
            for (int c = 0; c < 4; c++) bsh[c] = cur->sh[px * 4 + c];
            for (int c = 0; c < 2; c++) { bcc[c] = cur->cocg[px * 2 + c]; bao[c] = cur->aosky[px * 2 + c]; }
            v2 rc = reproject(m, bp);
            float base_lum = cur->luma[px];
            int base_block = std::min(std::max((int)B.at(i, j), 0), 127);
            float tol = 0.75f;
            bool do_block = true, do_normal = true;
            float dp = length(sub(mk3(bp.x, bp.y, bp.z), viewer));
            if (dp < 4.0f) { tol = 0.3f; }
            else if (dp < 6.0f) { tol = 0.65f; }
            else if (dp < 8.0f) { tol = 0.85f; }
            else if (dp < 16.0f) { tol = 1.414f; }
            else if (dp < 32.0f) { tol = 2.4f; }
            else if (dp < 48.0f) { tol = 3.5f; do_block = false; }
            else if (dp < 64.0f) { tol = 4.2f; do_block = false; }
            else if (dp < 96.0f) { tol = 6.25f; do_block = false; do_normal = false; }
            else if (dp < 128.0f) { tol = 9.0f; do_block = false; do_normal = false; }
            else if (dp < 200.0f) { tol = 14.0f; do_block = false; do_normal = false; }
            float tw = 0.0f, ssh[4] = {0, 0, 0, 0}, scc[2] = {0, 0}, sao[2] = {0, 0};
            float slum = 0.0f, sspp = 0.0f, smom = 0.0f;
            int successful = 0;
            for (int k = 0; k < 5; k++) {
                // Jitter is ivec2((noise - 0.5) * 1.0) == 0 for every pixel (:165)
                v2 sc = v2{rc.x + ((float)offs[k][0] + 0.0f) * texel_x, rc.y + ((float)offs[k][1] + 0.0f) * texel_y};
                const float b = 0.0035f;
                if (!(sc.x < 1.0f - b && sc.x > b && sc.y < 1.0f - b && sc.y > b)) continue;
                v4 pp = position_linear(cam, PT, sc);
                v3 pn = normal_from_id(PF.nearest(sc), 1.0f);
                v3 pd = mk3(std::fabs(bp.x - pp.x), std::fabs(bp.y - pp.y), std::fabs(bp.z - pp.z));
                float perr = dot(pd, pd);
                float cw = weights[k];
                int sblock = std::min(std::max(PB.nearest(sc), 0), 127);
                bool valid = false;
                if (perr < tol && ((pp.w < 0.0f) == (bp.w < 0.0f))) {
                    valid = true;
                    if (do_normal && !(pn.x == bn.x && pn.y == bn.y && pn.z == bn.z)) valid = false;
                    if (do_block && base_block != sblock) valid = false;
                }
                if (valid) {
                    float pu[4], psh[4], pcc[2], pao[2];
                    PU.linear(sc, pu);
                    PSH.linear(sc, psh);
                    PCC.linear(sc, pcc);
                    PAO.linear(sc, pao);
                    for (int c = 0; c < 4; c++) ssh[c] += psh[c] * cw;
                    for (int c = 0; c < 2; c++) scc[c] += pcc[c] * cw;
                    sspp += pu[0] * cw;
                    smom += pu[1] * cw;
                    slum += pu[2] * cw;
                    for (int c = 0; c < 2; c++) sao[c] += pao[c] * cw;
                    tw += cw;
                    successful++;
                }
            }
            if (tw > 0.001f) {
                for (int c = 0; c < 4; c++) ssh[c] /= tw;
                for (int c = 0; c < 2; c++) scc[c] /= tw;
                smom /= tw;
                sspp /= tw;
                slum /= tw;
                for (int c = 0; c < 2; c++) sao[c] /= tw;
            } else {
                successful = 0;
            }
            float inc = be_useful ? 1.0f : 0.0f;
            float spp_inc = sspp + inc;
            if (successful <= 0) spp_inc = 0.01f;
            float blend = fmaxg(1.0f / spp_inc, 0.05f);
            float mfac = fmaxg(1.0f / spp_inc, 0.05f);
            if (!be_useful) { blend = 0.99f; sspp = 0.0f; }
            float util_spp = spp_inc;
            if (successful <= 0) util_spp = 0.0f;
            float util_mom = (1.0f - mfac) * smom + mfac * (base_lum * base_lum);
            float store_luma = mixf(slum, base_lum, blend);
            float osh[4], occ[2], oao[2];
            for (int c = 0; c < 4; c++) osh[c] = mixf(ssh[c], bsh[c], blend);
            for (int c = 0; c < 2; c++) { occ[c] = mixf(scc[c], bcc[c], blend); oao[c] = mixf(sao[c], bao[c], blend); }
            if (successful <= 0) {
                for (int c = 0; c < 4; c++) osh[c] = bsh[c];
                for (int c = 0; c < 2; c++) { occ[c] = bcc[c]; oao[c] = bao[c]; }
            }
            for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(clampf(osh[c], -100.0f, 100.0f), fp16);
            for (int c = 0; c < 2; c++) out->cocg[px * 2 + c] = storage(clampf(occ[c], -10.0f, 100.0f), fp16);
            for (int c = 0; c < 2; c++) out->aosky[px * 2 + c] = storage(clampf(oao[c], 0.0f, 1.0f), fp16);
            out->util[px * 4 + 0] = storage(clampf(util_spp, -150.0f, 150.0f), fp16);
            out->util[px * 4 + 1] = storage(clampf(util_mom, -150.0f, 150.0f), fp16);
            out->util[px * 4 + 2] = storage(clampf(store_luma, -150.0f, 150.0f), fp16);
            out->util[px * 4 + 3] = 0.0f;
        }
    }
}

// SVGF/VarianceEstimate.glsl main (:73-193), DO_SPATIAL and
// AGGRESSIVE_DISOCCLUSION_HANDLING on (Core/Pipeline.cpp:2451-2452).
void vpto_variance(const vpto_camera* cam, const vpto_params* p,
                   const float* t, const uint8_t* face, const vpto_history* in, vpto_filtered* out) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const int fp16 = p->storage;
    const Plane T{t, W, H, 1}, SH{in->sh, W, H, 4}, CC{in->cocg, W, H, 2}, U{in->util, W, H, 4};
    const Plane8 F{face, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float thresh = 4.0f + 4.0f + 4.0f;
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v2 uv = texcoord(i, j, W, H);
            v4 bp = position_fetch(cam, T, i, j, uv);
            v3 bn = normal_from_id(F.at(i, j), 1.0f);
            float bsh[4], bcc[2];
            for (int c = 0; c < 4; c++) bsh[c] = SH.at(i, j, c);
            for (int c = 0; c < 2; c++) bcc[c] = CC.at(i, j, c);
            float bl = sh_to_y(bsh);
            float acc = U.at(i, j, 0);
            float bm = U.at(i, j, 1);
            float osh[4], occ[2], var;
            if (acc < thresh) {
                const float phi = 5.0f;
                float tw = 0.0f, tm = 0.0f, tl = 0.0f, tw2 = 0.0f;
                float tsh[4] = {0, 0, 0, 0}, tcc[2] = {0, 0};
                for (int x = -4; x <= 4; x++) {
                    for (int y = -4; y <= 4; y++) {
                        int si = i + x, sj = j + y;
                        if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
                        v2 sc = v2{uv.x + (float)x * texel_x, uv.y + (float)y * texel_y};
                        v4 sp = position_fetch(cam, T, si, sj, sc);
                        v3 sn = normal_from_id(F.at(si, sj), 1.0f);
                        float smom = U.at(si, sj, 1);
                        float ssh[4], scc[2];
                        for (int c = 0; c < 4; c++) ssh[c] = SH.at(si, sj, c);
                        for (int c = 0; c < 2; c++) scc[c] = CC.at(si, sj, c);
                        float sl = sh_to_y(ssh);
                        float nw = dm_pow(fmaxg(dot(bn, sn), 0.0f), 16.0f);
                        float dw = dm_pow(dm_exp(-std::fabs(sp.w - bp.w)), 2.0f);
                        float lw = std::fabs(sl - bl) / phi;
                        float wgt = (dm_exp(-lw) * nw) * dw;
                        float wgt2 = wgt;
                        wgt = fmaxg(wgt, 0.000000015f);
                        wgt2 = fmaxg(wgt2, 0.0000000015f);
                        tw += wgt;
                        tm += smom * wgt2;
                        for (int c = 0; c < 4; c++) tsh[c] += ssh[c] * wgt;
                        for (int c = 0; c < 2; c++) tcc[c] += scc[c] * wgt;
                        tl += sl * wgt2;
                        tw2 += wgt2;
                    }
                }
                if (tw > 0.0f) {
                    tm /= tw2;
                    tl /= tw2;
                    for (int c = 0; c < 2; c++) tcc[c] /= tw;
                    for (int c = 0; c < 4; c++) tsh[c] /= tw;
                }
                for (int c = 0; c < 4; c++) osh[c] = tsh[c];
                for (int c = 0; c < 2; c++) occ[c] = tcc[c];
                float al = tl * tl;
                var = tm - al;
                var *= 3.0f;
            } else {
                for (int c = 0; c < 4; c++) osh[c] = bsh[c];
                for (int c = 0; c < 2; c++) occ[c] = bcc[c];
                var = bm - bl * bl;
            }
            var *= thresh / acc;
            for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(clampf(osh[c], -100.0f, 100.0f), fp16);
            for (int c = 0; c < 2; c++) out->cocg[px * 2 + c] = storage(clampf(occ[c], -10.0f, 100.0f), fp16);
            out->variance[px] = storage(clampf(var, -1.0f, 50.0f), fp16);
        }
    }
}

// SVGF/SpatialFilter.glsl main (:175-355), u_LargeKernel off, DO_SPATIAL on.
void vpto_atrous(const vpto_camera* cam, const vpto_params* p, const vpto_frame* f, int step,
                 const float* t, const uint8_t* face, const float* t_view, const uint8_t* face_view,
                 const float* temporal_util, const vpto_filtered* in, const float* in_aosky, vpto_filtered* out) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const int fp16 = p->storage;
    // taps sample the full-resolution depth and face planes at arbitrary
    // points; the centre reads them at its own GI texel centre (the views)
    const Plane T{t, p->width, p->height, 1}, TV{t_view, W, H, 1};
    const Plane SH{in->sh, W, H, 4}, CC{in->cocg, W, H, 2}, V{in->variance, W, H, 1};
    const Plane AO{in_aosky, W, H, 2}, U{temporal_util, W, H, 4};
    const Plane8 F{face, p->width, p->height}, FV{face_view, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float atrous_w[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    const float gauss[2] = {0.60283f, 0.198585f};
    const bool filter_ao = step <= 4;
    const bool filter_sky = (step <= 6) || filter_ao;
    const float add_scale = mixf(1.0f, 2.4f, p->resolution_scale);
    const float phi_bias = fmaxg(p->color_phi_bias, 0.1f);
    const float tmod = f->time * 100.493850275f;
    const float tmod500 = tmod - 500.0f * std::floor(tmod / 500.0f);   // GLSL mod
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v2 uv = texcoord(i, j, W, H);
            // GradientNoise (:160-165)
            float gx = ((float)i + 0.5f) + tmod500, gy = ((float)j + 0.5f) + tmod500;
            float noise = fract(52.9829189f * fract(0.06711056f * gx + 0.00583715f * gy));
            int jit = f2i((noise - 0.5f) * ((float)step * 0.8f));
            float bd = TV.at(i, j, 0);
            v3 bn = normal_from_id(FV.at(i, j), 1.0f);
            float bsh[4], bcc[2], bao[2];
            for (int c = 0; c < 4; c++) bsh[c] = SH.at(i, j, c);
            for (int c = 0; c < 2; c++) { bcc[c] = CC.at(i, j, c); bao[c] = AO.at(i, j, c); }
            float bl = sh_to_y(bsh);
            // GaussianVariance (:94-129)
            float bvar = 0.0f, vsum = 0.0f, tk = 0.0f;
            for (int x = -1; x <= 1; x++) {
                for (int y = -1; y <= 1; y++) {
                    int si = i + x, sj = j + y;
                    if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
                    float kv = gauss[std::abs(x)] * gauss[std::abs(y)];
                    float v = V.at(si, sj, 0);
                    if (x == 0 && y == 0) bvar = v;
                    vsum += v * kv;
                    tk += kv;
                }
            }
            float vest = vsum / fmaxg(tk, 0.01f);
            float tsh[4] = {bsh[0], bsh[1], bsh[2], bsh[3]}, tcc[2] = {bcc[0], bcc[1]};
            float tw = 1.0f, tvar = bvar, tao[2] = {bao[0], bao[1]}, taow = 1.0f;
            float acc_frames = U.at(i, j, 0);
            bool strong = acc_frames <= 8.0f && step <= 8;
            float curve = 0.0f;
            if (vest < 0.01f) curve = 128.0f;
            else if (vest < 0.025f) curve = 112.0f;
            else if (vest < 0.05f) curve = 96.0f;
            else if (vest < 0.075f) curve = 84.0f;
            else if (vest < 0.1f) curve = 70.0f;
            float tweaked = vest;
            if (vest < 0.1f) {   // TweakVariance (:167-173)
                float fe = clampf(vest, 0.0f, 1.0f);
                float tt = 1.0f - fe;
                tweaked = fe * dm_pow(tt, curve + 6.0f);
            }
            float phi = std::sqrt(fmaxg(0.0f, 0.000001f + tweaked));
            phi /= phi_bias;
            for (int x = -1; x <= 1; x++) {
                for (int y = -1; y <= 1; y++) {
                    if (x == 0 && y == 0) continue;
                    float ox = ((float)x * (float)step) * add_scale + (float)jit * 0.5f;
                    float oy = ((float)y * (float)step) * add_scale + (float)jit * 0.5f;
                    v2 sc = v2{uv.x + ox * texel_x, uv.y + oy * texel_y};
                    if (!(sc.x > 0.0f && sc.x < 1.0f && sc.y > 0.0f && sc.y < 1.0f)) continue;
                    float sd;
                    T.linear(sc, &sd);
                    float dd = std::fabs(sd - bd);
                    v3 sn = normal_from_id(F.nearest(sc), 1.0f);
                    if ((bd < 0.0f) == (dd < 0.0f)) {
                        float ssh[4], scc[2], sv;
                        SH.linear(sc, ssh);
                        CC.linear(sc, scc);
                        float sl = sh_to_y(ssh);
                        V.linear(sc, &sv);
                        float nw = clampf(dm_pow(fmaxg(dot(bn, sn), 0.0f), 32.0f), 0.001f, 1.0f);
                        float lw = std::fabs(sl - bl) / phi;
                        float dw = clampf(dm_pow(dm_exp(-fmaxg(dd, 0.00001f)), 2.0f), 0.0001f, 1.0f);
                        float wgt = strong ? nw * dw : (dm_exp(-lw) * nw) * dw;
                        wgt = clampf(wgt, 0.001f, 1.0f);
                        float xw = atrous_w[std::abs(x)], yw = atrous_w[std::abs(y)];
                        wgt = (xw * yw) * wgt;
                        wgt = fmaxg(wgt, 0.00000001f);
                        for (int c = 0; c < 4; c++) tsh[c] += ssh[c] * wgt;
                        for (int c = 0; c < 2; c++) tcc[c] += scc[c] * wgt;
                        tvar += (wgt * wgt) * sv;
                        tw += wgt;
                        if (filter_sky || filter_ao) {
                            float aw = clampf(((xw * yw) * nw) * dw, 0.000001f, 1.0f);
                            float sao[2];
                            AO.linear(sc, sao);
                            tao[0] += sao[0] * aw;
                            tao[1] += sao[1] * aw;
                            taow += aw;
                        }
                    }
                }
            }
            for (int c = 0; c < 4; c++) tsh[c] /= tw;
            for (int c = 0; c < 2; c++) tcc[c] /= tw;
            tvar /= (tw * tw);
            tao[0] /= taow;
            tao[1] /= taow;
            if (!filter_ao) tao[0] = bao[0];
            for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(clampf(tsh[c], -100.0f, 100.0f), fp16);
            for (int c = 0; c < 2; c++) out->cocg[px * 2 + c] = storage(clampf(tcc[c], -10.0f, 100.0f), fp16);
            out->variance[px] = storage(clampf(tvar, -1.0f, 50.0f), fp16);
            out->aosky[px * 2 + 0] = storage(clampf(tao[0], 0.0f, 1.0f), fp16);
            out->aosky[px * 2 + 1] = storage(clampf(tao[1], 0.0f, 1.0f), fp16);
        }
    }
}

// The PBR G-buffer's roughness / metalness (GenerateGBuffer.glsl: nearest
// filtered, 0 for the sky, :362-363) for flat materials.
inline float pbr_rough(const vpto_world* w, int block) {
    return block > 0 ? material(w, std::min(block, 127)).rough : 0.0f;
}
inline float pbr_metal(const vpto_world* w, int block) {
    return block > 0 ? material(w, std::min(block, 127)).metal : 0.0f;
}

// texture(u_GBufferNormals, uv): the RGB16F normal G-buffer with GL_LINEAR,
// i.e. the face normals ((1, 1, 1) for the sky, :362) blended bilinearly.
inline v3 gnormal_linear(const Plane8& F, v2 uv) {
    const float x = uv.x * (float)F.W - 0.5f, y = uv.y * (float)F.H - 0.5f;
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float ax = x - x0, ay = y - y0;
    const int i0 = f2i(x0), j0 = f2i(y0);
    const v3 n00 = normal_from_id(F.at(i0, j0), 1.0f), n10 = normal_from_id(F.at(i0 + 1, j0), 1.0f);
    const v3 n01 = normal_from_id(F.at(i0, j0 + 1), 1.0f), n11 = normal_from_id(F.at(i0 + 1, j0 + 1), 1.0f);
    auto bl = [&](float a, float b, float c, float d) {
        const float lo = a * (1.0f - ax) + b * ax;
        const float hi = c * (1.0f - ax) + d * ax;
        return lo * (1.0f - ay) + hi * ay;
    };
    return mk3(bl(n00.x, n10.x, n01.x, n11.x), bl(n00.y, n10.y, n01.y, n11.y), bl(n00.z, n10.z, n01.z, n11.z));
}

// SpatiallyUpscaleBuffers (ColorPassFrag.glsl:535-653), which the colour pass
// always runs (:828): a 3x3 joint-bilateral gather of the GI planes with the
// a-trous kernel, depth weight exp(-2|dd|)^5.25 and normal weight
// max(n.n', 1e-6)^16; beyond 128 units the sun shadow is filtered over the
// centre and its four immediate neighbours, otherwise read at the pixel
// (BetterTexture at a texel centre); then +0.05 shadow bias (:641-643). Taps
// are one GI texel apart (TexelSize of u_DiffuseSHy, :565), so on a GI grid d
// times coarser they land on the G-buffer texel centres d texels apart (read
// there, REPEAT wrapped: the shader has no screen-space test here) and between
// GI texels (bilinear); with d = 1 every tap is a texel centre of both.
// With a reflection pass the specular indirect is gathered too, weighted by
// the GI weight / (12 |roughness - base roughness| + 1) * max(n.n', 0)^8
// (:595-603, the G-buffer's roughness and normal being the block's and the
// face's for flat materials).
struct UpscaledGI {
    float sh[4], cocg[2], ao, shadow, spec[4];
};
// With block textures (GN, GP non-null) the specular gather reads the tap's
// roughness and normal-mapped normal from the textured G-buffer
// (u_GBufferPBR, u_GBufferNormals, :596-599) against the base pixel's base_hf.
inline UpscaledGI upscale_gi(const vpto_world* w, const Plane& T, const Plane8& F, const Plane8& B, const Plane8& S,
                             const Plane& SH, const Plane& CC, const Plane& AO, const Plane* SP, int d, int i, int j,
                             v2 uv, v3 base_n, float base_d, float base_rough, const Plane* GN, const Plane* GP,
                             v3 base_hf) {
    const float texel_x = 1.0f / (float)SH.W, texel_y = 1.0f / (float)SH.H;
    static const float kw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    UpscaledGI u{};
    float tsh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, tcc[2] = {0.0f, 0.0f}, tsp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float tao = 0.0f, tw = 0.0f, tshadow = 0.0f, tsw = 0.0f, tspw = 0.0f;
    const bool filter_shadows = base_d > 128.0f;
    if (!filter_shadows) tshadow = (float)S.at(i, j);
    for (int x = -1; x <= 1; x++) {
        for (int y = -1; y <= 1; y++) {
            const int si = i + d * x, sj = j + d * y;
            float ssh[4], scc[2], sao[2], ssp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (d == 1) {
                for (int c = 0; c < 4; c++) ssh[c] = SH.at(si, sj, c);
                for (int c = 0; c < 2; c++) { scc[c] = CC.at(si, sj, c); sao[c] = AO.at(si, sj, c); }
                if (SP)
                    for (int c = 0; c < 4; c++) ssp[c] = SP->at(si, sj, c);
            } else {
                const v2 sc = v2{uv.x + (float)x * texel_x, uv.y + (float)y * texel_y};
                SH.linear(sc, ssh);
                CC.linear(sc, scc);
                AO.linear(sc, sao);
                if (SP) SP->linear(sc, ssp);
            }
            const float lda = 1.0f / (1.0f / T.at(si, sj, 0));
            const float ed = dm_exp(-(std::fabs(lda - base_d) * 2.0f));
            const float dw = dm_pow(ed, 5.25f);
            const v3 na = normal_from_id(F.at(si, sj), 1.0f);
            float nw = dm_pow(fmaxg(dot(na, base_n), 0.000001f), 16.0f);
            nw = fmaxg(nw, 0.0001f);
            const float kwt = kw[std::abs(x)] * kw[std::abs(y)];
            float wgt = clampf((nw * dw) * kwt, 0.0f, 1.0f);
            if (SP) {
                float ra, nsp;
                if (GN) {
                    ra = GP->at(si, sj, 0);
                    const v3 hf = mk3(GN->at(si, sj, 0), GN->at(si, sj, 1), GN->at(si, sj, 2));
                    nsp = dm_pow(fmaxg(dot(hf, base_hf), 0.0f), 8.0f);
                } else {
                    ra = pbr_rough(w, B.at(si, sj));
                    nsp = dm_pow(fmaxg(dot(na, base_n), 0.0f), 8.0f);
                }
                float spw = (wgt / ((std::fabs(ra - base_rough) * 12.0f) + 1.0f)) * nsp;
                spw = fmaxg(spw, 0.00000001f);
                for (int c = 0; c < 4; c++) tsp[c] += ssp[c] * spw;
                tspw += spw;
            }
            wgt = fmaxg(wgt, 0.00000001f);
            for (int c = 0; c < 4; c++) tsh[c] += ssh[c] * wgt;
            for (int c = 0; c < 2; c++) tcc[c] += scc[c] * wgt;
            tao += sao[0] * wgt;
            tw += wgt;
            if (filter_shadows && (x == 0 || y == 0)) {   // IsImmediateNeighbour (:524-530)
                const float sw = (kwt * clampf(dm_pow(ed, 32.0f), 0.00001f, 1.0f)) * (nw * nw);
                tshadow += (float)S.at(si, sj) * sw;
                tsw += sw;
            }
        }
    }
    tw = fmaxg(tw, 0.0000001f);
    for (int c = 0; c < 4; c++) u.sh[c] = tsh[c] / tw;
    for (int c = 0; c < 2; c++) u.cocg[c] = tcc[c] / tw;
    u.ao = tao / tw;
    tspw = fmaxg(tspw, 0.0000001f);
    for (int c = 0; c < 4; c++) u.spec[c] = tsp[c] / tspw;
    if (filter_shadows) tshadow = tshadow / tsw;
    tshadow += 0.05f;
    u.shadow = clampf(tshadow, 0.00000000000001f, 1.0f);
    return u;
}

// ColorPassFrag.glsl main (:747-1083), u_UseDFG on (Core/Pipeline.cpp:3683),
// VXAO with cutoff (:3669, :3679) only under SVGF (u_SVGFEnabled, :3680).
// Flat materials (gb_* NULL): the block table's albedo, roughness,
// metalness and emission, the face normal and a texture AO of 1; with block
// textures the textured G-buffer's albedo, normal-mapped normal, PBR and AO
// (u_GBufferAlbedos, u_GBufferNormals, u_GBufferPBR, u_GBufferAO, :797-803),
// the face normal staying where the shader reads u_NormalTexture.
static void shade_impl(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                       const vpto_frame* f, const float* t, const uint8_t* face, const uint8_t* block,
                       const uint8_t* shadow, const float* sh, const float* cocg, const float* aosky,
                       const float* spec, int row0, int row1, float* rgb, const float* gb_albedo,
                       const float* gb_normal, const float* gb_pbr, const float* gb_ao) {
    const int W = p->width, H = p->height;
    const int fp16 = p->storage;
    const v3 viewer = mk3(cam->position[0], cam->position[1], cam->position[2]);
    const v3 r0 = ray_origin(cam);
    const v3 sun = mk3(f->sun_dir[0], f->sun_dir[1], f->sun_dir[2]);
    const v3 moon = moon_dir_of(sun);
    const v3 sun_color = mk3(f->sun_radiance[0], f->sun_radiance[1], f->sun_radiance[2]);
    const v3 moon_color = mk3(f->moon_radiance[0], f->moon_radiance[1], f->moon_radiance[2]);
    float sun_vis = clampf(dot(sun, mk3(0.0f, 1.0f, 0.0f)) + 0.05f, 0.0f, 0.1f) * 12.0f;
    sun_vis = 1.0f - sun_vis;
    const bool vxao = p->denoiser == 0;
    const int d = gi_div(p), Wg = W / d, Hg = H / d;
    const Plane T{t, W, H, 1}, SH{sh, Wg, Hg, 4}, CC{cocg, Wg, Hg, 2}, AO{aosky, Wg, Hg, 2}, SP{spec, Wg, Hg, 4};
    const Plane8 F{face, W, H}, B{block, W, H}, S{shadow, W, H};
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = row0; j < row1; j++) {
        for (int i = 0; i < W; i++) {
            size_t px = (size_t)j * W + i;
            v2 uv = texcoord(i, j, W, H);
            v3 dir = normalize(ray_dir_at(cam, uv));
            // SamplePositionAt (:1122-1126) reads 1/t from the R32F depth plane
            float dist = 1.0f / (1.0f / t[px]);
            v3 wp = add(r0, muls(dir, dist));
            v3 n = normal_from_id(face[px], 1.0f);
            v3 color;
            if (dist > 0.0f) {
                int bid = std::min(std::max((int)block[px], 0), 127);
                const Material m = material(w, bid);
                v3 base_albedo = m.albedo, nh = n;
                float rough = m.rough, metal = m.metal, emissivity = (float)m.emissive, tex_ao = 1.0f;
                const bool tex = gb_albedo != nullptr;
                if (tex) {
                    base_albedo = mk3(gb_albedo[px * 3], gb_albedo[px * 3 + 1], gb_albedo[px * 3 + 2]);
                    nh = mk3(gb_normal[px * 3], gb_normal[px * 3 + 1], gb_normal[px * 3 + 2]);
                    rough = gb_pbr[px * 4];
                    metal = gb_pbr[px * 4 + 1];
                    emissivity = gb_pbr[px * 4 + 3];
                    tex_ao = gb_ao[px];
                }
                v3 albedo = basic_saturation(base_albedo, 1.0f - 0.1f);   // u_TextureDesatAmount = 0.1
                if (metal >= 0.1f - 0.01f) albedo = basic_saturation(albedo, 0.9f);
                const Plane GN{gb_normal, W, H, 3}, GP{gb_pbr, W, H, 4};
                const UpscaledGI up = upscale_gi(w, T, F, B, S, SH, CC, AO, spec ? &SP : nullptr, d, i, j, uv, n, dist,
                                                 rough, tex ? &GN : nullptr, tex ? &GP : nullptr, nh);
                float up_shadow = clampf(up.shadow, 0.0f, 1.0f);
                float rt_shadow = clampf(clampf(up_shadow + 0.0f, 0.0f, 1.0f), 0.0f, 1.0f);
                v3 indirect = sh_to_irradiance(up.sh, up.cocg, nh);   // IndirectN = NormalMapped (:834-840)
                const float vb = 0.00125f;
                if (vxao && uv.x > vb && uv.x < 1.0f - vb && uv.y > vb && uv.y < 1.0f - vb) {
                    float ao = up.ao;
                    float dxz = std::sqrt((wp.x - viewer.x) * (wp.x - viewer.x) + (wp.z - viewer.z) * (wp.z - viewer.z));
                    float fade = dxz < 256.0f ? 0.0f : 1.0f;
                    ao = mixf(ao, 1.0f, fade);
                    ao = dm_pow(ao, 2.2f);
                    indirect = muls(indirect, clampf(ao, 0.05f, 1.0f));
                }
                float sampled_ao = dm_pow(tex_ao, 1.25f);
                v3 sun_direct = directional_light(viewer, wp, sun, sun_color, sun_color, albedo, nh, rough, metal, rt_shadow);
                v3 moon_direct = directional_light(viewer, wp, moon, moon_color, moon_color, albedo, nh, rough, metal, rt_shadow);
                v3 direct = vmixv(sun_direct, moon_direct, mk3(sun_vis * 1.0f, sun_vis * 1.0f, sun_vis * 1.0f));
                direct = muls(direct, (!(emissivity > 0.05f)) ? 1.0f : 0.0f);
                direct = vmax(direct, 0.000001f);
                v3 diffuse_indirect = mul(indirect, albedo);
                v3 I = normalize(sub(wp, viewer));
                float idn = dot(nh, I);
                v3 R = sub(I, muls(nh, 2.0f * idn));
                // SpecularIndirect (:901-909): the upscaled reflection times
                // clamp(max(n.n, 1e-8)^2 * 1.5, 0.1, 1) inside the 0.0035 border
                v3 spec_ind = mk3(0, 0, 0);
                const float sb = 0.0035f;
                if (spec && uv.x > sb && uv.x < 1.0f - sb && uv.y > sb && uv.y < 1.0f - sb) {
                    const float att = clampf(dm_pow(fmaxg(dot(n, nh), 0.00000001f), 2.0f) * 1.5f, 0.1f, 1.0f);
                    spec_ind = muls(mk3(up.spec[0], up.spec[1], up.spec[2]), att);
                }
                spec_ind = vmax(spec_ind, 0.0001f);
                v3 Lo = normalize(sub(viewer, wp));
                v3 F0 = vmix(mk3(0.04f, 0.04f, 0.04f), albedo, metal);
                diffuse_indirect = muls(diffuse_indirect, clampf(sampled_ao, 0.2f, 1.01f));
                float nov = clampf(dot(nh, Lo), 0.0000000001f, 1.0f);
                // ComputeSpecularAO (:742-745) of the texture AO (1 for flat materials)
                float spec_ao = clampf(dm_pow(nov + tex_ao, dm_exp2(-16.0f * rough - 1.0f)) - 1.0f + tex_ao, 0.0f, 1.0f);
                spec_ao = dm_pow(spec_ao, 1.5f);
                float horizon = fming(1.0f + dot(R, nh), 1.0f);
                horizon = (horizon * horizon) * horizon;
                if (metal >= 0.1f) spec_ind = muls(spec_ind, 1.3f);
                spec_ind = muls(spec_ind, spec_ao);
                spec_ind = muls(spec_ind, horizon);
                v3 F = vclamp(fresnel_schlick_roughness(Lo, nh, F0, rough), 0.0f, 1.0f);
                v3 kD = sub(mk3(1, 1, 1), F);
                kD = muls(kD, 1.0f - metal);
                float ex = clampf(fmaxg(dot(neg(I), nh), 0.000001f), 0.0f, 1.0f);
                float ey = clampf(rough, 0.0f, 1.0f);
                v2 env = karis_env_brdf(ex, ey);
                v3 ind_spec = mul(spec_ind, mk3(F.x * env.x + env.y, F.y * env.x + env.y, F.z * env.x + env.y));
                v3 indirect_light = add(mul(kD, diffuse_indirect), ind_spec);
                color = add(direct, indirect_light);
            } else {
                color = sky_radiance(dir);
            }
            color = vmax(color, 0.000001f);
            rgb[px * 3 + 0] = storage(color.x, fp16);
            rgb[px * 3 + 1] = storage(color.y, fp16);
            rgb[px * 3 + 2] = storage(color.z, fp16);
        }
    }
}

void vpto_shade(const vpto_world* w, const vpto_camera* cam, const vpto_params* p,
                const vpto_frame* f, const float* t, const uint8_t* face, const uint8_t* block,
                const uint8_t* shadow, const float* sh, const float* cocg, const float* aosky,
                const float* spec, int row0, int row1, float* rgb) {
    shade_impl(w, cam, p, f, t, face, block, shadow, sh, cocg, aosky, spec, row0, row1, rgb, nullptr, nullptr, nullptr,
               nullptr);
}

void vpto_shade_textured(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                         const float* t, const uint8_t* face, const uint8_t* block, const uint8_t* shadow,
                         const float* sh, const float* cocg, const float* aosky, const float* spec, int row0, int row1,
                         float* rgb, const float* gb_albedo, const float* gb_normal, const float* gb_pbr,
                         const float* gb_ao) {
    shade_impl(w, cam, p, f, t, face, block, shadow, sh, cocg, aosky, spec, row0, row1, rgb, gb_albedo, gb_normal,
               gb_pbr, gb_ao);
}

// ------------------------------------------------------------ reflections --
// SHToIrradianceA (ReflectionTraceFrag.glsl:466-476): the stored irradiance
// of an SH texel, independent of direction.
inline v3 sh_to_irradiance_a(const float* sh, const float* cocg_in) {
    const float Y = fmaxg(0.0f, 3.544905f * sh[3]);
    const float k = (Y * 0.282095f) / (sh[3] + 1e-6f);
    const float co = cocg_in[0] * k, cg = cocg_in[1] * k;
    const float T = Y - cg * 0.5f;
    const float G = cg + T;
    const float B = T - co * 0.5f;
    const float R = B + co;
    return mk3(fmaxg(R, 0.0f), fmaxg(G, 0.0f), fmaxg(B, 0.0f));
}

// ImportanceSampleGGX (ReflectionTraceFrag.glsl:345-365)
inline v3 importance_sample_ggx(v3 N, float roughness, float xi_x, float xi_y) {
    const float alpha = roughness * roughness;
    const float alpha2 = alpha * alpha;
    const float phi = (2.0f * PI) * xi_x;
    const float cos_t = std::sqrt((1.0f - xi_y) / (1.0f + (alpha2 - 1.0f) * xi_y));
    const float sin_t = std::sqrt(1.0f - cos_t * cos_t);
    const v3 H = mk3(dm_cos(phi) * sin_t, dm_sin(phi) * sin_t, cos_t);
    const v3 up = std::fabs(N.z) < 0.999f ? mk3(0.0f, 0.0f, 1.0f) : mk3(1.0f, 0.0f, 0.0f);
    const v3 tangent = normalize(cross(up, N));
    const v3 bitangent = cross(N, tangent);
    const v3 s = mk3((tangent.x * H.x + bitangent.x * H.y) + N.x * H.z, (tangent.y * H.x + bitangent.y * H.y) + N.y * H.z,
                     (tangent.z * H.x + bitangent.z * H.y) + N.z * H.z);
    return normalize(s);
}

// GetReflectionDirection (ReflectionTraceFrag.glsl:621-646): of three GGX
// microfacet normals, the one closest to N; the random pairs come from the
// pixel's PCG stream instead of hash2 / blue noise.
inline v3 reflection_normal(v3 N, float R, uint32_t* rng) {
    R = fmaxg(R, 0.05f);
    float nearest = -100.0f;
    v3 best = N;
    for (int i = 0; i < 3; i++) {
        const float xi_x = rand01(rng) * 0.9f;
        const float xi_y = rand01(rng) * 0.65f;
        const v3 h = importance_sample_ggx(N, R, xi_x, xi_y);
        const float d = dot(h, N);
        if (d > nearest) {
            best = h;
            nearest = d;
        }
    }
    return best;
}

// GLSL reflect(I, N) = I - 2 * dot(N, I) * N
inline v3 reflect3(v3 I, v3 N) { return sub(I, muls(N, 2.0f * dot(N, I))); }

// CalculateDirectionalLight of the reflection trace (ReflectionTraceFrag.glsl:
// 313-336): its specular radiance is scaled by 0, so only the diffuse lobe
// remains; ndfGGX (:282-289), gaSchlickGGX (:300-305), fresnelSchlick (:307-310).
inline v3 reflection_directional_light(v3 viewer, v3 wp, v3 light_dir, v3 radiance, v3 albedo, v3 n, float rough,
                                       float metal, float shadow) {
    const float Epsilon = 0.00001f;
    const float sh = fming(shadow, 1.0f);
    const v3 Lo = normalize(sub(viewer, wp));
    const float cos_lo = fmaxg(0.0f, dot(n, Lo));
    const v3 F0 = vmix(mk3(0.04f, 0.04f, 0.04f), albedo, metal);
    const v3 Li = light_dir;
    const v3 Lh = normalize(add(Li, Lo));
    const float cos_li = fmaxg(0.0f, dot(n, Li));
    const float cos_lh = fmaxg(0.0f, dot(n, Lh));
    const float fk = dm_pow(1.0f - fmaxg(0.0f, dot(Lh, Lo)), 5.0f);
    const v3 F = add(F0, muls(sub(mk3(1.0f, 1.0f, 1.0f), F0), fk));
    const float alpha = rough * rough;
    const float alpha_sq = alpha * alpha;
    const float denom = (cos_lh * cos_lh) * (alpha_sq - 1.0f) + 1.0f;
    const float D = alpha_sq / ((PI * denom) * denom);
    const float r1 = rough + 1.0f;
    const float k = (r1 * r1) / 8.0f;
    const float G = (cos_li / (cos_li * (1.0f - k) + k)) * (cos_lo / (cos_lo * (1.0f - k) + k));
    const v3 kd = vmix(sub(mk3(1.0f, 1.0f, 1.0f), F), mk3(0.0f, 0.0f, 0.0f), metal);
    const v3 diffuse_brdf = mul(kd, albedo);
    const v3 spec_brdf = divs(muls(muls(F, D), G), fmaxg(Epsilon, (4.0f * cos_li) * cos_lo));
    const v3 radiance_s = muls(muls(radiance, 0.05f), 0.0f);
    const v3 result = add(muls(mul(diffuse_brdf, radiance), cos_li), muls(mul(spec_brdf, radiance_s), cos_li));
    return muls(vmax(result, 0.0f), clampf(1.0f - sh, 0.0f, 1.0f));
}

// The face UV of CalculateVectors (ReflectionTraceFrag.glsl:1388-1446) with
// the shader's UV.y = 1 - UV.y (:848).
// The textured G-buffer the reflection passes read with block textures
// (vpto_set_textured_gbuffer; off: the block table and the face normals):
// PBR nearest and the normal-mapped normal bilinear at uv, as GL samples them.
struct GbtState {
    const float* normal = nullptr;
    const float* pbr = nullptr;
    int W = 0, H = 0;
};
GbtState g_gbt;
inline float gbt_pbr(v2 uv, int c) {
    const Plane P{g_gbt.pbr, g_gbt.W, g_gbt.H, 4};
    return P.at(f2i(std::floor(uv.x * (float)g_gbt.W)), f2i(std::floor(uv.y * (float)g_gbt.H)), c);
}
inline v3 gbt_normal(v2 uv) {
    const Plane P{g_gbt.normal, g_gbt.W, g_gbt.H, 3};
    float n[3];
    P.linear(uv, n);
    return mk3(n[0], n[1], n[2]);
}
inline v3 gbt_normal_at(size_t px) {
    return mk3(g_gbt.normal[px * 3], g_gbt.normal[px * 3 + 1], g_gbt.normal[px * 3 + 2]);
}

// The block textures at a reflection hit (ReflectionTraceFrag.glsl :887-1007):
// albedo, PBR (level 0), the normal map at level 3 through the face's tangent
// basis and the emissive texel at level 2 (-1 without one); false without
// textures.
struct TexHit {
    v3 albedo, nmap;
    float rough, metal, ao, emis;
};
bool tex_reflection_hit(int rid, v3 hp, v3 hn, TexHit* out);

inline v2 face_uv(v3 p, v3 n) {
    v2 uv;
    if (n.z != 0.0f) uv = v2{fract(p.x), fract(p.y)};
    else if (n.y != 0.0f) uv = v2{fract(p.x), fract(p.z)};
    else uv = v2{fract(p.z), fract(p.y)};
    uv.y = 1.0f - uv.y;
    return uv;
}

struct ReflectionInputs {
    Plane T;             // full-resolution depth (GetPositionAt at the reprojected point)
    Plane8 F;            // full-resolution face ids
    Plane8 S;            // full-resolution sun shadow (R8, bilinear)
    Plane TV;            // the depth on the reflection (GI) grid
    Plane8 FV, BV;       // face and block ids on that grid
    Plane SH, CC, AO;    // denoised diffuse GI on that grid (DiffuseDenoiseFBO 0, 1, 3)
};

// ReflectionTraceFrag.glsl main (:717-1084) for one texel of the reflection
// grid, with u_RoughReflections on, u_ReprojectToScreenSpace on, LPV and cloud
// reflections off, no player and flat materials (albedo, roughness,
// metalness, emissive flag of the block; AO 1; the face normal as the
// normal map); PCG random numbers; no jitter.
void reflection_texel(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                      const float* view_proj, const ReflectionInputs& in, int i, int j, int Wg, int Hg, size_t q,
                      float* spec4, float* hit, float* mask, RowCount* cnt) {
    const v2 uv = texcoord(i, j, Wg, Hg);
    v4 P = position_fetch(cam, in.TV, i, j, uv);
    if (P.w < 0.0f) {
        for (int c = 0; c < 4; c++) spec4[c] = 0.0f;
        *hit = -1.0f;
        *mask = 0.0f;
        return;
    }
    const v3 viewer = mk3(cam->position[0], cam->position[1], cam->position[2]);
    const v3 cam_pos = ray_origin(cam);
    const v3 N = normal_from_id(in.FV.at(i, j), 1.0f);
    // NormalMappedInitial (:794): the linear normal G-buffer at the texel
    // centre, the face normal itself on the G-buffer's grid
    v3 NM = gi_div(p) == 1 ? N : gnormal_linear(in.F, uv);
    const Material base = material(w, std::min(std::max(in.BV.at(i, j), 0), 127));
    float base_rough = base.rough, base_metal = base.metal;
    if (g_gbt.normal) {
        base_rough = gbt_pbr(uv, 0);
        base_metal = gbt_pbr(uv, 1);
        NM = gi_div(p) == 1 ? gbt_normal_at(q) : gbt_normal(uv);
    }
    const v3 I = normalize(sub(mk3(P.x, P.y, P.z), viewer));
    P.x += N.x * 0.035f;
    P.y += N.y * 0.035f;
    P.z += N.z * 0.035f;
    const v3 pos = mk3(P.x, P.y, P.z);
    float dsh[4], dcc[2];
    for (int c = 0; c < 4; c++) dsh[c] = in.SH.at(i, j, c);
    for (int c = 0; c < 2; c++) dcc[c] = in.CC.at(i, j, c);
    const v3 base_indirect = sh_to_irradiance_a(dsh, dcc);
    const Lighting L = frame_lighting(f);
    const v3 sun_color = mk3(f->sun_radiance[0], f->sun_radiance[1], f->sun_radiance[2]);
    const v3 moon_color = mk3(f->moon_radiance[0], f->moon_radiance[1], f->moon_radiance[2]);
    const float sun_vis = 1.0f - L.sun_visibility;
    const v3 mixed = vmix(sun_color, moon_color, sun_vis);   // SAMPLED_COLOR_MIXED (:727-730)
    uint32_t rng = pcg_hash(pixel_seed(f, (uint32_t)q) ^ 0x5245464Cu);
    const int spp = std::min(std::max(p->reflection_spp, 1), 16);
    const float rbias = 0.85f;   // u_RoughnessBias (ReflectionRoughnessBias && DenoiseReflections)
    float total[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float avg_hit = 0.001f, meaningful = 0.0f, emask = 0.0f, computed_shadow = 0.0f;
    int shadow_itr = 0, total_hits = 0;
    for (int s = 0; s < spp; s++) {
        const v3 rn = reflection_normal(NM, clampf(base_rough * rbias, 0.01f, 1.0f), &rng);
        const v3 R = reflect3(I, rn);
        const TraceResult tr = traverse(w, pos, R, p->reflection_max_steps);
        cnt->add(4, tr.steps);
        const float T = tr.t;
        const v3 hp = add(pos, muls(R, T));
        v3 computed;
        if (T > 0.0f) {
            const v3 hn = tr.normal;
            const int rid = std::min(std::max(tr.block, 0), 127);
            // ReprojectReflectionToScreenSpace (:582-594)
            const v4 pr = mat_mul4(view_proj, hp.x, hp.y, hp.z, 1.0f);
            const v2 rc = v2{(pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f};
            const v4 pa = position_linear(cam, in.T, rc);
            const v3 na = normal_from_id(in.F.nearest(rc), 1.0f);
            const v3 pd = mk3(std::fabs(pa.x - hp.x), std::fabs(pa.y - hp.y), std::fabs(pa.z - hp.z));
            const float err = dot(pd, pd);
            const float tb = 0.032593f;   // InThresholdedScreenSpace (:217-221)
            const bool in_ss = rc.x > tb && rc.x < 1.0f - tb && rc.y > tb && rc.y < 1.0f - tb;
            const bool success = err < 0.095f && na.x == hn.x && na.y == hn.y && na.z == hn.z && in_ss;
            v3 ambient = base_indirect;
            if (success) {
                float rsh[4], rcc[2], rao[2];
                in.SH.linear(rc, rsh);
                in.CC.linear(rc, rcc);
                in.AO.linear(rc, rao);
                ambient = sh_to_irradiance_a(rsh, rcc);
                const float vxao = dm_pow(rao[0], 0.75f);
                if (pa.w > 0.0f && length(sub(mk3(pa.x, pa.y, pa.z), cam_pos)) < 40.0f) ambient = muls(ambient, vxao);
            }
            Material m = material(w, rid);
            const v3 radiance = muls(mixed, 0.6f);
            float ao = dm_pow(1.0f, 2.0f);
            v3 nmap = hn;
            TexHit th;
            const bool textured = tex_reflection_hit(rid, hp, hn, &th);
            if (textured) {
                m.albedo = th.albedo;
                m.rough = th.rough;
                m.metal = th.metal;
                ao = th.ao;
                nmap = th.nmap;
            }
            if (shadow_itr < std::max(spp / 4, 1)) {   // (:929-953)
                if (success && in_ss) {
                    computed_shadow = in.S.linearf(rc);
                } else {
                    const TraceResult sr = traverse(w, add(hp, muls(hn, 0.055f)), L.light_dir,
                                                    p->reflection_shadow_max_steps);
                    cnt->add(5, sr.steps);
                    computed_shadow = sr.t > 0.0f ? 1.0f : 0.0f;
                }
                shadow_itr++;
            }
            ambient = mul(muls(muls(ambient, 1.0f), clampf(ao, 0.1f, 1.0f)), m.albedo);
            v3 direct = add(ambient, reflection_directional_light(viewer, hp, L.light_dir, radiance, m.albedo, nmap,
                                                                  m.rough, m.metal, computed_shadow));
            // (:988-1007), Emissivity = 1 for a flat emissive block
            if (textured ? th.emis > 0.1f : m.emissive != 0) {
                float emissivity = textured ? th.emis : 1.0f;
                const v2 fuv = face_uv(hp, hn);
                const float bx = 0.02501f, by = 0.03001f;
                emissivity *= (fuv.x > bx && fuv.x < 1.0f - bx && fuv.y > by && fuv.y < 1.0f - by) ? 1.0f : 0.0f;
                direct = muls(m.albedo, fmaxg(emissivity * 19.0f * 1.0f, 2.0f));
                emask = 1.0f;
            }
            computed = direct;
            avg_hit += T;
            meaningful += 1.0f;
        } else {
            computed = muls(sky_radiance(normalize(R)), mixf(1.0f, 1.175f, base_metal > 0.05f ? 1.0f : 0.0f));
        }
        total[0] += computed.x;
        total[1] += computed.y;
        total[2] += computed.z;
        total[3] += 1.0f;
        total_hits++;
    }
    avg_hit /= fmaxg(meaningful, 0.01f);
    for (int c = 0; c < 4; c++) spec4[c] = clampf(total[c] / (float)total_hits, 0.0000001f, 100.0f);
    *hit = clampf(meaningful > 0.01f ? avg_hit : -1.0f, -10.0f, 200.0f);
    *mask = clampf(emask, 0.0f, 1.0f);
}

void vpto_trace_reflection(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                           const float* t, const uint8_t* face, const uint8_t* shadow, const float* t_view,
                           const uint8_t* face_view, const uint8_t* block_view, const float* den_sh,
                           const float* den_cocg, const float* den_aosky, int row0, int row1, float* spec,
                           float* hit, float* mask) {
    const int W = p->width, H = p->height, Wg = W / gi_div(p), Hg = H / gi_div(p);
    const int fp16 = p->storage;
    const ReflectionInputs in{Plane{t, W, H, 1},          Plane8{face, W, H},        Plane8{shadow, W, H},
                              Plane{t_view, Wg, Hg, 1},   Plane8{face_view, Wg, Hg}, Plane8{block_view, Wg, Hg},
                              Plane{den_sh, Wg, Hg, 4},   Plane{den_cocg, Wg, Hg, 2}, Plane{den_aosky, Wg, Hg, 2}};
    // u_Projection * u_View, evaluated left to right
    float m[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            m[c * 4 + r] = ((cam->proj[0 * 4 + r] * cam->view[c * 4 + 0] + cam->proj[1 * 4 + r] * cam->view[c * 4 + 1]) +
                            cam->proj[2 * 4 + r] * cam->view[c * 4 + 2]) +
                           cam->proj[3 * 4 + r] * cam->view[c * 4 + 3];
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = row0; j < row1; j++) {
        RowCount cnt;
        for (int i = 0; i < Wg; i++) {
            const size_t q = (size_t)j * Wg + i;
            float s4[4], h, mk;
            reflection_texel(w, cam, p, f, m, in, i, j, Wg, Hg, q, s4, &h, &mk, &cnt);
            for (int c = 0; c < 4; c++) spec[q * 4 + c] = storage(s4[c], fp16);
            hit[q] = storage(h, fp16);
            mask[q] = storage(mk, fp16);
        }
        cnt.flush();
    }
}

// BlurHitDistance_Bilateral.glsl (pass 1: 3x3) and
// BlurHitDistancePass2_Bilateral.glsl (pass 2: 3 x 5 taps, y in -2..2), both
// two GI texels apart (Scale 2), run on the reflection hit distance before the
// temporal filter (DENOISE_REFLECTION_HIT_DATA, Core/Pipeline.cpp:126,
// :3141-3215). Taps with a depth difference above 1, a miss, or another face
// are skipped; REPEAT wrap. The depth and face are the GI-grid views.
void vpto_spec_hit_blur(const vpto_params* p, int pass, const float* t_view, const uint8_t* face_view,
                        const float* hit_in, float* hit_out) {
    const int Wg = p->width / gi_div(p), Hg = p->height / gi_div(p);
    const Plane TV{t_view, Wg, Hg, 1}, HI{hit_in, Wg, Hg, 1};
    const Plane8 FV{face_view, Wg, Hg};
    static const float kw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    const int ry = pass == 2 ? 2 : 1;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Hg; j++) {
        for (int i = 0; i < Wg; i++) {
            const float bd = TV.at(i, j, 0), bh = HI.at(i, j, 0);
            const int bf = FV.at(i, j);
            float tw = 1.0f, td = bh;
            for (int x = -1; x <= 1; x++) {
                for (int y = -ry; y <= ry; y++) {
                    if (x == 0 && y == 0) continue;
                    const int si = i + 2 * x, sj = j + 2 * y;
                    const float e = std::fabs(TV.at(si, sj, 0) - bd);
                    const float ha = HI.at(si, sj, 0);
                    if (e > 1.0f || ha < 0.0f || FV.at(si, sj) != bf) continue;
                    const float wgt = kw[std::abs(x)] * kw[std::abs(y)];
                    td += ha * wgt;
                    tw += wgt;
                }
            }
            hit_out[(size_t)j * Wg + i] = storage(td / fmaxg(tw, 0.001f), p->storage);
        }
    }
}

// ClipToAABB (SpecularTemporalFilter.glsl:146-156)
inline v3 clip_to_aabb(v3 prev, v3 mn, v3 mx) {
    const v3 pc = muls(add(mx, mn), 0.5f);
    const v3 ec = muls(sub(mx, mn), 0.5f);
    const v3 vc = sub(prev, pc);
    const v3 vu = mk3(vc.x / ec.x, vc.y / ec.y, vc.z / ec.z);
    const v3 au = mk3(std::fabs(vu.x), std::fabs(vu.y), std::fabs(vu.z));
    const float denom = fmaxg(au.x, fmaxg(au.y, au.z));
    return denom > 1.0f ? add(pc, divs(vc, denom)) : prev;
}

inline float dist_sq(v3 a, v3 b) {
    const v3 c = sub(a, b);
    return dot(c, c);
}

// SpecularTemporalFilter.glsl main (:316-510) with USE_NEW_REPROJECTION,
// u_SmartClip, u_RoughnessWeight, u_TemporallyStabializeHitDistance,
// u_FireflyRejection and u_AggressiveFireflyRejection on
// (Core/Pipeline.cpp:3226-3262). TEMPORAL_SPEC is p->reflection_temporal;
// off, the output is the firefly-rejected current colour.
void vpto_spec_temporal(const vpto_world* w, const vpto_camera* cam, const vpto_camera* prev_cam,
                        const vpto_params* p, const float* t_view, const uint8_t* face_view,
                        const uint8_t* block_view, const float* prev_t, const uint8_t* prev_face,
                        const float* spec, const float* hit, const float* mask, const float* prev_out,
                        const float* prev_hit, const float* prev_stable, float* out, float* acc, float* stable) {
    const int W = p->width, H = p->height, Wg = W / gi_div(p), Hg = H / gi_div(p);
    const int fp16 = p->storage;
    const bool temporal = p->reflection_temporal != 0;
    const Plane TV{t_view, Wg, Hg, 1}, C{spec, Wg, Hg, 4}, M{mask, Wg, Hg, 1}, PC{prev_out, Wg, Hg, 4};
    const Plane PH{prev_hit, Wg, Hg, 1}, PS{prev_stable, Wg, Hg, 1}, PT{prev_t, W, H, 1};
    const Plane8 FV{face_view, Wg, Hg}, BV{block_view, Wg, Hg}, PF{prev_face, W, H};
    float m[16];   // u_PrevProjection * u_PrevView, left to right
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            m[c * 4 + r] = ((prev_cam->proj[0 * 4 + r] * prev_cam->view[c * 4 + 0] +
                             prev_cam->proj[1 * 4 + r] * prev_cam->view[c * 4 + 1]) +
                            prev_cam->proj[2 * 4 + r] * prev_cam->view[c * 4 + 2]) +
                           prev_cam->proj[3 * 4 + r] * prev_cam->view[c * 4 + 3];
    const v3 cur_pos = mk3(cam->position[0], cam->position[1], cam->position[2]);
    const v3 prev_pos = mk3(prev_cam->position[0], prev_cam->position[1], prev_cam->position[2]);
    const v3 ro = ray_origin(cam);
    const int ox[4] = {1, 0, -1, 0}, oy[4] = {0, 1, 0, -1};
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < Hg; j++) {
        for (int i = 0; i < Wg; i++) {
            const size_t q = (size_t)j * Wg + i;
            const v2 uv = texcoord(i, j, Wg, Hg);
            const v4 P = position_fetch(cam, TV, i, j, uv);
            const v3 n0 = normal_from_id(FV.at(i, j), 1.0f);
            float cc[4];
            for (int c = 0; c < 4; c++) cc[c] = C.at(i, j, c);
            float o_acc = 0.0f;
            const float hc = hit[q];
            float o_col[4], o_stable;
            // firefly rejection (:330-337, FireflyReject :267-305)
            if (mask[q] > 0.05f) {
                float a4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                int unlit = 0;
                for (int k = 0; k < 4; k++) {
                    if (M.at(i + ox[k], j + oy[k], 0) < 0.01f) {
                        for (int c = 0; c < 4; c++) a4[c] += C.at(i + ox[k], j + oy[k], c);
                        unlit++;
                    }
                }
                if (unlit >= 3)
                    for (int c = 0; c < 4; c++) cc[c] = a4[c] / (float)unlit;
            }
            if (P.w > 0.0f && temporal) {
                const bool sky = hc < 0.0f;
                const Material mt = material(w, std::min(std::max(BV.at(i, j), 0), 127));
                const float pr = g_gbt.pbr ? gbt_pbr(uv, 0) : mt.rough;
                const float rough = mixf(0.095f, pr, 1.0f), metal = g_gbt.pbr ? gbt_pbr(uv, 1) : mt.metal;
                bool less_valid = false;
                v2 rep = v2{0.0f, 0.0f};
                if (hc > 0.0f && !sky && rough <= 0.875f + 0.01f) {
                    const v3 I = normalize(sub(ro, mk3(P.x, P.y, P.z)));
                    const v3 rp = sub(mk3(P.x, P.y, P.z), muls(I, hc));
                    const v4 pr = mat_mul4(m, rp.x, rp.y, rp.z, 1.0f);
                    rep = v2{(pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f};
                    float pt;
                    PH.linear(rep, &pt);
                    if (std::fabs(pt - hc) >= 3.8f) less_valid = true;
                } else if (!sky) {
                    const v3 off = muls(sub(cur_pos, prev_pos), 0.6f);
                    const v3 wp = sub(mk3(P.x, P.y, P.z), off);
                    const v4 pr = mat_mul4(m, wp.x, wp.y, wp.z, 1.0f);
                    rep = v2{(pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f};
                }
                if (sky) {
                    const v3 I = normalize(sub(ro, mk3(P.x, P.y, P.z)));
                    const v3 rp = sub(mk3(P.x, P.y, P.z), muls(I, 64.0f));
                    const v4 pr = mat_mul4(m, rp.x, rp.y, rp.z, 1.0f);
                    rep = v2{(pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f};
                }
                const v4 pp = position_linear(cam, PT, rep);
                const float d = std::fabs(length(sub(mk3(pp.x, pp.y, pp.z), mk3(P.x, P.y, P.z))));
                const float rb = 0.01f;
                const v3 pn = normal_from_id(PF.nearest(rep), 1.0f);
                if (rep.x > 0.0f + rb && rep.x < 1.0f - rb && rep.y > 0.0f + rb && rep.y < 1.0f - rb && d < 1.0f &&
                    pn.x == n0.x && pn.y == n0.y && pn.z == n0.z) {
                    float pc[4];
                    PC.linear(rep, pc);
                    const v3 base_prev = mk3(pc[0], pc[1], pc[2]);
                    const bool moved = dist_sq(cur_pos, prev_pos) > 0.0001f;
                    if (rough < 0.5f + 0.01f && moved) {
                        // ReflectionClipping (:163-243) around this texel
                        float mn[4] = {1000.0f, 1000.0f, 1000.0f, 1000.0f}, mx[4] = {-1000.0f, -1000.0f, -1000.0f, -1000.0f};
                        const float texel_x = 1.0f / (float)Wg, texel_y = 1.0f / (float)Hg;
                        (void)texel_x;
                        (void)texel_y;
                        float add_max = 0.0f;
                        for (int x = -1; x <= 1; x++) {
                            for (int y = -1; y <= 1; y++) {
                                if (!(M.at(i + x, j + y, 0) < 0.01f)) add_max += 0.1f;
                                for (int c = 0; c < 4; c++) {
                                    const float sv = C.at(i + x, j + y, c);
                                    mn[c] = fming(sv, mn[c]);
                                    mx[c] = fmaxg(sv, mx[c]);
                                }
                            }
                        }
                        const v3 omn = mk3(mn[0], mn[1], mn[2]), omx = mk3(mx[0], mx[1], mx[2]);
                        const float rt = 0.275f + 0.01f;
                        const bool smoothish = rough < rt;
                        const bool roughish = rough > rt && rough < 0.50f + 0.01f;
                        if (smoothish) {
                            const float pr2 = rough * rough;
                            const float rt2 = rt * rt;
                            const float rr = 0.0f + (clampf((pr2 - 0.0f) / (rt2 - 0.0f), 0.0f, 1.0f) * (1.0f - 0.0f));
                            float bias = mixf(0.01f, 0.085f, rr);
                            if (rough > 0.235f) bias *= 1.55f;
                            for (int c = 0; c < 4; c++) {
                                mn[c] -= bias * 0.95f;
                                mx[c] += (bias * 0.95f) + add_max;
                            }
                        } else if (roughish) {
                            for (int c = 0; c < 4; c++) {
                                mn[c] -= 0.37f;
                                mx[c] += 0.37f + (add_max * 1.1f);
                            }
                        }
                        const float imp = mixf(0.05f, 0.25f, metal > 0.05f ? 1.0f : 0.0f);
                        v3 mn3 = vmix(mk3(mn[0], mn[1], mn[2]), omn, imp);
                        v3 mx3 = vmix(mk3(mx[0], mx[1], mx[2]), omx, imp);
                        const float bm = less_valid ? 0.5f : 0.0f;
                        mn3 = vmix(mn3, omn, bm);
                        mx3 = vmix(mx3, omx, bm);
                        mn[0] = mn3.x; mn[1] = mn3.y; mn[2] = mn3.z;
                        mx[0] = mx3.x; mx[1] = mx3.y; mx[2] = mx3.z;
                        const v3 prev3 = mk3(pc[0], pc[1], pc[2]);
                        const v3 cl = clip_to_aabb(prev3, mn3, mx3);
                        if (!(cl.x == prev3.x && cl.y == prev3.y && cl.z == prev3.z)) {
                            if (dist_sq(cl, mn3) > dist_sq(cl, mx3))
                                for (int c = 0; c < 4; c++) pc[c] = mx[c];
                            else
                                for (int c = 0; c < 4; c++) pc[c] = mn[c];
                        }
                    }
                    // GetAccumulationFactor (:308-313)
                    const float vx = (uv.x - rep.x) * (float)Wg, vy = (uv.y - rep.y) * (float)Hg;
                    float af = clampf(dm_exp(-std::sqrt(vx * vx + vy * vy)) * 0.9f + 0.750f, 0.00000001f, 0.96f);
                    af = clampf(af, 0.001f, 0.95f);
                    for (int c = 0; c < 4; c++) {
                        const float cv = fmaxg(cc[c], 0.0f), pv = fmaxg(pc[c], 0.0f);
                        o_col[c] = mixf(cv, pv, af);
                    }
                    o_acc = af;
                    o_stable = hc;
                    if (dist_sq(base_prev, mk3(fmaxg(pc[0], 0.0f), fmaxg(pc[1], 0.0f), fmaxg(pc[2], 0.0f))) < 0.2f) {
                        float ps;
                        PS.linear(rep, &ps);
                        o_stable = mixf(hc, ps, clampf(af * 1.1f, 0.0f, 0.9f));
                    }
                } else {
                    for (int c = 0; c < 4; c++) o_col[c] = cc[c];
                    o_acc = 0.0f;
                    o_stable = hc;
                }
            } else {
                for (int c = 0; c < 4; c++) o_col[c] = cc[c];
                o_stable = hc;
            }
            if (!temporal) o_acc = -1.0f;
            for (int c = 0; c < 4; c++) out[q * 4 + c] = storage(o_col[c], fp16);
            acc[q] = storage(o_acc, fp16);
            stable[q] = storage(o_stable, fp16);
        }
    }
}

// ReflectionDenoiserNew.glsl main (:140-473), one separable pass (dir 1: x,
// 0: y) of the 33-tap Gaussian with depth, normal, luminance, normal-map and
// roughness weights, u_RoughnessBias, u_NormalMapAware, u_HandleLobeDeviation
// and u_AmplifyReflectionTransversalWeight on, u_DeriveFromDiffuseSH off,
// NormalMapWeightStrength 0.75, RoughnessNormalWeightBiasStrength 1.075,
// radius bias 0, scale 1 (Core/Pipeline.cpp:3314-3440); u_ResolutionScale
// (ReflectionSuperSampleResolution) = 1 / gi_divisor and u_TemporalWeight =
// TEMPORAL_SPEC. The jitter int((noise - 0.5) * 0.75) is 0 for every noise in
// [0, 1). Taps at fractional offsets sample the full-resolution depth, face,
// block and normal planes; the centre reads the GI-grid views.
void vpto_spec_denoise(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, int dir, const float* t,
                       const uint8_t* face, const uint8_t* block, const float* t_view, const uint8_t* face_view,
                       const uint8_t* block_view, const float* in, const float* hit_data, const float* frames,
                       float* out) {
    static const float gauss[33] = {0.004013f, 0.005554f, 0.007527f, 0.00999f,  0.012984f, 0.016524f, 0.020594f,
                                    0.025133f, 0.030036f, 0.035151f, 0.040283f, 0.045207f, 0.049681f, 0.053463f,
                                    0.056341f, 0.058141f, 0.058754f, 0.058141f, 0.056341f, 0.053463f, 0.049681f,
                                    0.045207f, 0.040283f, 0.035151f, 0.030036f, 0.025133f, 0.020594f, 0.016524f,
                                    0.012984f, 0.00999f,  0.007527f, 0.005554f, 0.004013f};
    const int d = gi_div(p), W = p->width, H = p->height, Wg = W / d, Hg = H / d;
    const int fp16 = p->storage;
    const bool temporal_weight = p->reflection_temporal != 0;
    const Plane T{t, W, H, 1}, TV{t_view, Wg, Hg, 1}, IN{in, Wg, Hg, 4};
    const Plane8 F{face, W, H}, B{block, W, H}, FV{face_view, Wg, Hg}, BV{block_view, Wg, Hg};
    const float texel = dir ? 1.0f / (float)Wg : 1.0f / (float)Hg;
    const float res_scale = 1.0f / (float)d;
    const float EPS = 0.001f;
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < Hg; j++) {
        for (int i = 0; i < Wg; i++) {
            const size_t q = (size_t)j * Wg + i;
            const v2 uv = texcoord(i, j, Wg, Hg);
            const v4 bp = position_fetch(cam, TV, i, j, uv);
            const v3 bn = normal_from_id(FV.at(i, j), 1.0f);
            const bool base_sky = bp.w < 0.0f;
            float bc[4];
            for (int c = 0; c < 4; c++) bc[c] = IN.at(i, j, c);
            const float base_lum = dot(mk3(bc[0], bc[1], bc[2]), mk3(0.299f, 0.587f, 0.114f));
            const int bblock = BV.at(i, j);
            const bool gbt = g_gbt.pbr != nullptr;
            const float pbr_x = gbt ? gbt_pbr(uv, 0) : pbr_rough(w, bblock);
            const float pbr_y = gbt ? gbt_pbr(uv, 1) : pbr_metal(w, bblock);
            float br = pbr_x + 0.001f;
            const float raw_rough = br;
            br *= mixf(1.0f, 0.91f, 1.0f);
            const v3 nm_base = gbt ? (d == 1 ? gbt_normal_at(q) : gbt_normal(uv)) : (d == 1 ? bn : gnormal_linear(F, uv));
            float hd = hit_data[q] + 0.0001f;
            if (hd < 0.001f) hd = 1.75f;
            else hd = dm_pow(hd, 1.0f / 1.3f);
            if (br <= 0.25f + 0.05f) hd = clampf(hd, 0.0f, 8.0f);
            if (br <= 0.2f) hd = clampf(hd, 0.0f, 5.5f);
            const float shd = fmaxg(hd, 0.01f) * (raw_rough < 0.51f ? 0.5f : 0.85f);
            const v4 vs = mat_mul4(cam->view, bp.x, bp.y, bp.z, 1.0f);
            const float vlen = length(mk3(vs.x, vs.y, vs.z));
            float vlw = 0.001f + vlen;
            if (br > 0.135f) vlw = fmaxg(vlw, 0.750f);
            else vlw = fmaxg(vlw, 3.0f);
            if (br < 0.125f) vlw = clampf(vlw, 0.000001f, 6.0f);
            else if (br < 0.25f) vlw = clampf(vlw, 0.000001f, 8.0f + 1.0f);
            else if (br < 0.5f) vlw = clampf(vlw, 0.000001f, 16.0f);
            else if (br < 0.75f) vlw = clampf(vlw, 0.000001f, 24.0f);
            else vlw = clampf(vlw, 0.000001f, 32.0f);
            float tc = shd / fmaxg(shd + vlw, 0.00001f);
            if (raw_rough < 0.535f && bp.w < 50.0f) {
                const float rr = (((raw_rough - 0.0f) / (0.535f - 0.0f)) * (1.0f - 0.0f)) + 0.0f;
                const float te = mixf(3.5f, 2.0f, dm_pow(rr, 4.0f));
                tc = dm_pow(tc, te + 0.8125f);
            }
            const float rad_e = dm_pow(1.0f - br, 1.0f / 1.4f) * 5.0f;
            const float radius = clampf(dm_pow(mixf(1.0f * br, 1.0f, tc), rad_e), 0.0f, 1.0f);
            const float nm_radius = 1.0f - clampf(dm_pow(mixf(1.0f * br, 1.0f, tc), rad_e), 0.0f, 1.0f);
            int er = f2i(std::floor(radius * 15.0f));
            er = std::min(std::max(er, 1), 15);
            if (br > 0.897511f) er = 15;
            const int jitter = 0;
            float scale = mixf(1.0f, 2.0f, clampf(res_scale, 0.0000001f, 1.0f)) + 0.5f;
            int rbias = 0;
            if (pbr_y > 0.1f - EPS && br > 0.4f - EPS) rbias += 2;
            er = std::min(std::max(er + rbias + 0, 1), 15);
            if (raw_rough >= 0.5f - 0.01f) er += 1;
            scale *= 1.0f;
            float tw_t = 0.0f, afc = 0.01f;
            if (temporal_weight) {
                const float af = frames[q];
                afc = af < -0.1f ? 0.0f : (1.0f - af);
                afc = clampf(afc, 0.000001f, 1.0f);
                tw_t = clampf(afc * 0.85f, 0.0f, 1.0f);
                float flt = (float)er;
                flt = mixf(flt, flt + 2.0f, afc * 1.05f);
                er = f2i(flt);
            }
            float hf_e = (64.0f * 0.750f) * 1.350f;
            hf_e *= dm_pow(nm_radius, 1.0f / 1.33f);
            float hf_add = mixf(0.0f, 0.005f, br > 0.45f ? 1.0f : 0.0f);
            hf_add += mixf(0.0f, 0.0125f, br > 0.525f ? 1.0f : 0.0f);
            hf_add += mixf(0.0f, 0.022f, br > 0.625f ? 1.0f : 0.0f);
            hf_add += mixf(0.0f, 0.026f, br > 0.725f ? 1.0f : 0.0f);
            hf_add += mixf(0.0f, 0.031f, br > 0.75f ? 1.0f : 0.0f);
            er = std::min(std::max(er, 1), 15);
            float fc[4] = {0.0f, 0.0f, 0.0f, 0.0f}, tw = 0.0f;
            for (int s = -er; s <= er; s++) {
                const float so = (float)s;
                v2 sc = dir ? v2{uv.x + ((so * scale) * texel), uv.y} : v2{uv.x, uv.y + ((so * scale) * texel)};
                sc.x += ((float)jitter * texel) * 0.75f;
                sc.y += ((float)jitter * texel) * 0.75f;
                const float bias = 0.01f;
                if (!(sc.x > 0.0f + bias && sc.x < 1.0f - bias && sc.y > 0.0f + bias && sc.y < 1.0f - bias)) continue;
                // the centre tap is the texel itself; the others fall between texels
                float sdepth, sd[4];
                int sface, sblock;
                v3 nm_at;
                if (s == 0) {
                    sdepth = TV.at(i, j, 0);
                    sface = FV.at(i, j);
                    sblock = bblock;
                    for (int c = 0; c < 4; c++) sd[c] = bc[c];
                    nm_at = nm_base;
                } else {
                    T.linear(sc, &sdepth);
                    sface = F.nearest(sc);
                    sblock = B.nearest(sc);
                    IN.linear(sc, sd);
                    nm_at = gbt ? gbt_normal(sc) : gnormal_linear(F, sc);
                }
                const bool sample_sky = sdepth < 0.0f;
                if (sample_sky != base_sky) continue;
                const float dd = std::fabs(sdepth - bp.w) * 1.5f;
                const float dw = dm_pow(dm_exp(-dd), 2.0f);
                const v3 sn = normal_from_id(sface, 1.0f);
                const float nw = dm_pow(fmaxg(dot(bn, sn), 0.00000000001f), 32.0f);
                float lw = 1.0f;
                const float srough = gbt ? (s == 0 ? pbr_x : gbt_pbr(sc, 0)) : pbr_rough(w, sblock);
                const bool too_rough = srough >= 0.89f;
                if (!too_rough) {
                    const float luma = dot(mk3(sd[0], sd[1], sd[2]), mk3(0.299f, 0.587f, 0.114f));
                    float le = 1.0f / std::fabs(luma - base_lum);
                    le = dm_pow(le, 1.7f);
                    const float lwe = mixf(0.001f, 8.0f, dm_pow(srough, 16.0f));
                    lw = dm_pow(le, lwe + 0.8f);
                    lw = clampf(lw, 0.0000000001f, 1.0f);
                    lw = mixf(lw, 1.0f, tw_t);
                    lw = clampf(lw, 0.0000000001f, 1.0f);
                }
                float hfw = 1.0f;
                if (!too_rough && br < 0.8f && afc <= ((0.185f + 0.001f) + 0.001f) + 0.0001f) {
                    const float angle = dot(nm_at, nm_base);
                    hfw = dm_pow(clampf(angle, 0.00000001f, 1.0f), hf_e);
                    hfw = clampf(hfw + ((hf_add * 1.075f) * 1.4f), 0.00000000001f, 1.0f);
                }
                const float re = std::fabs(srough - br);
                float rtw = 1.0f / re;
                rtw = dm_pow(rtw, 12.0f);
                rtw = clampf(rtw, 0.00000000001f, 1.0f);
                const float kw = gauss[std::min(std::max(16 + s, 0), 32)];
                float cw = 1.0f;
                cw *= dw;
                cw *= nw;
                cw *= hfw;
                cw *= lw;
                cw *= rtw;
                cw *= kw;
                cw = clampf(cw, 0.000000001f, 1.0f);
                for (int c = 0; c < 4; c++) fc[c] += sd[c] * cw;
                tw += cw;
            }
            float o[4];
            if (tw > 0.001f) {
                for (int c = 0; c < 4; c++) fc[c] = fc[c] / tw;
                float smf = 1.0f;
                if (br <= 0.1f + 0.007f) {
                    smf = br * 16.0f;
                    smf = 1.0f - smf;
                    smf = dm_pow(smf, 4.0f);
                    smf = clampf(smf, 0.1f, 0.999f);
                }
                for (int c = 0; c < 4; c++) o[c] = mixf(bc[c], fc[c], smf);
            } else {
                for (int c = 0; c < 4; c++) o[c] = bc[c];
            }
            for (int c = 0; c < 4; c++) out[q * 4 + c] = storage(o[c], fp16);
        }
    }
}

// TemporalFilter.glsl main (:369-487) with u_DiffuseTemporal on and
// u_ShadowTemporal off, u_MinimumMix 0 and u_MaximumMix 0.96 (the non-SVGF
// path, Core/Pipeline.cpp:2618-2680). The shader writes colour (SH) and CoCg;
// AO passes through and the utility plane is zero.
void vpto_plain_temporal(const vpto_camera* cam, const vpto_camera* prev_cam, const vpto_params* p,
                         const float* t, const float* prev_t, const vpto_gi* cur, const vpto_history* prev,
                         vpto_history* out) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const int fp16 = p->storage;
    const Plane T{t, W, H, 1}, PT{prev_t, p->width, p->height, 1}, PSH{prev->sh, W, H, 4}, PCC{prev->cocg, W, H, 2};
    float m[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            m[c * 4 + r] = ((prev_cam->proj[0 * 4 + r] * prev_cam->view[c * 4 + 0] +
                             prev_cam->proj[1 * 4 + r] * prev_cam->view[c * 4 + 1]) +
                            prev_cam->proj[2 * 4 + r] * prev_cam->view[c * 4 + 2]) +
                           prev_cam->proj[3 * 4 + r] * prev_cam->view[c * 4 + 3];
    const float min_mix = clampf(0.0f, 0.01f, 0.9f), max_mix = clampf(0.96f, 0.1f, 0.98f);
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            const size_t px = (size_t)j * W + i;
            const v2 uv = texcoord(i, j, W, H);
            const v4 bp = position_fetch(cam, T, i, j, uv);
            float osh[4], occ[2];
            for (int c = 0; c < 4; c++) osh[c] = cur->sh[px * 4 + c];
            for (int c = 0; c < 2; c++) occ[c] = cur->cocg[px * 2 + c];
            if (bp.w > 0.0f) {
                const v4 pr = mat_mul4(m, bp.x, bp.y, bp.z, 1.0f);
                const v2 rc = v2{(pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f};
                float psh[4];
                PSH.linear(rc, psh);
                const v4 pp = position_linear(cam, PT, rc);
                const float bias = 0.01f;
                if (rc.x > 0.0f + bias && rc.x < 1.0f - bias && rc.y > 0.0f + bias && rc.y < 1.0f - bias) {
                    const float d = std::fabs(length(sub(mk3(pp.x, pp.y, pp.z), mk3(bp.x, bp.y, bp.z))));
                    if (!(d > 1.1f)) {
                        float bf = dm_exp(-d);
                        bf = clampf(bf, min_mix, max_mix);
                        const float bfc = clampf(bf, 0.0f, 0.96f);
                        float pcc[2];
                        PCC.linear(rc, pcc);
                        for (int c = 0; c < 4; c++) osh[c] = mixf(osh[c], psh[c], bfc);
                        for (int c = 0; c < 2; c++) occ[c] = mixf(occ[c], pcc[c], bf);
                    }
                }
            }
            for (int c = 0; c < 4; c++) out->sh[px * 4 + c] = storage(osh[c], fp16);
            for (int c = 0; c < 2; c++) out->cocg[px * 2 + c] = storage(occ[c], fp16);
            for (int c = 0; c < 2; c++) out->aosky[px * 2 + c] = storage(cur->aosky[px * 2 + c], fp16);
            for (int c = 0; c < 4; c++) out->util[px * 4 + c] = 0.0f;
        }
    }
}

// SampleVarianceCompute.glsl: 5x5 luminance variance of the temporal colour
// (REPEAT wrap at the borders).
void vpto_plain_variance(const vpto_params* p, const float* sh, float* variance) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const Plane SH{sh, W, H, 4};
#pragma omp parallel for schedule(static)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            float tx = 0.0f, ty = 0.0f;
            int n = 0;
            for (int a = -2; a <= 2; a++) {
                for (int b = -2; b <= 2; b++) {
                    const float l = luminance(mk3(SH.at(i + a, j + b, 0), SH.at(i + a, j + b, 1), SH.at(i + a, j + b, 2)));
                    tx += l;
                    ty += l * l;
                    n++;
                }
            }
            const float nn = fmaxg((float)n, 1.0f);
            tx /= nn;
            ty /= nn;
            variance[(size_t)j * W + i] = storage(fmaxg(0.0f, ty - tx * tx), p->storage);
        }
    }
}

// AtrousSpatialFilter.glsl main (:96-220), one iteration with step `step`
// (5x5 B3-spline taps). Its saturation / luminance / edge weights are computed
// and then discarded by the shader (AdditionalWeight is reset to 1), so only
// the position, normal, block and sky gates and the distance weight remain.
void vpto_plain_atrous(const vpto_camera* cam, const vpto_params* p, int step, const float* t, const uint8_t* face,
                       const uint8_t* block, const float* sh, const float* cocg, const float* aosky, float* out_sh,
                       float* out_cocg, float* out_aosky) {
    const int W = p->width / gi_div(p), H = p->height / gi_div(p);
    const int fp16 = p->storage;
    const Plane T{t, W, H, 1};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float weights[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            const size_t px = (size_t)j * W + i;
            const v2 uv = texcoord(i, j, W, H);
            const v4 bp = position_fetch(cam, T, i, j, uv);
            const v3 bn = normal_from_id(face[px], 1.0f);
            const int bblock = std::min(std::max((int)block[px], 0), 127);
            const bool bsky = bp.w < 0.0f;
            float tc[4] = {0, 0, 0, 0}, t2[2] = {0, 0}, tw = 0.0f;
            for (int tx = -2; tx <= 2; tx++) {
                for (int ty = -2; ty <= 2; ty++) {
                    const int ox = step * tx, oy = step * ty;
                    const int si = i + ox, sj = j + oy;
                    if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
                    const size_t sp_ = (size_t)sj * W + si;
                    const v2 sc = v2{uv.x + (float)ox * texel_x, uv.y + (float)oy * texel_y};
                    const v4 pa = position_fetch(cam, T, si, sj, sc);
                    const v3 na = normal_from_id(face[sp_], 1.0f);
                    const int ba = std::min(std::max((int)block[sp_], 0), 127);
                    const float err = (std::fabs(pa.x - bp.x) + std::fabs(pa.y - bp.y)) + std::fabs(pa.z - bp.z);
                    if (err < 4.25f && na.x == bn.x && na.y == bn.y && na.z == bn.z && ba == bblock &&
                        (pa.w < 0.0f) == bsky) {
                        const float dw = dm_pow(std::fabs(4.25f - err), 6.9f);
                        const float wgt = (weights[tx + 2] * weights[ty + 2]) * dw;
                        for (int c = 0; c < 4; c++) tc[c] += sh[sp_ * 4 + c] * wgt;
                        for (int c = 0; c < 2; c++) t2[c] += cocg[sp_ * 2 + c] * wgt;
                        tw += wgt;
                    }
                }
            }
            const float d = fmaxg(tw, 0.01f);
            for (int c = 0; c < 4; c++) out_sh[px * 4 + c] = storage(tc[c] / d, fp16);
            for (int c = 0; c < 2; c++) out_cocg[px * 2 + c] = storage(t2[c] / d, fp16);
            for (int c = 0; c < 2; c++) out_aosky[px * 2 + c] = aosky[px * 2 + c];
        }
    }
}

// High-spp ground truth of the diffuse GI over a crop: per pixel, `spp`
// samples of CalculateDiffuse (DiffuseRayTraceFrag.glsl:535-664), each on its
// own PCG stream, accumulated in float64 with Welford's update per chunk of
// `chunk` samples, chunks merged in order with Chan et al.'s pairwise update.
// Channels: SH (4), CoCg (2), AO.
void vpto_ground_truth(const vpto_world* w, const vpto_camera* cam, const vpto_params* p, const vpto_frame* f,
                       const float* t, const uint8_t* face, int x0, int y0, int cw, int ch, int spp, int chunk,
                       uint32_t seed, double* mean_out, double* m2_out) {
    const int W = p->width, H = p->height;
    const v3 r0 = ray_origin(cam);
    const Lighting L = frame_lighting(f);
    const int nchunks = (spp + chunk - 1) / chunk;
    const int CH = 7;
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < cw * ch; q++) {
        const int i = x0 + q % cw, j = y0 + q / cw;
        const size_t px = (size_t)j * W + i;
        const v3 dir = normalize(ray_dir_at(cam, texcoord(i, j, W, H)));
        const float d = t[px];
        const v3 pos = add(r0, muls(dir, d));
        const v3 nrm = normal_from_id(face[px], 0.5f);
        RowCount cnt;
        double n = 0.0, mean[7], m2[7];
        for (int k = 0; k < CH; k++) mean[k] = m2[k] = 0.0;
        for (int c = 0; c < nchunks; c++) {
            double cn = 0.0, cmean[7], cm2[7];
            for (int k = 0; k < CH; k++) cmean[k] = cm2[k] = 0.0;
            const int k0 = c * chunk, k1 = std::min(spp, k0 + chunk);
            for (int s = k0; s < k1; s++) {
                float v[7], sh[4], cocg[2];
                if (d < 0.0f) {
                    irradiance_to_sh(muls(sky_radiance(dir), 2.66f), nrm, sh, cocg);
                    v[6] = 1.0f;
                } else {
                    uint32_t rng = pcg_hash((uint32_t)px + pcg_hash((uint32_t)s + pcg_hash(seed ^ 0x9E3779B9u)));
                    v3 odir = mk3(0, 0, 0);
                    bool sky = false;
                    v4 x = calculate_diffuse(w, p, f, L, pos, nrm, &rng, &odir, &sky, &cnt);
                    irradiance_to_sh(vclamp(mk3(x.x, x.y, x.z), 0.0f, 8.0f), odir, sh, cocg);
                    v[6] = x.w;
                }
                v[0] = sh[0]; v[1] = sh[1]; v[2] = sh[2]; v[3] = sh[3];
                v[4] = cocg[0]; v[5] = cocg[1];
                cn += 1.0;
                for (int k = 0; k < CH; k++) {
                    const double x = (double)v[k];
                    const double delta = x - cmean[k];
                    cmean[k] = cmean[k] + delta / cn;
                    cm2[k] = cm2[k] + delta * (x - cmean[k]);
                }
            }
            if (cn == 0.0) continue;
            if (n == 0.0) {
                n = cn;
                for (int k = 0; k < CH; k++) { mean[k] = cmean[k]; m2[k] = cm2[k]; }
                continue;
            }
            const double tot = n + cn;
            for (int k = 0; k < CH; k++) {
                const double delta = cmean[k] - mean[k];
                mean[k] = mean[k] + delta * (cn / tot);
                m2[k] = (m2[k] + cm2[k]) + (delta * delta) * ((n * cn) / tot);
            }
            n = tot;
        }
        for (int k = 0; k < CH; k++) {
            mean_out[(size_t)q * CH + k] = mean[k];
            m2_out[(size_t)q * CH + k] = m2[k];
        }
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Textured G-buffer: GenerateGBuffer.glsl main (:347-419) with parallax off
// (u_POM, Core/Pipeline.cpp:264) and no lava block, sampling the block
// texture arrays (Core/BlockDatabase.cpp:60-90) as the CUDA path defines
// GL's texture fetches: REPEAT wrap, LINEAR / LINEAR_MIPMAP_LINEAR with an
// isotropic level of detail log2(max(|dP/dx|, |dP/dy|) * size), fp32 bilinear
// weights, texel = byte / 255 (sRGB-decoded for albedo), mip levels the
// rounded 2 x 2 mean per 8-bit channel, and dFdx / dFdy the fine differences
// inside the 2 x 2 pixel quad with the partner's position projected onto this
// pixel's face axes (zero for a partner outside the image).
namespace {

struct OTexArray {
    std::vector<uint8_t> texels;
    std::vector<long long> level_off;
    int layers = 0, channels = 0, size = 0, levels = 0;
};

OTexArray build_tex_array(const uint8_t* src, int layers, int channels, int size) {
    OTexArray a;
    a.layers = layers;
    a.channels = channels;
    a.size = size;
    int levels = 1;
    while ((size >> (levels - 1)) > 1) levels++;
    a.levels = levels;
    long long off = 0;
    for (int l = 0; l < levels; l++) {
        a.level_off.push_back(off);
        off += (long long)layers * (size >> l) * (size >> l);
    }
    a.texels.assign((size_t)off * channels, 0);
    std::memcpy(a.texels.data(), src, (size_t)layers * size * size * channels);
    for (int l = 0; l + 1 < levels; l++) {
        const int s1 = size >> l, s2 = size >> (l + 1);
        const uint8_t* in = a.texels.data() + a.level_off[l] * channels;
        uint8_t* out = a.texels.data() + a.level_off[l + 1] * channels;
        for (int layer = 0; layer < layers; layer++)
            for (int y = 0; y < s2; y++)
                for (int x = 0; x < s2; x++)
                    for (int c = 0; c < channels; c++) {
                        const uint8_t* r0 = in + (((size_t)layer * s1 + 2 * y) * s1 + 2 * x) * channels;
                        const uint8_t* r1 = r0 + (size_t)s1 * channels;
                        out[(((size_t)layer * s2 + y) * s2 + x) * channels + c] =
                            (uint8_t)(((int)r0[c] + (int)r0[channels + c] + (int)r1[c] + (int)r1[channels + c] + 2) >> 2);
                    }
    }
    return a;
}

float tex_value(uint8_t v, const float* srgb) { return srgb ? srgb[v] : (float)v / 255.0f; }

void tex_bilinear(const OTexArray& a, int level, int layer, float u, float v, int nch, const float* srgb, float* out) {
    const int sl = a.size >> level;
    const float x = u * (float)sl - 0.5f, y = v * (float)sl - 0.5f;
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float ax = x - x0, ay = y - y0, bx = 1.0f - ax, by = 1.0f - ay;
    const int i0 = wrapi(f2i(x0), sl), j0 = wrapi(f2i(y0), sl);
    const int i1 = i0 + 1 == sl ? 0 : i0 + 1, j1 = j0 + 1 == sl ? 0 : j0 + 1;
    const uint8_t* base = a.texels.data() + (a.level_off[level] + (long long)layer * sl * sl) * a.channels;
    const uint8_t* p00 = base + ((size_t)j0 * sl + i0) * a.channels;
    const uint8_t* p10 = base + ((size_t)j0 * sl + i1) * a.channels;
    const uint8_t* p01 = base + ((size_t)j1 * sl + i0) * a.channels;
    const uint8_t* p11 = base + ((size_t)j1 * sl + i1) * a.channels;
    for (int c = 0; c < nch; c++) {
        const float v00 = tex_value(p00[c], srgb), v10 = tex_value(p10[c], srgb);
        const float v01 = tex_value(p01[c], srgb), v11 = tex_value(p11[c], srgb);
        const float lo = v00 * bx + v10 * ax;
        const float hi = v01 * bx + v11 * ax;
        out[c] = lo * by + hi * ay;
    }
}

float tex_lod(int size, float dxu, float dxv, float dyu, float dyv) {
    const float s = (float)size;
    const float ax = dxu * s, ay = dxv * s, bx = dyu * s, by = dyv * s;
    const float rx = std::sqrt(ax * ax + ay * ay), ry = std::sqrt(bx * bx + by * by);
    return dm_log2(fmaxg(rx, ry));
}

void tex_sample(const OTexArray& a, int layer_id, float u, float v, float lam, int nch, const float* srgb, float* out) {
    const int layer = std::min(std::max(layer_id, 0), a.layers - 1);
    const int q = a.levels - 1;
    if (!(lam > 0.0f)) {
        tex_bilinear(a, 0, layer, u, v, nch, srgb, out);
        return;
    }
    if (lam >= (float)q) {
        tex_bilinear(a, q, layer, u, v, nch, srgb, out);
        return;
    }
    const float d1f = std::floor(lam);
    const int d1 = (int)d1f;
    const float f = lam - d1f;
    float t1[4], t2[4];
    tex_bilinear(a, d1, layer, u, v, nch, srgb, t1);
    tex_bilinear(a, d1 + 1, layer, u, v, nch, srgb, t2);
    for (int c = 0; c < nch; c++) out[c] = (1.0f - f) * t1[c] + f * t2[c];
}

// CalculateVectors' face coordinates: (x, y) for +-Z, (x, z) for +-Y, (z, y) for +-X
v2 face_coords(v3 p, int f) {
    const int axis = f >> 1;
    return axis == 0 ? v2{p.x, p.y} : (axis == 1 ? v2{p.x, p.z} : v2{p.z, p.y});
}

v3 gbuffer_position(const vpto_camera* cam, int W, int H, const float* t, int i, int j, float* dist) {
    const float d = 1.0f / (1.0f / t[(size_t)j * W + i]);
    *dist = d;
    return add(ray_origin(cam), muls(normalize(ray_dir_at(cam, texcoord(i, j, W, H))), d));
}

float quad_diff(bool odd, float self, float partner) { return odd ? self - partner : partner - self; }
float dot2(v2 a) { return a.x * a.x + a.y * a.y; }

}  // namespace

extern "C" void vpto_generate_gbuffer(const vpto_camera* cam, const vpto_params* p, const vpto_block_textures* tx,
                                      const float* t, const uint8_t* face, const uint8_t* block, float* albedo,
                                      float* normal, float* pbr, float* ao) {
    const int W = p->width, H = p->height, fp16 = p->storage, S = tx->size;
    const OTexArray A = build_tex_array(tx->albedo, tx->albedo_layers, 4, S);
    const OTexArray N_ = build_tex_array(tx->normal, tx->normal_layers, 4, S);
    const OTexArray P_ = build_tex_array(tx->pbr, tx->pbr_layers, 4, S);
    OTexArray E;
    if (tx->emissive) E = build_tex_array(tx->emissive, tx->emissive_layers, 1, S);
    // sRGB decode of a byte (IEC 61966-2-1)
    float srgb[256];
    for (int v = 0; v < 256; v++) {
        const float x = (float)v / 255.0f;
        srgb[v] = x <= 0.04045f ? x / 12.92f : dm_pow((x + 0.055f) / 1.055f, 2.4f);
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            const size_t px = (size_t)j * W + i;
            float dist;
            const v3 pos = gbuffer_position(cam, W, H, t, i, j, &dist);
            if (dist < 0.0f) {
                for (int c = 0; c < 3; c++) {
                    albedo[px * 3 + c] = storage(0.0f, fp16);
                    normal[px * 3 + c] = storage(1.0f, fp16);
                }
                for (int c = 0; c < 4; c++) pbr[px * 4 + c] = storage(0.0f, fp16);
                ao[px] = storage(0.0f, fp16);
                continue;
            }
            const int f = std::min((int)face[px], 5);
            const int bid = std::min(std::max((int)block[px], 0), 127);
            const v2 P = face_coords(pos, f);
            const v2 F{fract(P.x), fract(P.y)};
            const v2 O{fract(F.x + 0.25f), fract(F.y + 0.25f)};
            const int ix = i ^ 1, jy = j ^ 1;
            v2 Fx = F, Ox = O, Fy = F, Oy = O;
            if (ix < W) {
                float dn;
                const v2 Pn = face_coords(gbuffer_position(cam, W, H, t, ix, j, &dn), f);
                Fx = v2{fract(Pn.x), fract(Pn.y)};
                Ox = v2{fract(Fx.x + 0.25f), fract(Fx.y + 0.25f)};
            }
            if (jy < H) {
                float dn;
                const v2 Pn = face_coords(gbuffer_position(cam, W, H, t, i, jy, &dn), f);
                Fy = v2{fract(Pn.x), fract(Pn.y)};
                Oy = v2{fract(Fy.x + 0.25f), fract(Fy.y + 0.25f)};
            }
            const bool ox = i & 1, oy = j & 1;
            v2 dx{quad_diff(ox, F.x, Fx.x), quad_diff(ox, F.y, Fx.y)};
            v2 dy{quad_diff(oy, F.x, Fy.x), quad_diff(oy, F.y, Fy.y)};
            const v2 dx2{quad_diff(ox, O.x, Ox.x), quad_diff(ox, O.y, Ox.y)};
            const v2 dy2{quad_diff(oy, O.x, Oy.x), quad_diff(oy, O.y, Oy.y)};
            if (dot2(dx) + dot2(dy) > dot2(dx2) + dot2(dy2)) {
                dx = dx2;
                dy = dy2;
            }
            int ia = tx->albedo_id[bid], in_ = tx->normal_id[bid], ip = tx->pbr_id[bid];
            const int ie = tx->emissive ? tx->emissive_id[bid] : -1;
            if (bid == tx->grass[0]) {
                const int k = f == 2 ? 1 : (f == 3 ? 7 : 4);
                ia = tx->grass[k];
                in_ = tx->grass[k + 1];
                ip = tx->grass[k + 2];
            }
            const v2 uv{1.0f - F.x, 1.0f - F.y};
            const float lam = tex_lod(S, dx.x, dx.y, dy.x, dy.y);
            const v3 T = f < 4 ? mk3(1.0f, 0.0f, 0.0f) : mk3(0.0f, 0.0f, -1.0f);
            const v3 B = f < 2 ? mk3(0.0f, 1.0f, 0.0f) : (f < 4 ? mk3(0.0f, 0.0f, 1.0f) : mk3(0.0f, -1.0f, 0.0f));
            const v3 Nf = normal_from_id(f, 1.0f);
            float nm[4], pb[4], al[4];
            tex_sample(N_, in_, uv.x, uv.y, lam, 3, nullptr, nm);
            for (int c = 0; c < 3; c++) nm[c] = nm[c] * 2.0f - 1.0f;
            const v3 nmap = mk3((T.x * nm[0] + B.x * nm[1]) + Nf.x * nm[2], (T.y * nm[0] + B.y * nm[1]) + Nf.y * nm[2],
                                (T.z * nm[0] + B.z * nm[1]) + Nf.z * nm[2]);
            tex_sample(P_, ip, uv.x, uv.y, lam, 4, nullptr, pb);
            float emis = 0.0f;
            if (ie > -1) {
                const v2 ux{1.0f - Fx.x, 1.0f - Fx.y}, uy{1.0f - Fy.x, 1.0f - Fy.y};
                const float lam_e = tex_lod(S, quad_diff(ox, uv.x, ux.x), quad_diff(ox, uv.y, ux.y),
                                            quad_diff(oy, uv.x, uy.x), quad_diff(oy, uv.y, uy.y));
                float e[4];
                tex_sample(E, ie, uv.x, uv.y, lam_e, 1, nullptr, e);
                emis = e[0];
            }
            tex_sample(A, ia, uv.x, uv.y, lam, 3, srgb, al);
            const float lb = 0.02f;
            const float inside = (uv.x > lb && uv.x < 1.0f - lb && uv.y > lb && uv.y < 1.0f - lb) ? 1.0f : 0.0f;
            for (int c = 0; c < 3; c++) albedo[px * 3 + c] = storage(al[c], fp16);
            normal[px * 3 + 0] = storage(nmap.x, fp16);
            normal[px * 3 + 1] = storage(nmap.y, fp16);
            normal[px * 3 + 2] = storage(nmap.z, fp16);
            for (int c = 0; c < 3; c++) pbr[px * 4 + c] = storage(clampf(pb[c], 0.0f, 1.0f), fp16);
            pbr[px * 4 + 3] = storage(clampf(emis, 0.0f, 1.0f) * inside, fp16);
            ao[px] = storage(clampf(pb[3], 0.00000001f, 1.0f), fp16);
        }
    }
}

// Block textures of the diffuse bounce hits (test state of the oracle).
namespace {
struct OTexState {
    bool on = false, has_e = false;
    OTexArray A, N, P, E;
    std::vector<int> albedo_id, normal_id, pbr_id, emissive_id;
    int grass[10];
    int transparent[128];
    float srgb[256];
};
OTexState g_tex;
}  // namespace

extern "C" void vpto_set_block_textures(const vpto_block_textures* tx) {
    g_tex = OTexState{};
    if (!tx) return;
    g_tex.A = build_tex_array(tx->albedo, tx->albedo_layers, 4, tx->size);
    g_tex.N = build_tex_array(tx->normal, tx->normal_layers, 4, tx->size);
    g_tex.P = build_tex_array(tx->pbr, tx->pbr_layers, 4, tx->size);
    g_tex.normal_id.assign(tx->normal_id, tx->normal_id + 128);
    g_tex.pbr_id.assign(tx->pbr_id, tx->pbr_id + 128);
    for (int k = 0; k < 10; k++) g_tex.grass[k] = tx->grass[k];
    for (int b = 0; b < 128; b++) g_tex.transparent[b] = tx->transparent[b] ? 1 : 0;
    g_tex.has_e = tx->emissive != nullptr;
    if (g_tex.has_e) g_tex.E = build_tex_array(tx->emissive, tx->emissive_layers, 1, tx->size);
    g_tex.albedo_id.assign(tx->albedo_id, tx->albedo_id + 128);
    g_tex.emissive_id.assign(tx->emissive_id, tx->emissive_id + 128);
    for (int v = 0; v < 256; v++) {
        const float x = (float)v / 255.0f;
        g_tex.srgb[v] = x <= 0.04045f ? x / 12.92f : dm_pow((x + 0.055f) / 1.055f, 2.4f);
    }
    g_tex.on = true;
}

namespace {
bool tex_bounce_material(int bid, v3 ip, v3 hn, v3* albedo, float* rough, float* emis, bool* has_emis) {
    if (!g_tex.on) return false;
    const v2 P = face_coords(ip, normal_id(hn));
    const float u = fract(P.x), v = fract(P.y);
    const int layer = g_tex.albedo_id[bid], el = g_tex.emissive_id[bid];
    auto level = [&](const OTexArray& a, int id, int lv, int nch, const float* srgb, float* out) {
        const int l = std::min(std::max(id, 0), a.layers - 1);
        tex_bilinear(a, std::min(lv, a.levels - 1), l, u, v, nch, srgb, out);
    };
    float al[4], pb[4];
    level(g_tex.A, layer, 3, 3, g_tex.srgb, al);
    level(g_tex.P, layer, 2, 3, nullptr, pb);
    *albedo = mk3(al[0], al[1], al[2]);
    *rough = pb[0];
    *has_emis = g_tex.has_e && el >= 0;
    *emis = 0.0f;
    if (*has_emis) {
        float e[4];
        level(g_tex.E, el, 0, 1, nullptr, e);
        *emis = e[0];
    }
    return true;
}
}  // namespace

bool tex_reflection_hit(int rid, v3 hp, v3 hn, TexHit* out) {
    if (!g_tex.on) return false;
    const int f = normal_id(hn);
    int ia = g_tex.albedo_id[rid], in_ = g_tex.normal_id[rid], ip = g_tex.pbr_id[rid];
    const int ie = g_tex.has_e ? g_tex.emissive_id[rid] : -1;
    if (rid == g_tex.grass[0]) {
        const int k = f == 2 ? 1 : (f == 3 ? 7 : 4);
        ia = g_tex.grass[k];
        in_ = g_tex.grass[k + 1];
        ip = g_tex.grass[k + 2];
    }
    const v2 fuv = face_uv(hp, hn);
    auto level = [&](const OTexArray& a, int id, int lv, int nch, const float* srgb, float* o) {
        const int l = std::min(std::max(id, 0), a.layers - 1);
        tex_bilinear(a, std::min(lv, a.levels - 1), l, fuv.x, fuv.y, nch, srgb, o);
    };
    float al[4], pb[4], nm[4];
    level(g_tex.A, ia, 0, 3, g_tex.srgb, al);
    level(g_tex.P, ip, 0, 4, nullptr, pb);
    level(g_tex.N, in_, 3, 3, nullptr, nm);
    out->albedo = mk3(al[0], al[1], al[2]);
    out->rough = pb[0];
    out->metal = pb[1];
    out->ao = dm_pow(pb[3], 2.0f);
    for (int c = 0; c < 3; c++) nm[c] = nm[c] * 2.0f - 1.0f;
    const v3 T = f < 4 ? mk3(1.0f, 0.0f, 0.0f) : mk3(0.0f, 0.0f, -1.0f);
    const v3 B = f < 2 ? mk3(0.0f, 1.0f, 0.0f) : (f < 4 ? mk3(0.0f, 0.0f, 1.0f) : mk3(0.0f, -1.0f, 0.0f));
    out->nmap = mk3((T.x * nm[0] + B.x * nm[1]) + hn.x * nm[2], (T.y * nm[0] + B.y * nm[1]) + hn.y * nm[2],
                    (T.z * nm[0] + B.z * nm[1]) + hn.z * nm[2]);
    out->emis = -1.0f;
    if (ie > -1) {
        float e[4];
        level(g_tex.E, ie, 2, 1, nullptr, e);
        out->emis = e[0];
    }
    return true;
}

extern "C" void vpto_set_textured_gbuffer(const float* normal, const float* pbr, int W, int H) {
    g_gbt = GbtState{};
    if (!normal || !pbr) return;
    g_gbt.normal = normal;
    g_gbt.pbr = pbr;
    g_gbt.W = W;
    g_gbt.H = H;
}

namespace {
bool alpha_active(const vpto_params* p) { return p->alpha_test != 0 && g_tex.on; }
bool alpha_active_shadows(const vpto_params* p) { return p->alpha_test_shadows != 0 && g_tex.on; }

bool alpha_stop(v3 p, v3 n, int type, v3 cam, float k, int flip_x, int lod_bias) {
    const int id = std::min(std::max(type, 0), 127);
    if (!g_tex.on || !g_tex.transparent[id]) return true;
    const v2 fc = face_coords(p, normal_id(n));
    const float u = flip_x ? 1.0f - fract(fc.x) : fract(fc.x), v = 1.0f - fract(fc.y);
    const float D = length(sub(p, cam));
    const int lod = std::min(std::max(f2i(dm_log2((float)g_tex.A.size / ((1.0f / D) * k))) + lod_bias, 0), 8);
    const OTexArray& a = g_tex.A;
    const int layer = std::min(std::max(g_tex.albedo_id[id], 0), a.layers - 1);
    float o[4];
    tex_bilinear(a, std::min(lod, a.levels - 1), layer, u, v, 4, nullptr, o);
    return o[3] > 0.975f;
}
}  // namespace

// Test hook: irradiance_to_sh / sh_to_irradiance over n items (vpt_oracle.h).
extern "C" void vpto_sh_codec(int op, int n, const float* in, float* out) {
    for (int k = 0; k < n; k++) {
        if (op == 0) {
            const float* a = in + 6 * k;
            irradiance_to_sh(mk3(a[0], a[1], a[2]), mk3(a[3], a[4], a[5]), out + 6 * k, out + 6 * k + 4);
        } else {
            const float* a = in + 9 * k;
            const v3 r = sh_to_irradiance(a, a + 4, mk3(a[6], a[7], a[8]));
            out[3 * k] = r.x;
            out[3 * k + 1] = r.y;
            out[3 * k + 2] = r.z;
        }
    }
}

// Test hook: DiffuseRayBRDF = diffuse_hammon(n, -incident, d, roughness) over n items.
extern "C" void vpto_diffuse_brdf(int n, const float* in, float* out) {
    for (int k = 0; k < n; k++) {
        const float* a = in + 10 * k;
        out[k] = diffuse_hammon(mk3(a[0], a[1], a[2]), neg(mk3(a[3], a[4], a[5])), mk3(a[6], a[7], a[8]), a[9]);
    }
}
