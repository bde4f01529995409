// DF-accelerated voxel DDA (VoxelTraversalDF, InitialRayTraceFrag.glsl:307-374;
// identical loops at ShadowRayTraceFrag.glsl:222-289 and
// DiffuseRayTraceFrag.glsl:1043-1110) written as a resumable state machine:
// ray_start sets up the loop, dda_step runs one iteration of the loop body,
// ray_finish evaluates the code after the loop. `traverse` runs it to the end.
// All arithmetic is IEEE fp32 without fused multiply-adds, so hit voxel, face
// and step count are bit-identical to the CPU restatement.
#pragma once
#include "common.cuh"

namespace vpt {

// int(floor(ToConservativeEuclidean(Dist))) (InitialRayTraceFrag.glsl:89-92, :328-330);
// texelFetch(R8)*255 gives back the stored integer exactly.
__device__ __forceinline__ int euclid_steps(int dist) {
    float D = (float)dist;
    float e = (D == 1.0f) ? 1.0f : D * 0.57735026918f;
    return f2i_floor(e);
}

struct RayState {
    v3 o;            // current origin
    v3 d;            // direction
    v3 init;         // initial origin
    float ix, iy, iz;  // 1 / direction
    int itr;         // loop counter
    int max_steps;
    int min_idx;
    int inter;       // Intersection flag
};

struct TraceResult {
    float t;
    v3 normal;
    int block;
    int cell[3];
    int steps;
};

__device__ __forceinline__ void ray_start(RayState& r, v3 origin, v3 dir, int max_steps) {
    r.o = origin;
    r.d = dir;
    r.init = origin;
    r.ix = 1.0f / dir.x;
    r.iy = 1.0f / dir.y;
    r.iz = 1.0f / dir.z;
    r.itr = 0;
    r.max_steps = max_steps;
    r.min_idx = 0;
    r.inter = 0;
}

// One exact DDA face step (:341-356), the E == 1 branch's body; updates the
// origin and MinIdx.
__device__ __forceinline__ void dda_face_step(RayState& r) {
    const int sx = isign(r.d.x), sy = isign(r.d.y), sz = isign(r.d.z);
    const int hx = (1 + sx) >> 1, hy = (1 + sy) >> 1, hz = (1 + sz) >> 1;
    int gx = f2i(r.o.x), gy = f2i(r.o.y), gz = f2i(r.o.z);
    float wx = r.o.x - (float)gx, wy = r.o.y - (float)gy, wz = r.o.z - (float)gz;
    const float dfx = ((float)hx - wx) * r.ix;
    const float dfy = ((float)hy - wy) * r.iy;
    const float dfz = ((float)hz - wz) * r.iz;
    const int m = (dfx < dfy && sx != 0) ? ((dfx < dfz || sz == 0) ? 0 : 2) : ((dfy < dfz || sz == 0) ? 1 : 2);
    const float dm = m == 0 ? dfx : (m == 1 ? dfy : dfz);
    wx = wx + r.d.x * dm;
    wy = wy + r.d.y * dm;
    wz = wz + r.d.z * dm;
    if (m == 0) { gx += sx; wx = (float)(1 - hx); }
    else if (m == 1) { gy += sy; wy = (float)(1 - hy); }
    else { gz += sz; wz = (float)(1 - hz); }
    r.o.x = (float)gx + wx;
    r.o.y = (float)gy + wy;
    r.o.z = (float)gz + wz;
    if (m == 0) r.o.x = r.o.x + (float)sx * 0.0001f;
    else if (m == 1) r.o.y = r.o.y + (float)sy * 0.0001f;
    else r.o.z = r.o.z + (float)sz * 0.0001f;
    r.min_idx = m;
}

// One iteration of the traversal loop in two halves around its one memory
// access: dda_fetch returns true if the loop ends before the distance-field
// gather (step cap, or the ray left the volume), else the gather's address;
// dda_apply takes the gathered distance and returns true once the loop is
// over. B is the distance-field layout (df_index).
template <int B = 0>
__device__ __forceinline__ bool dda_fetch(const WorldView& w, RayState& r, int* addr) {
    if (r.itr >= r.max_steps) return true;
    const int lx = f2i_floor(r.o.x);
    const int ly = f2i_floor(r.o.y);
    const int lz = f2i_floor(r.o.z);
    if (!in_volume(w, lx, ly, lz)) {
        r.inter = 0;
        return true;
    }
    *addr = df_index<B>(w, lx, ly, lz);
    return false;
}

__device__ __forceinline__ bool dda_apply(RayState& r, int dist) {
    const int e = euclid_steps(dist);
    if (e == 0) return true;
    if (e == 1) {
        dda_face_step(r);
        r.inter = 1;
    } else {
        // jump by the conservative Euclidean radius (:361)
        const float k = (float)(e - 1);
        r.o.x = r.o.x + k * r.d.x;
        r.o.y = r.o.y + k * r.d.y;
        r.o.z = r.o.z + k * r.d.z;
    }
    r.itr++;
    return r.itr >= r.max_steps;
}

// One iteration of the traversal loop; returns true once the loop is over.
template <int B = 0>
__device__ __forceinline__ bool dda_step(const WorldView& w, RayState& r) {
    int addr = 0;
    if (dda_fetch<B>(w, r, &addr)) return true;
    return dda_apply(r, (int)__ldg(w.df + addr));
}

// The code after the loop (:365-373).
__device__ __forceinline__ TraceResult ray_finish(const WorldView& w, const RayState& r) {
    TraceResult t;
    t.cell[0] = f2i_floor(r.o.x);
    t.cell[1] = f2i_floor(r.o.y);
    t.cell[2] = f2i_floor(r.o.z);
    t.steps = r.itr;
    t.normal = mk3(0.0f, 0.0f, 0.0f);
    t.block = 0;
    t.t = -1.0f;
    if (r.inter) {
        const int m = r.min_idx;
        const int s = m == 0 ? isign(r.d.x) : (m == 1 ? isign(r.d.y) : isign(r.d.z));
        const float nv = (float)(-s);
        if (m == 0) t.normal.x = nv; else if (m == 1) t.normal.y = nv; else t.normal.z = nv;
        t.block = get_voxel(w, t.cell[0], t.cell[1], t.cell[2]);
        t.t = t.block > 0 ? length(sub(r.o, r.init)) : -1.0f;
    }
    return t;
}

template <int B = 0>
__device__ __forceinline__ TraceResult traverse(const WorldView& w, v3 origin, v3 direction, int max_steps) {
    RayState r;
    ray_start(r, origin, direction, max_steps);
    while (!dda_step<B>(w, r)) {
    }
    return ray_finish(w, r);
}

// Two rays traversed together by one thread, their DDA steps interleaved so
// that both distance-field gathers of an iteration are in flight at once (the
// gather latency is what bounds a lone ray). Each ray's state evolves exactly
// as in traverse; a ray with live == false is not traced.
template <int B = 0>
__device__ __forceinline__ void traverse2(const WorldView& w, v3 o0, v3 d0, int n0, bool live0, v3 o1, v3 d1, int n1,
                                          bool live1, TraceResult* r0, TraceResult* r1) {
    RayState a, b;
    ray_start(a, o0, d0, n0);
    ray_start(b, o1, d1, n1);
    bool fa = !live0, fb = !live1;
    while (!(fa && fb)) {
        int ia = 0, ib = 0;
        const bool ea = fa || dda_fetch<B>(w, a, &ia);
        const bool eb = fb || dda_fetch<B>(w, b, &ib);
        const int va = ea ? 0 : (int)__ldg(w.df + ia);
        const int vb = eb ? 0 : (int)__ldg(w.df + ib);
        fa = ea || dda_apply(a, va);
        fb = eb || dda_apply(b, vb);
    }
    if (live0) *r0 = ray_finish(w, a);
    if (live1) *r1 = ray_finish(w, b);
}

// The normal of the last face step: normal[MinIdx] = -sign(direction[MinIdx]).
__device__ __forceinline__ v3 step_normal(const RayState& r) {
    const int m = r.min_idx;
    const int s = m == 0 ? isign(r.d.x) : (m == 1 ? isign(r.d.y) : isign(r.d.z));
    v3 n = mk3(0.0f, 0.0f, 0.0f);
    if (m == 0) n.x = (float)(-s); else if (m == 1) n.y = (float)(-s); else n.z = (float)(-s);
    return n;
}

// VoxelTraversalDF_AlphaTest (InitialRayTraceFrag.glsl:204-305): as the DF
// traversal, but at a solid voxel (E == 0) `stop(origin, normal, block)`
// (StopRay, :189-202) decides whether the ray ends there; if not, up to four
// exact face steps look for a voxel that stops it, after which the loop goes
// on from one direction length back (origin += (E - 1) * direction, E = 0).
template <int B, typename Stop>
__device__ __forceinline__ TraceResult traverse_alpha(const WorldView& w, v3 origin, v3 direction, int max_steps,
                                                      const Stop& stop) {
    RayState r;
    ray_start(r, origin, direction, max_steps);
    bool inter = false;
    for (r.itr = 0; r.itr < max_steps; r.itr++) {
        const int lx = f2i_floor(r.o.x), ly = f2i_floor(r.o.y), lz = f2i_floor(r.o.z);
        if (!in_volume(w, lx, ly, lz)) {
            inter = false;
            break;
        }
        const int e = euclid_steps((int)__ldg(w.df + df_index<B>(w, lx, ly, lz)));
        if (e == 0) {
            if (stop(r.o, step_normal(r), get_voxel(w, lx, ly, lz))) break;
            for (int k = 0; k < 4; k++) {
                dda_face_step(r);
                const int cx = f2i_floor(r.o.x), cy = f2i_floor(r.o.y), cz = f2i_floor(r.o.z);
                const int bt = get_voxel(w, cx, cy, cz);
                if (bt > 0 && stop(r.o, step_normal(r), bt)) {
                    TraceResult t;
                    t.cell[0] = cx;
                    t.cell[1] = cy;
                    t.cell[2] = cz;
                    t.steps = r.itr;
                    t.normal = step_normal(r);
                    t.block = bt;
                    t.t = length(sub(r.o, r.init));
                    return t;
                }
            }
        }
        if (e == 1) {
            dda_face_step(r);
            inter = true;
        } else {
            const float k = (float)(e - 1);
            r.o.x = r.o.x + k * r.d.x;
            r.o.y = r.o.y + k * r.d.y;
            r.o.z = r.o.z + k * r.d.z;
        }
    }
    r.inter = inter ? 1 : 0;
    return ray_finish(w, r);
}

// GetNormalID (InitialRayTraceFrag.glsl:143-185): exact compares, 0 if none match.
__device__ __forceinline__ int normal_id(v3 n) {
    if (n.x == 0.0f && n.y == 0.0f && n.z == 1.0f) return 0;
    if (n.x == 0.0f && n.y == 0.0f && n.z == -1.0f) return 1;
    if (n.x == 0.0f && n.y == 1.0f && n.z == 0.0f) return 2;
    if (n.x == 0.0f && n.y == -1.0f && n.z == 0.0f) return 3;
    if (n.x == -1.0f && n.y == 0.0f && n.z == 0.0f) return 4;
    if (n.x == 1.0f && n.y == 0.0f && n.z == 0.0f) return 5;
    return 0;
}

}  // namespace vpt
