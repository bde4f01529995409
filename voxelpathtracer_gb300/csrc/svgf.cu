// SVGF denoiser kernels: pre-temporal 3x3 spatial pass, temporal
// reprojection/accumulation, variance estimate and the a-trous iterations
// (Core/Pipeline.cpp:2284-2615). One thread per pixel, 32x8 blocks so a warp
// reads 32 consecutive pixels of a row.
//
// Taps at integer offsets are direct fetches (what texture() returns at a
// texel centre); taps at fractional coordinates are fp32 bilinear with REPEAT
// wrap, the footprint computed once per tap and shared by every plane read
// there. Multi-channel planes are read with one vector load per texel. The
// kernels are bound by L1 load throughput and the per-tap weight arithmetic.
#include "kernels.cuh"

namespace vpt {

namespace {

__device__ __forceinline__ bool pixel_of(int W, int H, int* i, int* j) {
    *i = blockIdx.x * blockDim.x + threadIdx.x;
    *j = blockIdx.y * blockDim.y + threadIdx.y;
    return *i < W && *j < H;
}

// A value as a plane of storage type S holds it (fp16 planes round to half).
__device__ __forceinline__ float as_stored(float v, const float*) { return v; }
__device__ __forceinline__ float as_stored(float v, const __half*) { return __half2float(__float2half_rn(v)); }

// The pre-filter's tap fetches at an in-image texel (si, sj): the depth, and
// the SH, CoCg, face and AO/sky; from the planes, or from a shared-memory
// tile of the 34 x 10 texels around a 32 x 8 block.
template <typename S>
struct PreGlobal {
    int W;
    const S *t, *sh, *cocg, *aosky;
    const uint8_t* face;
    __device__ __forceinline__ float depth(int si, int sj) const { return ld(t + (size_t)sj * W + si); }
    __device__ __forceinline__ void tap(int si, int sj, float4* s4, float2* s2, int* f, float2* a2) const {
        const size_t q = (size_t)sj * W + si;
        *s4 = ld4(sh + 4 * q);
        *s2 = ld2(cocg + 2 * q);
        *f = __ldg(face + q);
        *a2 = ld2(aosky + 2 * q);
    }
};
constexpr int kPreTW = 34, kPreTH = 10, kPreN = kPreTW * kPreTH;
struct PreTile {
    const float4 *A, *B;
    const float2* C;   // (depth, face)
    int tx0, ty0;
    __device__ __forceinline__ float depth(int si, int sj) const { return C[(sj - ty0) * kPreTW + si - tx0].x; }
    __device__ __forceinline__ void tap(int si, int sj, float4* s4, float2* s2, int* f, float2* a2) const {
        const int k = (sj - ty0) * kPreTW + si - tx0;
        *s4 = A[k];
        const float4 b = B[k];
        *s2 = make_float2(b.x, b.y);
        *a2 = make_float2(b.z, b.w);
        *f = __float_as_int(C[k].y);
    }
};

// Spatial3x3Initial.glsl main (:96-176) for texel (i, j) with texture
// coordinate uv and reconstructed position bp; out: SH (4), CoCg (2), AO/sky
// (2) and the luminance passed through.
template <typename S, class PF = PreGlobal<S>>
__device__ __forceinline__ void pre_filter_texel(const CamView& cam, int W, int H, const Plane<S, 1>& T,
                                                 const uint8_t* face, const S* sh, const S* cocg, const S* luma,
                                                 const S* aosky, int i, int j, v2 uv, v4 bp, float* o_sh,
                                                 float* o_cc, float* o_ao, float* o_luma, const PF* pf = nullptr) {
    const PreGlobal<S> pg{W, T.p, sh, cocg, aosky, face};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float aw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    const size_t px = (size_t)j * W + i;
    const int bf = __ldg(face + px);
    const float nw3 = dpow(3.0f, 16.0f);   // the normal weight of two misses
    const float4 bsh = ld4(sh + 4 * px);
    const float2 bcc = ld2(cocg + 2 * px), bao = ld2(aosky + 2 * px);
    float bshv[4] = {bsh.x, bsh.y, bsh.z, bsh.w};
    const float bl = sh_to_y(bshv);
    const float butil = ld(luma + px);
    // packed sums: SH (2 pairs), CoCg, AO/sky, (weight, AO/sky weight)
    float2 t01 = make_float2(bsh.x, bsh.y), t23 = make_float2(bsh.z, bsh.w), tcc2 = bcc, tao2 = bao;
    float2 tww = make_float2(1.0f, 1.0f);
    const float phi = 4.0f;
    // the tap loops stay rolled where the kernel's unrolled body overflows the
    // instruction cache (measured: warps stalled on instruction fetch)
#pragma unroll 1
    for (int x = -1; x <= 1; x++) {
#pragma unroll
        for (int y = -1; y <= 1; y++) {
            if (x == 0 && y == 0) continue;
            const int si = i + x, sj = j + y;
            if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
            v2 sc = mk2(uv.x + (float)x * texel_x, uv.y + (float)y * texel_y);
            // GetPositionAt: position_fetch's operations on the tap's depth
            const float sd = pf ? pf->depth(si, sj) : pg.depth(si, sj);
            const v3 spp = add(ray_origin(cam), muls(normalize(ray_dir_at(cam, sc)), sd));
            v3 pd = mk3(fabsf(spp.x - bp.x), fabsf(spp.y - bp.y), fabsf(spp.z - bp.z));
            float dist_sqr = dot(pd, pd);
            if (dist_sqr < 1.0f) {
                float4 s4;
                float2 s2, a2;
                int sf;
                if (pf) pf->tap(si, sj, &s4, &s2, &sf, &a2);
                else pg.tap(si, sj, &s4, &s2, &sf, &a2);
                float ssh[4] = {s4.x, s4.y, s4.z, s4.w};
                const int fc = face_cos(bf, sf);
                float sl = sh_to_y(ssh);
                // pow(max(dot(n, n'), 0), 16) for a clamped dot of 0, 1 or 3
                float nw = fc == 0 ? 0.0f : (fc == 1 ? 1.0f : nw3);
                float lw = fabsf(sl - bl) / phi;
                float wgt = dexp(-lw - nw);
                wgt = fmaxf(wgt, 0.01f);
                wgt = ((x == 0 ? aw[0] : aw[1]) * aw[y < 0 ? -y : y]) * wgt;
                wgt = fmaxf(wgt, 0.01f);
                wgt = clampf(wgt, 0.0f, 1.0f);
                t01 = pacc(t01, make_float2(s4.x, s4.y), wgt);
                t23 = pacc(t23, make_float2(s4.z, s4.w), wgt);
                tcc2 = pacc(tcc2, s2, wgt);
                tao2 = pacc(tao2, a2, wgt);
                tww = padd(tww, splat(wgt));
            }
        }
    }
    const float tw = fmaxf(tww.x, 0.01f);
    o_sh[0] = t01.x / tw;
    o_sh[1] = t01.y / tw;
    o_sh[2] = t23.x / tw;
    o_sh[3] = t23.y / tw;
    o_cc[0] = tcc2.x / tw;
    o_cc[1] = tcc2.y / tw;
    const float awt = fmaxf(tww.y, 0.01f);
    o_ao[0] = tao2.x / awt;
    o_ao[1] = tao2.y / awt;
    *o_luma = butil;
}

template <typename S>
__global__ void __launch_bounds__(256) k_spatial_initial(CamView cam, int W, int H, const S* t, const uint8_t* face,
                                                         const S* sh, const S* cocg, const S* luma, const S* aosky,
                                                         S* o_sh, S* o_cocg, S* o_luma, S* o_aosky) {
    __shared__ float4 s_a[kPreN], s_b[kPreN];
    __shared__ float2 s_c[kPreN];
    pdl_enter();
    // the block's 3x3 neighbourhoods, loaded once (taps outside the image are
    // skipped by the filter and never read)
    const int tx0 = (int)blockIdx.x * 32 - 1, ty0 = (int)blockIdx.y * 8 - 1;
    for (int q = threadIdx.y * 32 + threadIdx.x; q < kPreN; q += 256) {
        const int ly = q / kPreTW, lx = q - ly * kPreTW;
        const int si = tx0 + lx, sj = ty0 + ly;
        if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
        const size_t g = (size_t)sj * W + si;
        const float2 cc = ld2(cocg + 2 * g), ao = ld2(aosky + 2 * g);
        s_a[q] = ld4(sh + 4 * g);
        s_b[q] = make_float4(cc.x, cc.y, ao.x, ao.y);
        s_c[q] = make_float2(ld(t + g), __int_as_float((int)__ldg(face + g)));
    }
    __syncthreads();
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const size_t px = (size_t)j * W + i;
    const v2 uv = texcoord(i, j, W, H);
    const v4 bp = position_fetch(cam, T, i, j, uv);
    float psh[4], pcc[2], pao[2], pl;
    const PreTile tile{s_a, s_b, s_c, tx0, ty0};
    pre_filter_texel<S, PreTile>(cam, W, H, T, face, sh, cocg, luma, aosky, i, j, uv, bp, psh, pcc, pao, &pl, &tile);
    st4(o_sh + 4 * px, psh[0], psh[1], psh[2], psh[3]);
    st2(o_cocg + 2 * px, pcc[0], pcc[1]);
    st2(o_aosky + 2 * px, pao[0], pao[1]);
    st(o_luma + px, pl);
}

// SVGF/TemporalFilter.glsl main (:132-360). t / face / block: this frame's
// G-buffer on the GI grid; prev_t / prev_face / prev_block: the previous
// G-buffer at its own Wf x Hf, sampled at the reprojected points (kScaled
// when that grid is finer than the GI grid, so the two need separate
// bilinear footprints).
// The temporal pass for texel (i, j) with texture coordinate uv, position bp
// and this frame's (pre-filtered) SH bsh, CoCg bcc, AO/sky bao and luminance
// base_lum, as the planes hold them.
// The history taps' weighted sums of the temporal pass (the loop of
// TemporalFilter.glsl main over the five reprojected taps): the part that
// reads only the G-buffers and the previous frame's history.
struct TemporalSums {
    float2 sh01, sh23, cc, ao, sm, lw;   // lw = (luminance sum, weight sum)
    int successful;
};
template <typename S, bool kScaled>
__device__ __forceinline__ TemporalSums temporal_gather(const CamView& cam, int W, int H, int Wf, int Hf,
                                                        const TemporalArgs& a, const uint8_t* face,
                                                        const uint8_t* block, const S* prev_t,
                                                        const uint8_t* prev_face, const uint8_t* prev_block, int i,
                                                        int j, v4 bp, const S* p_sh, const S* p_cocg,
                                                        const S* p_util, const S* p_aosky) {
    const Plane8 PF{prev_face, Wf, Hf}, PB{prev_block, Wf, Hf};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    // taps k = 0..4 at (1, 0), (0, 1), (0, 0), (-1, 0), (0, -1), weights 3/32 and 9/64 at the centre
    const size_t px = (size_t)j * W + i;
    const v3 bn = normal_from_id(__ldg(face + px), 1.0f);
    const v4 pr = mat_mul4(a.prev_view_proj, bp.x, bp.y, bp.z, 1.0f);
    const v2 rc = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
    const int base_block = min(max((int)__ldg(block + px), 0), 127);
    float tol = 0.75f;
    bool do_block = true, do_normal = true;
    const float dp = length(sub(mk3(bp.x, bp.y, bp.z), ray_origin(cam)));
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
    // packed sums: SH (2 pairs), CoCg, AO/sky, (spp, moment), (luminance, weight)
    float2 p_sh01 = make_float2(0.0f, 0.0f), p_sh23 = p_sh01, p_cc = p_sh01, p_ao = p_sh01, p_sm = p_sh01,
           p_lw = p_sh01;
    int successful = 0;
#pragma unroll 1   // rolled: the unrolled body overflows the instruction cache
    for (int k = 0; k < 5; k++) {
        const int offx = k == 0 ? 1 : (k == 3 ? -1 : 0), offy = k == 1 ? 1 : (k == 4 ? -1 : 0);
        // Jitter is ivec2((noise - 0.5) * 1.0) == 0 for every pixel (:165)
        v2 sc = mk2(rc.x + ((float)offx + 0.0f) * texel_x, rc.y + ((float)offy + 0.0f) * texel_y);
        const float b = 0.0035f;
        if (!(sc.x < 1.0f - b && sc.x > b && sc.y < 1.0f - b && sc.y > b)) continue;
        const Bilin fp = bilin(sc, W, H);
        const Bilin fq = kScaled ? bilin(sc, Wf, Hf) : fp;
        const float pt = bl1(prev_t, fq);
        const v3 pdir = normalize(ray_dir_at(cam, sc));
        const v3 pp = add(ray_origin(cam), muls(pdir, pt));
        v3 pn = normal_from_id(PF.nearest(sc), 1.0f);
        v3 pd = mk3(fabsf(bp.x - pp.x), fabsf(bp.y - pp.y), fabsf(bp.z - pp.z));
        float perr = dot(pd, pd);
        const float cw = k == 2 ? 9.0f / 64.0f : 3.0f / 32.0f;
        int sblock = min(max(PB.nearest(sc), 0), 127);
        bool valid = false;
        if (perr < tol && ((pt < 0.0f) == (bp.w < 0.0f))) {
            valid = true;
            if (do_normal && !(pn.x == bn.x && pn.y == bn.y && pn.z == bn.z)) valid = false;
            if (do_block && base_block != sblock) valid = false;
        }
        if (valid) {
            float4 pu = bl4(p_util, fp), psh = bl4(p_sh, fp);
            float2 pcc = bl2(p_cocg, fp), pao = bl2(p_aosky, fp);
            p_sh01 = pacc(p_sh01, make_float2(psh.x, psh.y), cw);
            p_sh23 = pacc(p_sh23, make_float2(psh.z, psh.w), cw);
            p_cc = pacc(p_cc, pcc, cw);
            p_sm = pacc(p_sm, make_float2(pu.x, pu.y), cw);
            p_lw = sadd(p_lw, pmul(make_float2(pu.z, cw), make_float2(cw, 1.0f)));   // (lum * cw, cw * 1 == cw)
            p_ao = pacc(p_ao, pao, cw);
            successful++;
        }
    }
    return TemporalSums{p_sh01, p_sh23, p_cc, p_ao, p_sm, p_lw, successful};
}

// The rest of the pass for texel px: the sums blended with this frame's
// (pre-filtered) SH bsh, CoCg bcc, AO/sky bao and luminance base_lum as the
// planes hold them, and the history written.
template <typename S>
__device__ __forceinline__ void temporal_blend(const TemporalArgs& a, size_t px, const TemporalSums& ts, float4 bsh,
                                               float2 bcc, float2 bao, float base_lum, S* o_sh, S* o_cocg,
                                               S* o_util, S* o_aosky) {
    const float2 p_sh01 = ts.sh01, p_sh23 = ts.sh23, p_cc = ts.cc, p_ao = ts.ao, p_sm = ts.sm, p_lw = ts.lw;
    int successful = ts.successful;
    float ssh[4] = {p_sh01.x, p_sh01.y, p_sh23.x, p_sh23.y}, scc[2] = {p_cc.x, p_cc.y}, sao[2] = {p_ao.x, p_ao.y};
    float sspp = p_sm.x, smom = p_sm.y, slum = p_lw.x;
    const float tw = p_lw.y;
    if (tw > 0.001f) {
        for (int c = 0; c < 4; c++) ssh[c] /= tw;
        scc[0] /= tw;
        scc[1] /= tw;
        smom /= tw;
        sspp /= tw;
        slum /= tw;
        sao[0] /= tw;
        sao[1] /= tw;
    } else {
        successful = 0;
    }
    const float inc = a.be_useful ? 1.0f : 0.0f;
    float spp_inc = sspp + inc;
    if (successful <= 0) spp_inc = 0.01f;
    float blend_f = fmaxf(1.0f / spp_inc, 0.05f);
    const float mfac = fmaxf(1.0f / spp_inc, 0.05f);
    if (!a.be_useful) { blend_f = 0.99f; sspp = 0.0f; }
    float util_spp = spp_inc;
    if (successful <= 0) util_spp = 0.0f;
    const float util_mom = (1.0f - mfac) * smom + mfac * (base_lum * base_lum);
    const float store_luma = mixf(slum, base_lum, blend_f);
    float osh[4], occ[2], oao[2];
    const float bshv[4] = {bsh.x, bsh.y, bsh.z, bsh.w};
    for (int c = 0; c < 4; c++) osh[c] = mixf(ssh[c], bshv[c], blend_f);
    occ[0] = mixf(scc[0], bcc.x, blend_f);
    occ[1] = mixf(scc[1], bcc.y, blend_f);
    oao[0] = mixf(sao[0], bao.x, blend_f);
    oao[1] = mixf(sao[1], bao.y, blend_f);
    if (successful <= 0) {
        for (int c = 0; c < 4; c++) osh[c] = bshv[c];
        occ[0] = bcc.x; occ[1] = bcc.y;
        oao[0] = bao.x; oao[1] = bao.y;
    }
    st4(o_sh + 4 * px, clampf(osh[0], -100.0f, 100.0f), clampf(osh[1], -100.0f, 100.0f),
        clampf(osh[2], -100.0f, 100.0f), clampf(osh[3], -100.0f, 100.0f));
    st2(o_cocg + 2 * px, clampf(occ[0], -10.0f, 100.0f), clampf(occ[1], -10.0f, 100.0f));
    st2(o_aosky + 2 * px, clampf(oao[0], 0.0f, 1.0f), clampf(oao[1], 0.0f, 1.0f));
    st4(o_util + 4 * px, clampf(util_spp, -150.0f, 150.0f), clampf(util_mom, -150.0f, 150.0f),
        clampf(store_luma, -150.0f, 150.0f), 0.0f);
}

// The whole temporal pass for texel (i, j) with position bp.
template <typename S, bool kScaled>
__device__ __forceinline__ void temporal_texel(const CamView& cam, int W, int H, int Wf, int Hf, const TemporalArgs& a,
                                               const uint8_t* face, const uint8_t* block, const S* prev_t,
                                               const uint8_t* prev_face, const uint8_t* prev_block, int i, int j,
                                               v2 uv, v4 bp, float4 bsh, float2 bcc, float2 bao, float base_lum,
                                               const S* p_sh, const S* p_cocg, const S* p_util, const S* p_aosky,
                                               S* o_sh, S* o_cocg, S* o_util, S* o_aosky) {
    (void)uv;
    const TemporalSums ts = temporal_gather<S, kScaled>(cam, W, H, Wf, Hf, a, face, block, prev_t, prev_face,
                                                        prev_block, i, j, bp, p_sh, p_cocg, p_util, p_aosky);
    temporal_blend<S>(a, (size_t)j * W + i, ts, bsh, bcc, bao, base_lum, o_sh, o_cocg, o_util, o_aosky);
}

template <typename S, bool kScaled>
__global__ void __launch_bounds__(256, 4) k_temporal(CamView cam, int W, int H, int Wf, int Hf, TemporalArgs a, const S* t,
                                                  const uint8_t* face, const uint8_t* block, const S* prev_t,
                                                  const uint8_t* prev_face, const uint8_t* prev_block,
                                                  const S* c_sh, const S* c_cocg, const S* c_luma, const S* c_aosky,
                                                  const S* p_sh, const S* p_cocg, const S* p_util, const S* p_aosky,
                                                  S* o_sh, S* o_cocg, S* o_util, S* o_aosky) {
    pdl_enter();
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const size_t px = (size_t)j * W + i;
    const v2 uv = texcoord(i, j, W, H);
    const v4 bp = position_fetch(cam, T, i, j, uv);
    temporal_texel<S, kScaled>(cam, W, H, Wf, Hf, a, face, block, prev_t, prev_face, prev_block, i, j, uv, bp,
                               ld4(c_sh + 4 * px), ld2(c_cocg + 2 * px), ld2(c_aosky + 2 * px), ld(c_luma + px), p_sh,
                               p_cocg, p_util, p_aosky, o_sh, o_cocg, o_util, o_aosky);
}

// The temporal pass in two launches, so that its history gather (all but
// the final blend) can run beside the diffuse trace and the pre-filter:
// k_temporal_gather stores each texel's sums (four float4: SH; CoCg, AO/sky;
// moments, luminance and weight; taps accepted), k_temporal_blend blends them
// with the pre-filtered planes once those exist. GI and G-buffer on one grid.
template <typename S>
__global__ void __launch_bounds__(256, 4) k_temporal_gather(CamView cam, int W, int H, TemporalArgs a, const S* t,
                                                         const uint8_t* face, const uint8_t* block, const S* prev_t,
                                                         const uint8_t* prev_face, const uint8_t* prev_block,
                                                         const S* p_sh, const S* p_cocg, const S* p_util,
                                                         const S* p_aosky, float4* sums) {
    pdl_enter();
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const size_t px = (size_t)j * W + i;
    const v4 bp = position_fetch(cam, T, i, j, texcoord(i, j, W, H));
    const TemporalSums ts = temporal_gather<S, false>(cam, W, H, W, H, a, face, block, prev_t, prev_face, prev_block,
                                                      i, j, bp, p_sh, p_cocg, p_util, p_aosky);
    float4* o = sums + 4 * px;
    o[0] = make_float4(ts.sh01.x, ts.sh01.y, ts.sh23.x, ts.sh23.y);
    o[1] = make_float4(ts.cc.x, ts.cc.y, ts.ao.x, ts.ao.y);
    o[2] = make_float4(ts.sm.x, ts.sm.y, ts.lw.x, ts.lw.y);
    o[3] = make_float4(__int_as_float(ts.successful), 0.0f, 0.0f, 0.0f);
}

template <typename S>
__global__ void __launch_bounds__(256) k_temporal_blend(int W, int H, TemporalArgs a, const float4* sums,
                                                        const S* c_sh, const S* c_cocg, const S* c_luma,
                                                        const S* c_aosky, S* o_sh, S* o_cocg, S* o_util,
                                                        S* o_aosky) {
    pdl_enter();
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const size_t px = (size_t)j * W + i;
    const float4* q = sums + 4 * px;
    const float4 s0 = q[0], s1 = q[1], s2 = q[2], s3 = q[3];
    const TemporalSums ts{make_float2(s0.x, s0.y), make_float2(s0.z, s0.w), make_float2(s1.x, s1.y),
                          make_float2(s1.z, s1.w), make_float2(s2.x, s2.y), make_float2(s2.z, s2.w),
                          __float_as_int(s3.x)};
    temporal_blend<S>(a, px, ts, ld4(c_sh + 4 * px), ld2(c_cocg + 2 * px), ld2(c_aosky + 2 * px), ld(c_luma + px),
                      o_sh, o_cocg, o_util, o_aosky);
}

// Spatial3x3Initial and the temporal pass in one kernel: the temporal pass
// reads the pre-filtered planes only at its own texel, so each thread filters
// its texel and goes on with the result, rounded as the planes would store
// it. The pre-filtered planes are still written (kWritePre) for callers that
// read them. Not the default (vpt_tuning.fused_prefilter): at 1920x1080 it
// measured 0.358 ms against 0.318 ms for the two launches, the pre-filter's
// 9 taps running at the temporal kernel's register budget (64 per thread, 4
// blocks per SM) instead of its own (48).
template <typename S, bool kScaled, bool kWritePre>
__global__ void __launch_bounds__(256, 4) k_pre_temporal(CamView cam, int W, int H, int Wf, int Hf, TemporalArgs a,
                                                      const S* t, const uint8_t* face, const uint8_t* block,
                                                      const S* prev_t, const uint8_t* prev_face,
                                                      const uint8_t* prev_block, const S* g_sh, const S* g_cocg,
                                                      const S* g_luma, const S* g_aosky, S* c_sh, S* c_cocg,
                                                      S* c_luma, S* c_aosky, const S* p_sh, const S* p_cocg,
                                                      const S* p_util, const S* p_aosky, S* o_sh, S* o_cocg,
                                                      S* o_util, S* o_aosky) {
    pdl_enter();
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const size_t px = (size_t)j * W + i;
    const v2 uv = texcoord(i, j, W, H);
    const v4 bp = position_fetch(cam, T, i, j, uv);
    float psh[4], pcc[2], pao[2], pl;
    pre_filter_texel<S>(cam, W, H, T, face, g_sh, g_cocg, g_luma, g_aosky, i, j, uv, bp, psh, pcc, pao, &pl);
    if (kWritePre) {
        st4(c_sh + 4 * px, psh[0], psh[1], psh[2], psh[3]);
        st2(c_cocg + 2 * px, pcc[0], pcc[1]);
        st2(c_aosky + 2 * px, pao[0], pao[1]);
        st(c_luma + px, pl);
    }
    const S* q = nullptr;
    temporal_texel<S, kScaled>(
        cam, W, H, Wf, Hf, a, face, block, prev_t, prev_face, prev_block, i, j, uv, bp,
        make_float4(as_stored(psh[0], q), as_stored(psh[1], q), as_stored(psh[2], q), as_stored(psh[3], q)),
        make_float2(as_stored(pcc[0], q), as_stored(pcc[1], q)), make_float2(as_stored(pao[0], q), as_stored(pao[1], q)),
        as_stored(pl, q), p_sh, p_cocg, p_util, p_aosky, o_sh, o_cocg, o_util, o_aosky);
}

// SVGF/VarianceEstimate.glsl main (:73-193) with DO_SPATIAL and
// AGGRESSIVE_DISOCCLUSION_HANDLING on. Only the hit distance of the taps'
// reconstructed positions is used (the depth weight), so no ray is rebuilt.
//
// A texel with fewer than 12 accumulated frames takes the 81-tap estimate,
// every other one the temporal moments. Once a history has grown, the young
// texels are the few the camera's motion disoccluded, spread over many warps,
// each of which would run the 81-tap loop for a lane or two; so every thread
// first finishes its texel if it is old, and the block's young texels are
// then listed in shared memory and estimated by consecutive threads (the
// same per-texel arithmetic, only the thread that runs it changes).
// kYoung: the texel's history is younger than 12 frames (the caller tested it).
// The 81-tap branch's texel fetches: depth, face, second moment, SH, CoCg
// and the SH's luminance at an in-image texel (si, sj), from the planes or
// from a shared-memory tile of the block's 9x9 neighbourhoods (kVarHalo = 4
// around the 32 x 8 block, three float4 per texel: SH; CoCg, moment,
// luminance; depth, face).
template <typename S>
struct VarGlobal {
    int W;
    const S* t;
    const uint8_t* face;
    const S *sh, *cocg, *util;
    __device__ __forceinline__ void tap(int si, int sj, float* sd, int* sf, float* smom, float4* s4, float2* s2,
                                        float* sl) const {
        const size_t q = (size_t)sj * W + si;
        *sd = ld(t + q);
        *sf = __ldg(face + q);
        *smom = ld(util + 4 * q + 1);
        *s4 = ld4(sh + 4 * q);
        *s2 = ld2(cocg + 2 * q);
        const float ssh[4] = {s4->x, s4->y, s4->z, s4->w};
        *sl = sh_to_y(ssh);
    }
};
constexpr int kVarHalo = 4, kVarTW = 32 + 2 * kVarHalo, kVarTH = 8 + 2 * kVarHalo, kVarN = kVarTW * kVarTH;
struct VarTile {
    const float4* T;   // 3 * kVarN
    int tx0, ty0;
    __device__ __forceinline__ void tap(int si, int sj, float* sd, int* sf, float* smom, float4* s4, float2* s2,
                                        float* sl) const {
        const int k = (sj - ty0) * kVarTW + (si - tx0);
        *s4 = T[k];
        const float4 b = T[kVarN + k];
        const float2 c = *reinterpret_cast<const float2*>(T + 2 * kVarN + k);
        *s2 = make_float2(b.x, b.y);
        *smom = b.z;
        *sl = b.w;
        *sd = c.x;
        *sf = __float_as_int(c.y);
    }
};

template <typename S, bool kYoung, class VF = VarGlobal<S>>
__device__ __forceinline__ void variance_texel(int W, int H, int i, int j, const S* t, const uint8_t* face,
                                               const S* i_sh, const S* i_cocg, const S* i_util, S* o_sh, S* o_cocg,
                                               S* o_var, const VF* vf = nullptr) {
    const float thresh = 4.0f + 4.0f + 4.0f;
    const size_t px = (size_t)j * W + i;
    const float4 bsh = ld4(i_sh + 4 * px);
    const float2 bcc = ld2(i_cocg + 2 * px);
    const float bshv[4] = {bsh.x, bsh.y, bsh.z, bsh.w};
    const float bl = sh_to_y(bshv);
    const float4 bu = ld4(i_util + 4 * px);
    const float acc = bu.x;
    const float bm = bu.y;
    float osh[4], occ[2], var;
    if (kYoung) {   // acc < thresh
        const float bd = ld(t + px);
        const int bf = __ldg(face + px);
        // normal weight pow(max(dot(n, n'), 0), 16) for a clamped dot of 0, 1, 3
        const float nw3 = dpow(3.0f, 16.0f);
        // (tw, tw2), (tm, tl), SH and CoCg sums as packed pairs
        float2 tww = make_float2(0.0f, 0.0f), tml = make_float2(0.0f, 0.0f);
        float2 tsh01 = make_float2(0.0f, 0.0f), tsh23 = make_float2(0.0f, 0.0f), tcc = make_float2(0.0f, 0.0f);
        for (int x = -4; x <= 4; x++) {
            const int si = i + x;
            if (si < 0 || si >= W) continue;
#pragma unroll 3
            for (int y = -4; y <= 4; y++) {
                const int sj = j + y;
                if (sj < 0 || sj >= H) continue;
                float sd, smom, sl;
                int sf;
                float4 s4;
                float2 s2;
                vf->tap(si, sj, &sd, &sf, &smom, &s4, &s2, &sl);
                const int fc = face_cos(bf, sf);
                const float nw = fc == 0 ? 0.0f : (fc == 1 ? 1.0f : nw3);
                const float lw = div5(fabsf(sl - bl));   // / phi, phi = 5
                const float2 e = dexp_pair_np(-fabsf(sd - bd), -lw);
                const float dw = e.x * e.x;   // pow(e, 2) for e in [0, 1]
                float wgt = (e.y * nw) * dw;
                float wgt2 = wgt;
                wgt = fmaxf(wgt, 0.000000015f);
                wgt2 = fmaxf(wgt2, 0.0000000015f);
                tww = padd(tww, make_float2(wgt, wgt2));
                tml = pacc(tml, make_float2(smom, sl), wgt2);
                tsh01 = pacc(tsh01, make_float2(s4.x, s4.y), wgt);
                tsh23 = pacc(tsh23, make_float2(s4.z, s4.w), wgt);
                tcc = pacc(tcc, s2, wgt);
            }
        }
        const float tw = tww.x, tw2 = tww.y;
        float tm = tml.x, tl = tml.y;
        osh[0] = tsh01.x; osh[1] = tsh01.y; osh[2] = tsh23.x; osh[3] = tsh23.y;
        occ[0] = tcc.x;
        occ[1] = tcc.y;
        if (tw > 0.0f) {
            tm /= tw2;
            tl /= tw2;
            occ[0] /= tw;
            occ[1] /= tw;
            for (int c = 0; c < 4; c++) osh[c] /= tw;
        }
        const float al = tl * tl;
        var = tm - al;
        var *= 3.0f;
    } else {
        for (int c = 0; c < 4; c++) osh[c] = bshv[c];
        occ[0] = bcc.x;
        occ[1] = bcc.y;
        var = bm - bl * bl;
    }
    var *= thresh / acc;
    st4(o_sh + 4 * px, clampf(osh[0], -100.0f, 100.0f), clampf(osh[1], -100.0f, 100.0f),
        clampf(osh[2], -100.0f, 100.0f), clampf(osh[3], -100.0f, 100.0f));
    st2(o_cocg + 2 * px, clampf(occ[0], -10.0f, 100.0f), clampf(occ[1], -10.0f, 100.0f));
    st(o_var + px, clampf(var, -1.0f, 50.0f));
}

template <typename S>
__global__ void __launch_bounds__(256) k_variance(int W, int H, const S* t, const uint8_t* face, const S* i_sh,
                                                  const S* i_cocg, const S* i_util, S* o_sh, S* o_cocg, S* o_var) {
    pdl_enter();
    __shared__ uint32_t s_young[256];   // young texels of the block: i | j << 16
    __shared__ int s_n;
    __shared__ float4 s_vt[3 * kVarN];
    if (threadIdx.x == 0 && threadIdx.y == 0) s_n = 0;
    __syncthreads();
    int i, j;
    const bool in = pixel_of(W, H, &i, &j);
    bool young = false;
    if (in) {
        young = ld4(i_util + 4 * ((size_t)j * W + i)).x < 4.0f + 4.0f + 4.0f;
        if (!young) variance_texel<S, false>(W, H, i, j, t, face, i_sh, i_cocg, i_util, o_sh, o_cocg, o_var);
    }
    const unsigned m = __ballot_sync(0xffffffffu, young);
    const int lane = threadIdx.x & 31;   // blocks are 32 x 8: a warp is one row of the block
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&s_n, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (young) s_young[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i | ((uint32_t)j << 16);
    __syncthreads();
    const int k = threadIdx.y * blockDim.x + threadIdx.x;
    const int n = s_n;
    const int tx0 = (int)blockIdx.x * 32 - kVarHalo, ty0 = (int)blockIdx.y * 8 - kVarHalo;
    // A block with a warp's worth of young texels or more (every block while
    // the history is young) stages their neighbourhoods in shared memory
    // once: 640 texels instead of 81 gathers per young texel, the luminance
    // computed once per texel (uniform per block).
    if (n >= 32) {
        for (int q = k; q < kVarN; q += 256) {
            const int ly = q / kVarTW, lx = q - ly * kVarTW;
            const int si = tx0 + lx, sj = ty0 + ly;
            float4 A = make_float4(0.0f, 0.0f, 0.0f, 0.0f), B = A, Cc = A;
            if (si >= 0 && si < W && sj >= 0 && sj < H) {   // texels outside the image are never read
                float sd, smom, sl;
                int sf;
                float4 s4;
                float2 s2;
                const VarGlobal<S> g{W, t, face, i_sh, i_cocg, i_util};
                g.tap(si, sj, &sd, &sf, &smom, &s4, &s2, &sl);
                A = s4;
                B = make_float4(s2.x, s2.y, smom, sl);
                Cc = make_float4(sd, __int_as_float(sf), 0.0f, 0.0f);
            }
            s_vt[q] = A;
            s_vt[kVarN + q] = B;
            s_vt[2 * kVarN + q] = Cc;
        }
        __syncthreads();
        if (k < n) {
            const uint32_t q = s_young[k];
            const VarTile vt{s_vt, tx0, ty0};
            variance_texel<S, true, VarTile>(W, H, (int)(q & 0xffffu), (int)(q >> 16), t, face, i_sh, i_cocg, i_util,
                                             o_sh, o_cocg, o_var, &vt);
        }
    } else if (k < n) {
        const uint32_t q = s_young[k];
        const VarGlobal<S> g{W, t, face, i_sh, i_cocg, i_util};
        variance_texel<S, true>(W, H, (int)(q & 0xffffu), (int)(q >> 16), t, face, i_sh, i_cocg, i_util, o_sh,
                                o_cocg, o_var, &g);
    }
}

// The texel fetches of one a-trous tap at texture coordinate sc: depth
// (bilinear, on the G-buffer's own grid), nearest face, and the bilinear SH,
// CoCg, variance and AO/sky of the filter's input planes. Gathered from
// global memory (each tap's wrapped footprint is a valid address, so every
// load of the unrolled taps can be in flight together).
template <typename S, bool kScaled>
struct AtrousGlobal {
    int W, H, Wf, Hf;
    const S* tf;
    const uint8_t* ff;
    const S *sh, *cocg, *var, *ao;
    __device__ __forceinline__ float var_at(int si, int sj) const { return ld(var + (size_t)sj * W + si); }
    __device__ __forceinline__ void tap(v2 sc, bool need_ao, float* sd, int* sface, float4* s4, float2* s2,
                                        float* sv, float2* sao) const {
        const Plane8 F{ff, Wf, Hf};
        const Bilin fp = bilin(sc, W, H);
        const Bilin fq = kScaled ? bilin(sc, Wf, Hf) : fp;
        *sd = bl1s(tf, fq);
        *sface = F.nearest(sc);
        *s4 = bl4(sh, fp);
        *s2 = bl2(cocg, fp);
        *sv = bl1s(var, fp);
        *sao = need_ao ? bl2(ao, fp) : make_float2(0.0f, 0.0f);
    }
};

// The same fetches from a shared-memory tile of the block's neighbourhood
// (kHalo texels around the 32 x kRows block; the G-buffer on the planes' grid),
// three float4 per texel: (SH), (CoCg, variance, AO), (sky, depth, face).
// The footprint and weights are computed with bilin's operations, so a tap
// blends the same values with the same weights; a tap whose footprint leaves
// the tile takes the global fetch.
template <typename S, int kHalo, int kRows>
struct AtrousTile {
    static constexpr int TW = 32 + 2 * kHalo, TH = kRows + 2 * kHalo;
    const float4* A;
    const float4* B;
    const float4* C;
    int tx0, ty0;
    AtrousGlobal<S, false> g;
    __device__ __forceinline__ float var_at(int si, int sj) const { return B[(sj - ty0) * TW + (si - tx0)].z; }
    __device__ __forceinline__ void tap(v2 sc, bool need_ao, float* sd, int* sface, float4* s4, float2* s2,
                                        float* sv, float2* sao) const {
        const float x = sc.x * (float)g.W - 0.5f;
        const float y = sc.y * (float)g.H - 0.5f;
        const float x0 = floorf(x), y0 = floorf(y);
        Bilin b;
        b.ax = x - x0;
        b.ay = y - y0;
        b.bx = 1.0f - b.ax;
        b.by = 1.0f - b.ay;
        const int li = f2i(x0) - tx0, lj = f2i(y0) - ty0;
        const int ni = f2i_floor(sc.x * (float)g.W) - tx0, nj = f2i_floor(sc.y * (float)g.H) - ty0;
        if (!((unsigned)li < (unsigned)(TW - 1) && (unsigned)lj < (unsigned)(TH - 1) && (unsigned)ni < (unsigned)TW &&
              (unsigned)nj < (unsigned)TH)) {
            g.tap(sc, need_ao, sd, sface, s4, s2, sv, sao);
            return;
        }
        const int k00 = lj * TW + li, k10 = k00 + 1, k01 = k00 + TW, k11 = k01 + 1;
        const float4 a00 = A[k00], a10 = A[k10], a01 = A[k01], a11 = A[k11];
        const float4 b00 = B[k00], b10 = B[k10], b01 = B[k01], b11 = B[k11];
        const float2 c00 = *reinterpret_cast<const float2*>(C + k00), c10 = *reinterpret_cast<const float2*>(C + k10);
        const float2 c01 = *reinterpret_cast<const float2*>(C + k01), c11 = *reinterpret_cast<const float2*>(C + k11);
        // the tile's float4 texels blend as packed pairs: (SH x, y), (SH z, w), (CoCg), (variance, AO), (sky, depth)
        const float2 sxy = blend2(b, xy(a00), xy(a10), xy(a01), xy(a11));
        const float2 szw = blend2(b, zw(a00), zw(a10), zw(a01), zw(a11));
        *s2 = blend2(b, xy(b00), xy(b10), xy(b01), xy(b11));
        const float2 va = blend2(b, zw(b00), zw(b10), zw(b01), zw(b11));
        const float2 sk = blend2(b, c00, c10, c01, c11);
        *s4 = make_float4(sxy.x, sxy.y, szw.x, szw.y);
        *sv = va.x;
        *sd = sk.y;
        *sface = __float_as_int(C[nj * TW + ni].z);
        *sao = need_ao ? make_float2(va.y, sk.x) : make_float2(0.0f, 0.0f);
    }
    static __device__ __forceinline__ float2 xy(float4 v) { return make_float2(v.x, v.y); }
    static __device__ __forceinline__ float2 zw(float4 v) { return make_float2(v.z, v.w); }
};

// SVGF/SpatialFilter.glsl main (:175-355), 3x3 taps (u_LargeKernel off), for
// texel (i, j). A tap contributes only when (BaseDepth < 0) == (DepthDiff <
// 0), i.e. when the centre is not sky (DepthDiff = abs(...) >= 0); sky
// centres keep their own values, so their tap loop is skipped. t / face: the
// G-buffer on the GI grid (the centre); the taps read the G-buffer on its own
// grid through `fe`.
// The per-texel state of atrous_texels.
struct AtrousPix {
    size_t px;
    float bd;
    float2 bao;
    v2 uv;
    float jo, bl, phi;
    int bf;
    bool in, act, strong;
    float tsh[4], tcc[2], tw, tvar, tao[2], taow;
};

// kP texels (i, j[p]) per thread, their taps issued together tap by tap (the
// fetches of every texel of a tap before any of their weights), each texel's
// arithmetic that of one texel alone. The kernels use kP = 1: two texels a
// thread measured slower at every register budget (0.78-0.88 against 0.65 ms
// per frame for the five iterations); this form of the one-texel code keeps
// its state in registers without spills (0.667 -> 0.648 ms).
template <typename S, class Fetch, int kP>
__device__ __forceinline__ void atrous_texels(int W, int H, const AtrousArgs& a, int i, const int* jv, const bool* inv,
                                              const S* t, const uint8_t* face, const S* t_util, const S* i_sh,
                                              const S* i_cocg, const S* i_aosky, S* o_sh, S* o_cocg, S* o_var,
                                              S* o_aosky, const Fetch& fe) {
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float aw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    const float gauss[2] = {0.60283f, 0.198585f};
    const int step = a.step;
    const bool filter_ao = step <= 4;
    const bool filter_sky = (step <= 6) || filter_ao;
    AtrousPix P[kP];
    bool any = false;
#pragma unroll
    for (int p = 0; p < kP; p++) {
        AtrousPix& q = P[p];
        const int j = jv[p];
        q.in = inv[p];
        q.act = false;
        if (!q.in) continue;
        q.px = (size_t)j * W + i;
        q.bd = ld(t + q.px);
        const float4 bsh = ld4(i_sh + 4 * q.px);
        const float2 bcc = ld2(i_cocg + 2 * q.px);
        q.bao = ld2(i_aosky + 2 * q.px);
        // GaussianVariance (:94-129)
        float bvar = 0.0f, vsum = 0.0f, tk = 0.0f;
#pragma unroll
        for (int x = -1; x <= 1; x++) {
#pragma unroll
            for (int y = -1; y <= 1; y++) {
                const int si = i + x, sj = j + y;
                if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
                const float kv = gauss[x < 0 ? -x : x] * gauss[y < 0 ? -y : y];
                const float v = fe.var_at(si, sj);
                if (x == 0 && y == 0) bvar = v;
                vsum += v * kv;
                tk += kv;
            }
        }
        q.tsh[0] = bsh.x; q.tsh[1] = bsh.y; q.tsh[2] = bsh.z; q.tsh[3] = bsh.w;
        q.tcc[0] = bcc.x; q.tcc[1] = bcc.y;
        q.tw = 1.0f; q.tvar = bvar; q.tao[0] = q.bao.x; q.tao[1] = q.bao.y; q.taow = 1.0f;
        if (q.bd < 0.0f) continue;
        q.act = true;
        any = true;
        q.uv = texcoord(i, j, W, H);
        // GradientNoise (:160-165)
        const float gx = ((float)i + 0.5f) + a.tmod500, gy = ((float)j + 0.5f) + a.tmod500;
        const float noise = fract(52.9829189f * fract(0.06711056f * gx + 0.00583715f * gy));
        const int jit = f2i((noise - 0.5f) * ((float)step * 0.8f));
        q.bf = __ldg(face + q.px);
        const float bshv[4] = {bsh.x, bsh.y, bsh.z, bsh.w};
        q.bl = sh_to_y(bshv);
        const float vest = vsum / fmaxf(tk, 0.01f);
        const float acc_frames = ld(t_util + 4 * q.px);
        q.strong = acc_frames <= 8.0f && step <= 8;
        float curve = 0.0f;
        if (vest < 0.01f) curve = 128.0f;
        else if (vest < 0.025f) curve = 112.0f;
        else if (vest < 0.05f) curve = 96.0f;
        else if (vest < 0.075f) curve = 84.0f;
        else if (vest < 0.1f) curve = 70.0f;
        float tweaked = vest;
        if (vest < 0.1f) {   // TweakVariance (:167-173)
            const float fe_ = clampf(vest, 0.0f, 1.0f);
            const float tt = 1.0f - fe_;
            tweaked = fe_ * dpow(tt, curve + 6.0f);
        }
        float phi = sqrtf(fmaxf(0.0f, 0.000001f + tweaked));
        q.phi = phi / a.phi_bias;
        q.jo = (float)jit * 0.5f;
    }
    if (any) {
        // rolled: the eight unrolled taps overflow the instruction cache
#pragma unroll 1
        for (int x = -1; x <= 1; x++) {
#pragma unroll 1
            for (int y = -1; y <= 1; y++) {
                if (x == 0 && y == 0) continue;
                v2 sc[kP];
                float sd[kP], sv[kP];
                int sface[kP];
                float4 s4[kP];
                float2 s2[kP], sao[kP];
#pragma unroll
                for (int p = 0; p < kP; p++) {
                    if (!P[p].act) continue;
                    const float ox = ((float)x * (float)step) * a.add_scale + P[p].jo;
                    const float oy = ((float)y * (float)step) * a.add_scale + P[p].jo;
                    sc[p] = mk2(P[p].uv.x + ox * texel_x, P[p].uv.y + oy * texel_y);
                    fe.tap(sc[p], filter_sky || filter_ao, &sd[p], &sface[p], &s4[p], &s2[p], &sv[p], &sao[p]);
                }
#pragma unroll
                for (int p = 0; p < kP; p++) {
                    AtrousPix& q = P[p];
                    if (!q.act) continue;
                    if (!(sc[p].x > 0.0f && sc[p].x < 1.0f && sc[p].y > 0.0f && sc[p].y < 1.0f)) continue;
                    const float dd = fabsf(sd[p] - q.bd);
                    const float ssh[4] = {s4[p].x, s4[p].y, s4[p].z, s4[p].w};
                    const float sl = sh_to_y(ssh);
                    // clamp(pow(max(dot(n, n'), 0), 32), 0.001, 1) for a clamped dot of 0, 1 or 3
                    const float nw = face_cos(q.bf, sface[p]) > 0 ? 1.0f : 0.001f;
                    // young histories: no luminance weight (nor its division and exponential); otherwise the
                    // depth and luminance exponentials as one packed polynomial
                    const float dn = -fmaxf(dd, 0.00001f);
                    float de, le = 0.0f;
                    if (q.strong) {
                        de = dexp(dn);
                    } else {
                        const float2 e = dexp_pair_np(dn, -(fabsf(sl - q.bl) / q.phi));   // both <= 0
                        de = e.x;
                        le = e.y;
                    }
                    const float dw = clampf(de * de, 0.0001f, 1.0f);   // pow(e, 2) for e in [0, 1)
                    float wgt = q.strong ? nw * dw : (le * nw) * dw;
                    wgt = clampf(wgt, 0.001f, 1.0f);
                    const float xw = x == 0 ? aw[0] : aw[1], yw = y == 0 ? aw[0] : aw[1];
                    wgt = (xw * yw) * wgt;
                    wgt = fmaxf(wgt, 0.00000001f);
                    q.tsh[0] += ssh[0] * wgt;
                    q.tsh[1] += ssh[1] * wgt;
                    q.tsh[2] += ssh[2] * wgt;
                    q.tsh[3] += ssh[3] * wgt;
                    q.tcc[0] += s2[p].x * wgt;
                    q.tcc[1] += s2[p].y * wgt;
                    q.tvar += (wgt * wgt) * sv[p];
                    q.tw += wgt;
                    if (filter_sky || filter_ao) {
                        const float awt = clampf(((xw * yw) * nw) * dw, 0.000001f, 1.0f);
                        q.tao[0] += sao[p].x * awt;
                        q.tao[1] += sao[p].y * awt;
                        q.taow += awt;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int p = 0; p < kP; p++) {
        AtrousPix& q = P[p];
        if (!q.in) continue;
        for (int c = 0; c < 4; c++) q.tsh[c] /= q.tw;
        q.tcc[0] /= q.tw;
        q.tcc[1] /= q.tw;
        q.tvar /= (q.tw * q.tw);
        q.tao[0] /= q.taow;
        q.tao[1] /= q.taow;
        if (!filter_ao) q.tao[0] = q.bao.x;
        st4(o_sh + 4 * q.px, clampf(q.tsh[0], -100.0f, 100.0f), clampf(q.tsh[1], -100.0f, 100.0f),
            clampf(q.tsh[2], -100.0f, 100.0f), clampf(q.tsh[3], -100.0f, 100.0f));
        st2(o_cocg + 2 * q.px, clampf(q.tcc[0], -10.0f, 100.0f), clampf(q.tcc[1], -10.0f, 100.0f));
        st(o_var + q.px, clampf(q.tvar, -1.0f, 50.0f));
        st2(o_aosky + 2 * q.px, clampf(q.tao[0], 0.0f, 1.0f), clampf(q.tao[1], 0.0f, 1.0f));
    }
}

// One texel (i, j).
template <typename S, class Fetch>
__device__ __forceinline__ void atrous_texel(int W, int H, const AtrousArgs& a, int i, int j, const S* t,
                                             const uint8_t* face, const S* t_util, const S* i_sh, const S* i_cocg,
                                             const S* i_aosky, S* o_sh, S* o_cocg, S* o_var, S* o_aosky,
                                             const Fetch& fe) {
    const int jv[1] = {j};
    const bool inv[1] = {true};
    atrous_texels<S, Fetch, 1>(W, H, a, i, jv, inv, t, face, t_util, i_sh, i_cocg, i_aosky, o_sh, o_cocg, o_var,
                               o_aosky, fe);
}

// One a-trous iteration gathering its taps from the planes (kScaled when the
// G-buffer's grid Wf x Hf is finer than the GI grid W x H).
template <typename S, bool kScaled>
__global__ void __launch_bounds__(256, 4) k_atrous(int W, int H, int Wf, int Hf, AtrousArgs a, const S* t,
                                                const uint8_t* face, const S* tf, const uint8_t* ff,
                                                const S* t_util, const S* i_sh, const S* i_cocg, const S* i_var,
                                                const S* i_aosky, S* o_sh, S* o_cocg, S* o_var, S* o_aosky) {
    pdl_enter();
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const AtrousGlobal<S, kScaled> fe{W, H, Wf, Hf, tf, ff, i_sh, i_cocg, i_var, i_aosky};
    atrous_texel<S>(W, H, a, i, j, t, face, t_util, i_sh, i_cocg, i_aosky, o_sh, o_cocg, o_var, o_aosky, fe);
}

// One a-trous iteration of a small step (every tap's footprint within kHalo
// texels of the centre) by 32 x kRows blocks: a block whose neighbourhood
// lies inside the image first stages it in shared memory (dynamic, 48 bytes
// per texel) with coalesced loads (each texel read once per block instead of
// once per tap that touches it, fp16 planes converted once), then every tap
// reads the tile. Blocks at the image border gather from the planes as
// k_atrous does.
template <typename S, int kHalo, int kRows>
__global__ void __launch_bounds__(32 * kRows, 1024 / (32 * kRows)) k_atrous_tile(
    int W, int H, AtrousArgs a, const S* t, const uint8_t* face, const S* tf, const uint8_t* ff, const S* t_util,
    const S* i_sh, const S* i_cocg, const S* i_var, const S* i_aosky, S* o_sh, S* o_cocg, S* o_var, S* o_aosky) {
    using Tile = AtrousTile<S, kHalo, kRows>;
    constexpr int TW = Tile::TW, TH = Tile::TH, N = TW * TH, kThreads = 32 * kRows;
    extern __shared__ float4 s_tile[];   // 3 * N
    pdl_enter();
    const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * kRows + threadIdx.y;
    const bool in = i < W && j < H;
    const int tx0 = (int)blockIdx.x * 32 - kHalo, ty0 = (int)blockIdx.y * kRows - kHalo;
    const AtrousGlobal<S, false> g{W, H, W, H, tf, ff, i_sh, i_cocg, i_var, i_aosky};
    if (!(tx0 >= 0 && ty0 >= 0 && tx0 + TW <= W && ty0 + TH <= H)) {   // border block (uniform)
        if (in) atrous_texel<S>(W, H, a, i, j, t, face, t_util, i_sh, i_cocg, i_aosky, o_sh, o_cocg, o_var, o_aosky, g);
        return;
    }
    for (int k = threadIdx.y * 32 + threadIdx.x; k < N; k += kThreads) {
        const int ly = k / TW, lx = k - ly * TW;
        const size_t q = (size_t)(ty0 + ly) * W + (tx0 + lx);
        const float4 sh = ld4(i_sh + 4 * q);
        const float2 cc = ld2(i_cocg + 2 * q), ao = ld2(i_aosky + 2 * q);
        const float v = ld(i_var + q), d = ld(tf + q);
        const int f = __ldg(ff + q);
        s_tile[k] = sh;
        s_tile[N + k] = make_float4(cc.x, cc.y, v, ao.x);
        s_tile[2 * N + k] = make_float4(ao.y, d, __int_as_float(f), 0.0f);
    }
    __syncthreads();
    if (!in) return;
    const Tile fe{s_tile, s_tile + N, s_tile + 2 * N, tx0, ty0, g};
    atrous_texel<S>(W, H, a, i, j, t, face, t_util, i_sh, i_cocg, i_aosky, o_sh, o_cocg, o_var, o_aosky, fe);
}

inline dim3 grid2(int W, int H) { return dim3((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8)); }
const dim3 kBlock2(32, 8);

template <typename S>
cudaError_t launch_all_spatial_initial(const CamView& cam, int W, int H, const void* t, const uint8_t* face, GIIn in,
                                       GIOut out, cudaStream_t s) {
    pdl_launch(k_spatial_initial<S>, grid2(W, H), kBlock2, 0, s, cam, W, H, (const S*)t, face, (const S*)in.sh,
               (const S*)in.cocg, (const S*)in.luma, (const S*)in.aosky, (S*)out.sh, (S*)out.cocg, (S*)out.luma,
               (S*)out.aosky);
    return cudaGetLastError();
}

template <typename S, bool kScaled>
cudaError_t launch_temporal(const CamView& cam, int W, int H, int Wf, int Hf, const TemporalArgs& a, const void* t,
                            const uint8_t* face, const uint8_t* block, const void* prev_t, const uint8_t* prev_face,
                            const uint8_t* prev_block, GIIn cur, HistIO prev, HistIO out, cudaStream_t s) {
    pdl_launch(k_temporal<S, kScaled>, grid2(W, H), kBlock2, 0, s,
        cam, W, H, Wf, Hf, a, (const S*)t, face, block, (const S*)prev_t, prev_face, prev_block, (const S*)cur.sh,
        (const S*)cur.cocg, (const S*)cur.luma, (const S*)cur.aosky, (const S*)prev.sh, (const S*)prev.cocg,
        (const S*)prev.util, (const S*)prev.aosky, (S*)out.sh, (S*)out.cocg, (S*)out.util, (S*)out.aosky);
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_temporal_gather(const CamView& cam, int W, int H, const TemporalArgs& a, const void* t,
                                   const uint8_t* face, const uint8_t* block, const void* prev_t,
                                   const uint8_t* prev_face, const uint8_t* prev_block, HistIO prev, void* sums,
                                   cudaStream_t s) {
    pdl_launch(k_temporal_gather<S>, grid2(W, H), kBlock2, 0, s, cam, W, H, a, (const S*)t, face, block,
               (const S*)prev_t, prev_face, prev_block, (const S*)prev.sh, (const S*)prev.cocg, (const S*)prev.util,
               (const S*)prev.aosky, (float4*)sums);
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_temporal_blend(int W, int H, const TemporalArgs& a, const void* sums, GIIn cur, HistIO out,
                                  cudaStream_t s) {
    pdl_launch(k_temporal_blend<S>, grid2(W, H), kBlock2, 0, s, W, H, a, (const float4*)sums, (const S*)cur.sh,
               (const S*)cur.cocg, (const S*)cur.luma, (const S*)cur.aosky, (S*)out.sh, (S*)out.cocg, (S*)out.util,
               (S*)out.aosky);
    return cudaGetLastError();
}

template <typename S, bool kScaled>
cudaError_t launch_pre_temporal(const CamView& cam, int W, int H, int Wf, int Hf, const TemporalArgs& a, const void* t,
                                const uint8_t* face, const uint8_t* block, const void* prev_t,
                                const uint8_t* prev_face, const uint8_t* prev_block, GIIn gi, GIOut pre, HistIO prev,
                                HistIO out, cudaStream_t s) {
    pdl_launch(k_pre_temporal<S, kScaled, true>, grid2(W, H), kBlock2, 0, s,
        cam, W, H, Wf, Hf, a, (const S*)t, face, block, (const S*)prev_t, prev_face, prev_block, (const S*)gi.sh,
        (const S*)gi.cocg, (const S*)gi.luma, (const S*)gi.aosky, (S*)pre.sh, (S*)pre.cocg, (S*)pre.luma,
        (S*)pre.aosky, (const S*)prev.sh, (const S*)prev.cocg, (const S*)prev.util, (const S*)prev.aosky, (S*)out.sh,
        (S*)out.cocg, (S*)out.util, (S*)out.aosky);
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_variance(int W, int H, const void* t, const uint8_t* face, HistIO in, FiltIO out, cudaStream_t s) {
    pdl_launch(k_variance<S>, grid2(W, H), kBlock2, 0, s, W, H, (const S*)t, face, (const S*)in.sh, (const S*)in.cocg,
               (const S*)in.util, (S*)out.sh, (S*)out.cocg, (S*)out.variance);
    return cudaGetLastError();
}

// The halo a shared-memory tile needs for an iteration's taps: |offset| <=
// step * add_scale + |jitter| / 2, the jitter f2i((noise - 0.5) * 0.8 step)
// at most 0.4 step in magnitude; plus the bilinear footprint's second texel
// and a margin for the rounding of the texture coordinates.
inline int atrous_tile_need(const AtrousArgs& a) {
    if (!(a.add_scale >= 0.0f) || a.step > 64) return 1 << 20;
    const float jit = floorf(0.4f * (float)a.step);
    return (int)floorf((float)a.step * a.add_scale + 0.5f * jit + 0.01f) + 1;
}

template <typename S, int kHalo, int kRows>
cudaError_t launch_atrous_tile(int W, int H, const AtrousArgs& a, const void* t, const uint8_t* face, const void* tf,
                               const uint8_t* ff, const void* temporal_util, FiltIO in, const void* in_aosky,
                               FiltIO out, cudaStream_t s) {
    using Tile = AtrousTile<S, kHalo, kRows>;
    const size_t smem = (size_t)3 * Tile::TW * Tile::TH * sizeof(float4);
    auto k = k_atrous_tile<S, kHalo, kRows>;
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    pdl_launch(k, dim3((unsigned)((W + 31) / 32), (unsigned)((H + kRows - 1) / kRows)), dim3(32, kRows), smem, s, W,
               H, a, (const S*)t, face, (const S*)tf, ff, (const S*)temporal_util, (const S*)in.sh,
               (const S*)in.cocg, (const S*)in.variance, (const S*)in_aosky, (S*)out.sh, (S*)out.cocg,
               (S*)out.variance, (S*)out.aosky);
    return cudaGetLastError();
}

template <typename S, bool kScaled>
cudaError_t launch_atrous(int W, int H, int Wf, int Hf, const AtrousArgs& a, const void* t, const uint8_t* face,
                          const void* tf, const uint8_t* ff, const void* temporal_util, FiltIO in,
                          const void* in_aosky, FiltIO out, cudaStream_t s) {
    if (!kScaled) {   // the steps whose neighbourhood fits a shared-memory tile
        const int need = atrous_tile_need(a);
        if (need <= 3) return launch_atrous_tile<S, 3, 8>(W, H, a, t, face, tf, ff, temporal_util, in, in_aosky, out, s);
        if (need <= 5) return launch_atrous_tile<S, 5, 8>(W, H, a, t, face, tf, ff, temporal_util, in, in_aosky, out, s);
        // step 4 (halo 11) measured slower tiled (32 x 16 blocks, two per SM: 0.670 against 0.666 ms per frame
        // for the five iterations), steps 8 and 16 need halos of 21 and 41
    }
    pdl_launch(k_atrous<S, kScaled>, grid2(W, H), kBlock2, 0, s, W, H, Wf, Hf, a, (const S*)t, face, (const S*)tf, ff,
               (const S*)temporal_util, (const S*)in.sh, (const S*)in.cocg, (const S*)in.variance,
               (const S*)in_aosky, (S*)out.sh, (S*)out.cocg, (S*)out.variance, (S*)out.aosky);
    return cudaGetLastError();
}

}  // namespace

cudaError_t svgf_spatial_initial(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                                 GIIn in, GIOut out, cudaStream_t s) {
    return fp16 ? launch_all_spatial_initial<__half>(cam, W, H, t, face, in, out, s)
                : launch_all_spatial_initial<float>(cam, W, H, t, face, in, out, s);
}

cudaError_t svgf_temporal(const CamView& cam, int W, int H, int Wf, int Hf, int fp16, const TemporalArgs& a,
                          const void* t, const uint8_t* face, const uint8_t* block,
                          const void* prev_t, const uint8_t* prev_face, const uint8_t* prev_block,
                          GIIn cur, HistIO prev, HistIO out, cudaStream_t s) {
    const bool scaled = Wf != W || Hf != H;
    if (fp16)
        return scaled ? launch_temporal<__half, true>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face,
                                                      prev_block, cur, prev, out, s)
                      : launch_temporal<__half, false>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face,
                                                       prev_block, cur, prev, out, s);
    return scaled ? launch_temporal<float, true>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face, prev_block,
                                                 cur, prev, out, s)
                  : launch_temporal<float, false>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face, prev_block,
                                                  cur, prev, out, s);
}

cudaError_t svgf_temporal_gather(const CamView& cam, int W, int H, int fp16, const TemporalArgs& a, const void* t,
                                 const uint8_t* face, const uint8_t* block, const void* prev_t,
                                 const uint8_t* prev_face, const uint8_t* prev_block, HistIO prev, void* sums,
                                 cudaStream_t s) {
    return fp16 ? launch_temporal_gather<__half>(cam, W, H, a, t, face, block, prev_t, prev_face, prev_block, prev,
                                                 sums, s)
                : launch_temporal_gather<float>(cam, W, H, a, t, face, block, prev_t, prev_face, prev_block, prev,
                                                sums, s);
}

cudaError_t svgf_temporal_blend(int W, int H, int fp16, const TemporalArgs& a, const void* sums, GIIn cur,
                                HistIO out, cudaStream_t s) {
    return fp16 ? launch_temporal_blend<__half>(W, H, a, sums, cur, out, s)
                : launch_temporal_blend<float>(W, H, a, sums, cur, out, s);
}

cudaError_t svgf_pre_temporal(const CamView& cam, int W, int H, int Wf, int Hf, int fp16, const TemporalArgs& a,
                              const void* t, const uint8_t* face, const uint8_t* block, const void* prev_t,
                              const uint8_t* prev_face, const uint8_t* prev_block, GIIn gi, GIOut pre, HistIO prev,
                              HistIO out, cudaStream_t s) {
    const bool scaled = Wf != W || Hf != H;
    if (fp16)
        return scaled ? launch_pre_temporal<__half, true>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face,
                                                          prev_block, gi, pre, prev, out, s)
                      : launch_pre_temporal<__half, false>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face,
                                                           prev_block, gi, pre, prev, out, s);
    return scaled ? launch_pre_temporal<float, true>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face,
                                                     prev_block, gi, pre, prev, out, s)
                  : launch_pre_temporal<float, false>(cam, W, H, Wf, Hf, a, t, face, block, prev_t, prev_face,
                                                      prev_block, gi, pre, prev, out, s);
}

cudaError_t svgf_variance(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                          HistIO in, FiltIO out, cudaStream_t s) {
    (void)cam;
    return fp16 ? launch_variance<__half>(W, H, t, face, in, out, s) : launch_variance<float>(W, H, t, face, in, out, s);
}

cudaError_t svgf_atrous(const CamView& cam, int W, int H, int Wf, int Hf, int fp16, const AtrousArgs& a,
                        const void* t, const uint8_t* face, const void* tf, const uint8_t* ff,
                        const void* temporal_util, FiltIO in, const void* in_aosky, FiltIO out, cudaStream_t s) {
    (void)cam;
    const bool scaled = Wf != W || Hf != H;
    if (fp16)
        return scaled ? launch_atrous<__half, true>(W, H, Wf, Hf, a, t, face, tf, ff, temporal_util, in, in_aosky, out, s)
                      : launch_atrous<__half, false>(W, H, Wf, Hf, a, t, face, tf, ff, temporal_util, in, in_aosky, out, s);
    return scaled ? launch_atrous<float, true>(W, H, Wf, Hf, a, t, face, tf, ff, temporal_util, in, in_aosky, out, s)
                  : launch_atrous<float, false>(W, H, Wf, Hf, a, t, face, tf, ff, temporal_util, in, in_aosky, out, s);
}

namespace {
// The G-buffer read at the texel centres of a GI grid Wg x Hg coarser than
// its own W x H: texture() of the depth (bilinear, REPEAT wrap) and nearest
// face and block, which is what the GI passes' GetPositionAt and normal /
// block fetches at their own texel centres return; the depth is stored in
// the storage type.
template <typename S>
__global__ void __launch_bounds__(256) k_gi_view(int W, int H, int Wg, int Hg, const S* t, const uint8_t* face,
                                                 const uint8_t* block, S* tv, uint8_t* fv, uint8_t* bv) {
    int i, j;
    if (!pixel_of(Wg, Hg, &i, &j)) return;
    const v2 uv = texcoord(i, j, Wg, Hg);
    const Bilin fp = bilin(uv, W, H);
    const Plane8 F{face, W, H}, B{block, W, H};
    const size_t q = (size_t)j * Wg + i;
    st(tv + q, bl1(t, fp));
    fv[q] = (uint8_t)F.nearest(uv);
    bv[q] = (uint8_t)B.nearest(uv);
}
}  // namespace

cudaError_t gi_view(int W, int H, int Wg, int Hg, int fp16, const void* t, const uint8_t* face, const uint8_t* block,
                    void* tv, uint8_t* fv, uint8_t* bv, cudaStream_t s) {
    if (fp16)
        k_gi_view<__half><<<grid2(Wg, Hg), kBlock2, 0, s>>>(W, H, Wg, Hg, (const __half*)t, face, block, (__half*)tv,
                                                            fv, bv);
    else
        k_gi_view<float><<<grid2(Wg, Hg), kBlock2, 0, s>>>(W, H, Wg, Hg, (const float*)t, face, block, (float*)tv, fv,
                                                           bv);
    return cudaGetLastError();
}

}  // namespace vpt
