// SVGF denoiser kernels: pre-temporal 3x3 spatial pass, temporal
// reprojection/accumulation, variance estimate and the a-trous iterations
// (Core/Pipeline.cpp:2284-2615). One thread per pixel; neighbourhood taps at
// integer offsets are direct fetches (what texture() returns at a texel
// centre), taps at fractional coordinates are fp32 bilinear with REPEAT wrap.
// Planes are bandwidth-bound streams read through the L1/L2 caches.
#include "kernels.cuh"

namespace vpt {

namespace {

__device__ __forceinline__ bool pixel_of(int W, int H, int* i, int* j) {
    *i = blockIdx.x * blockDim.x + threadIdx.x;
    *j = blockIdx.y * blockDim.y + threadIdx.y;
    return *i < W && *j < H;
}

// Spatial3x3Initial.glsl main (:96-176)
template <typename S>
__global__ void __launch_bounds__(256) k_spatial_initial(CamView cam, int W, int H, const S* t, const uint8_t* face,
                                                         const S* sh, const S* cocg, const S* luma, const S* aosky,
                                                         S* o_sh, S* o_cocg, S* o_luma, S* o_aosky) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const Plane<S, 4> SH{sh, W, H};
    const Plane<S, 2> CC{cocg, W, H}, AO{aosky, W, H};
    const Plane8 F{face, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float aw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    size_t px = (size_t)j * W + i;
    v2 uv = texcoord(i, j, W, H);
    v4 bp = position_fetch(cam, T, i, j, uv);
    v3 bn = normal_from_id(F.at_in(i, j), 1.0f);
    float bsh[4], bcc[2], bao[2];
    for (int c = 0; c < 4; c++) bsh[c] = SH.at_in(i, j, c);
    for (int c = 0; c < 2; c++) { bcc[c] = CC.at_in(i, j, c); bao[c] = AO.at_in(i, j, c); }
    float bl = sh_to_y(bsh);
    float butil = ld(luma + px);
    float tsh[4] = {bsh[0], bsh[1], bsh[2], bsh[3]}, tcc[2] = {bcc[0], bcc[1]}, tao[2] = {bao[0], bao[1]};
    float tw = 1.0f, taow = 1.0f;
    const float phi = 4.0f;
    for (int x = -1; x <= 1; x++) {
        for (int y = -1; y <= 1; y++) {
            if (x == 0 && y == 0) continue;
            int si = i + x, sj = j + y;
            if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
            v2 sc = mk2(uv.x + (float)x * texel_x, uv.y + (float)y * texel_y);
            v4 sp = position_fetch(cam, T, si, sj, sc);
            v3 pd = mk3(fabsf(sp.x - bp.x), fabsf(sp.y - bp.y), fabsf(sp.z - bp.z));
            float dist_sqr = dot(pd, pd);
            if (dist_sqr < 1.0f) {
                float ssh[4], scc[2];
                for (int c = 0; c < 4; c++) ssh[c] = SH.at_in(si, sj, c);
                for (int c = 0; c < 2; c++) scc[c] = CC.at_in(si, sj, c);
                v3 sn = normal_from_id(F.at_in(si, sj), 1.0f);
                float sl = sh_to_y(ssh);
                float nw = dpow(fmaxf(dot(bn, sn), 0.0f), 16.0f);
                float lw = fabsf(sl - bl) / phi;
                float wgt = dexp(-lw - nw);
                wgt = fmaxf(wgt, 0.01f);
                wgt = (aw[abs(x)] * aw[abs(y)]) * wgt;
                wgt = fmaxf(wgt, 0.01f);
                wgt = clampf(wgt, 0.0f, 1.0f);
                for (int c = 0; c < 4; c++) tsh[c] += ssh[c] * wgt;
                for (int c = 0; c < 2; c++) tcc[c] += scc[c] * wgt;
                tw += wgt;
                for (int c = 0; c < 2; c++) tao[c] += AO.at_in(si, sj, c) * wgt;
                taow += wgt;
            }
        }
    }
    tw = fmaxf(tw, 0.01f);
    for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, tsh[c] / tw);
    for (int c = 0; c < 2; c++) st(o_cocg + px * 2 + c, tcc[c] / tw);
    float awt = fmaxf(taow, 0.01f);
    for (int c = 0; c < 2; c++) st(o_aosky + px * 2 + c, tao[c] / awt);
    st(o_luma + px, butil);
}

// SVGF/TemporalFilter.glsl main (:132-360)
template <typename S>
__global__ void __launch_bounds__(256) k_temporal(CamView cam, int W, int H, TemporalArgs a, const S* t,
                                                  const uint8_t* face, const uint8_t* block, const S* prev_t,
                                                  const uint8_t* prev_face, const uint8_t* prev_block,
                                                  const S* c_sh, const S* c_cocg, const S* c_luma, const S* c_aosky,
                                                  const S* p_sh, const S* p_cocg, const S* p_util, const S* p_aosky,
                                                  S* o_sh, S* o_cocg, S* o_util, S* o_aosky) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H}, PT{prev_t, W, H};
    const Plane8 F{face, W, H}, B{block, W, H}, PF{prev_face, W, H}, PB{prev_block, W, H};
    const Plane<S, 4> PSH{p_sh, W, H}, PU{p_util, W, H};
    const Plane<S, 2> PCC{p_cocg, W, H}, PAO{p_aosky, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float weights[5] = {3.0f / 32.0f, 3.0f / 32.0f, 9.0f / 64.0f, 3.0f / 32.0f, 3.0f / 32.0f};
    const int offx[5] = {1, 0, 0, -1, 0};
    const int offy[5] = {0, 1, 0, 0, -1};
    size_t px = (size_t)j * W + i;
    v2 uv = texcoord(i, j, W, H);
    v4 bp = position_fetch(cam, T, i, j, uv);
    v3 bn = normal_from_id(F.at_in(i, j), 1.0f);
    float bsh[4], bcc[2], bao[2];
    for (int c = 0; c < 4; c++) bsh[c] = ld(c_sh + px * 4 + c);
    for (int c = 0; c < 2; c++) { bcc[c] = ld(c_cocg + px * 2 + c); bao[c] = ld(c_aosky + px * 2 + c); }
    v4 pr = mat_mul4(a.prev_view_proj, bp.x, bp.y, bp.z, 1.0f);
    v2 rc = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
    float base_lum = ld(c_luma + px);
    int base_block = min(max((int)B.at_in(i, j), 0), 127);
    float tol = 0.75f;
    bool do_block = true, do_normal = true;
    float dp = length(sub(mk3(bp.x, bp.y, bp.z), ray_origin(cam)));
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
    float tw = 0.0f, ssh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, scc[2] = {0.0f, 0.0f}, sao[2] = {0.0f, 0.0f};
    float slum = 0.0f, sspp = 0.0f, smom = 0.0f;
    int successful = 0;
    for (int k = 0; k < 5; k++) {
        v2 sc = mk2(rc.x + ((float)offx[k] + 0.0f) * texel_x, rc.y + ((float)offy[k] + 0.0f) * texel_y);
        const float b = 0.0035f;
        if (!(sc.x < 1.0f - b && sc.x > b && sc.y < 1.0f - b && sc.y > b)) continue;
        v4 pp = position_linear(cam, PT, sc);
        v3 pn = normal_from_id(PF.nearest(sc), 1.0f);
        v3 pd = mk3(fabsf(bp.x - pp.x), fabsf(bp.y - pp.y), fabsf(bp.z - pp.z));
        float perr = dot(pd, pd);
        float cw = weights[k];
        int sblock = min(max(PB.nearest(sc), 0), 127);
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
    float inc = a.be_useful ? 1.0f : 0.0f;
    float spp_inc = sspp + inc;
    if (successful <= 0) spp_inc = 0.01f;
    float blend = fmaxf(1.0f / spp_inc, 0.05f);
    float mfac = fmaxf(1.0f / spp_inc, 0.05f);
    if (!a.be_useful) { blend = 0.99f; sspp = 0.0f; }
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
    for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, clampf(osh[c], -100.0f, 100.0f));
    for (int c = 0; c < 2; c++) st(o_cocg + px * 2 + c, clampf(occ[c], -10.0f, 100.0f));
    for (int c = 0; c < 2; c++) st(o_aosky + px * 2 + c, clampf(oao[c], 0.0f, 1.0f));
    st(o_util + px * 4 + 0, clampf(util_spp, -150.0f, 150.0f));
    st(o_util + px * 4 + 1, clampf(util_mom, -150.0f, 150.0f));
    st(o_util + px * 4 + 2, clampf(store_luma, -150.0f, 150.0f));
    st(o_util + px * 4 + 3, 0.0f);
}

// SVGF/VarianceEstimate.glsl main (:73-193) with DO_SPATIAL and
// AGGRESSIVE_DISOCCLUSION_HANDLING on.
template <typename S>
__global__ void __launch_bounds__(256) k_variance(CamView cam, int W, int H, const S* t, const uint8_t* face,
                                                  const S* i_sh, const S* i_cocg, const S* i_util, S* o_sh,
                                                  S* o_cocg, S* o_var) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const Plane<S, 4> SH{i_sh, W, H}, U{i_util, W, H};
    const Plane<S, 2> CC{i_cocg, W, H};
    const Plane8 F{face, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float thresh = 4.0f + 4.0f + 4.0f;
    size_t px = (size_t)j * W + i;
    v2 uv = texcoord(i, j, W, H);
    float bsh[4], bcc[2];
    for (int c = 0; c < 4; c++) bsh[c] = SH.at_in(i, j, c);
    for (int c = 0; c < 2; c++) bcc[c] = CC.at_in(i, j, c);
    float bl = sh_to_y(bsh);
    float acc = U.at_in(i, j, 0);
    float bm = U.at_in(i, j, 1);
    float osh[4], occ[2], var;
    if (acc < thresh) {
        v4 bp = position_fetch(cam, T, i, j, uv);
        v3 bn = normal_from_id(F.at_in(i, j), 1.0f);
        const float phi = 5.0f;
        float tw = 0.0f, tm = 0.0f, tl = 0.0f, tw2 = 0.0f;
        float tsh[4] = {0.0f, 0.0f, 0.0f, 0.0f}, tcc[2] = {0.0f, 0.0f};
        for (int x = -4; x <= 4; x++) {
            for (int y = -4; y <= 4; y++) {
                int si = i + x, sj = j + y;
                if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
                v2 sc = mk2(uv.x + (float)x * texel_x, uv.y + (float)y * texel_y);
                v4 sp = position_fetch(cam, T, si, sj, sc);
                v3 sn = normal_from_id(F.at_in(si, sj), 1.0f);
                float smom = U.at_in(si, sj, 1);
                float ssh[4], scc[2];
                for (int c = 0; c < 4; c++) ssh[c] = SH.at_in(si, sj, c);
                for (int c = 0; c < 2; c++) scc[c] = CC.at_in(si, sj, c);
                float sl = sh_to_y(ssh);
                float nw = dpow(fmaxf(dot(bn, sn), 0.0f), 16.0f);
                float dw = dpow(dexp(-fabsf(sp.w - bp.w)), 2.0f);
                float lw = fabsf(sl - bl) / phi;
                float wgt = (dexp(-lw) * nw) * dw;
                float wgt2 = wgt;
                wgt = fmaxf(wgt, 0.000000015f);
                wgt2 = fmaxf(wgt2, 0.0000000015f);
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
    for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, clampf(osh[c], -100.0f, 100.0f));
    for (int c = 0; c < 2; c++) st(o_cocg + px * 2 + c, clampf(occ[c], -10.0f, 100.0f));
    st(o_var + px, clampf(var, -1.0f, 50.0f));
}

// SVGF/SpatialFilter.glsl main (:175-355), 3x3 taps (u_LargeKernel off).
template <typename S>
__global__ void __launch_bounds__(256) k_atrous(CamView cam, int W, int H, AtrousArgs a, const S* t,
                                                const uint8_t* face, const S* t_util, const S* i_sh,
                                                const S* i_cocg, const S* i_var, const S* i_aosky, S* o_sh,
                                                S* o_cocg, S* o_var, S* o_aosky) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H}, V{i_var, W, H};
    const Plane<S, 4> SH{i_sh, W, H}, U{t_util, W, H};
    const Plane<S, 2> CC{i_cocg, W, H}, AO{i_aosky, W, H};
    const Plane8 F{face, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float aw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
    const float gauss[2] = {0.60283f, 0.198585f};
    const int step = a.step;
    const bool filter_ao = step <= 4;
    const bool filter_sky = (step <= 6) || filter_ao;
    size_t px = (size_t)j * W + i;
    v2 uv = texcoord(i, j, W, H);
    // GradientNoise (:160-165)
    float gx = ((float)i + 0.5f) + a.tmod500, gy = ((float)j + 0.5f) + a.tmod500;
    float noise = fract(52.9829189f * fract(0.06711056f * gx + 0.00583715f * gy));
    int jit = f2i((noise - 0.5f) * ((float)step * 0.8f));
    float bd = T.at_in(i, j, 0);
    v3 bn = normal_from_id(F.at_in(i, j), 1.0f);
    float bsh[4], bcc[2], bao[2];
    for (int c = 0; c < 4; c++) bsh[c] = SH.at_in(i, j, c);
    for (int c = 0; c < 2; c++) { bcc[c] = CC.at_in(i, j, c); bao[c] = AO.at_in(i, j, c); }
    float bl = sh_to_y(bsh);
    // GaussianVariance (:94-129)
    float bvar = 0.0f, vsum = 0.0f, tk = 0.0f;
    for (int x = -1; x <= 1; x++) {
        for (int y = -1; y <= 1; y++) {
            int si = i + x, sj = j + y;
            if (si < 0 || si >= W || sj < 0 || sj >= H) continue;
            float kv = gauss[abs(x)] * gauss[abs(y)];
            float v = V.at_in(si, sj, 0);
            if (x == 0 && y == 0) bvar = v;
            vsum += v * kv;
            tk += kv;
        }
    }
    float vest = vsum / fmaxf(tk, 0.01f);
    float tsh[4] = {bsh[0], bsh[1], bsh[2], bsh[3]}, tcc[2] = {bcc[0], bcc[1]};
    float tw = 1.0f, tvar = bvar, tao[2] = {bao[0], bao[1]}, taow = 1.0f;
    float acc_frames = U.at_in(i, j, 0);
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
        tweaked = fe * dpow(tt, curve + 6.0f);
    }
    float phi = sqrtf(fmaxf(0.0f, 0.000001f + tweaked));
    phi /= a.phi_bias;
    for (int x = -1; x <= 1; x++) {
        for (int y = -1; y <= 1; y++) {
            if (x == 0 && y == 0) continue;
            float ox = ((float)x * (float)step) * a.add_scale + (float)jit * 0.5f;
            float oy = ((float)y * (float)step) * a.add_scale + (float)jit * 0.5f;
            v2 sc = mk2(uv.x + ox * texel_x, uv.y + oy * texel_y);
            if (!(sc.x > 0.0f && sc.x < 1.0f && sc.y > 0.0f && sc.y < 1.0f)) continue;
            float sd;
            T.linear(sc, &sd);
            float dd = fabsf(sd - bd);
            v3 sn = normal_from_id(F.nearest(sc), 1.0f);
            if ((bd < 0.0f) == (dd < 0.0f)) {
                float ssh[4], scc[2], sv;
                SH.linear(sc, ssh);
                CC.linear(sc, scc);
                float sl = sh_to_y(ssh);
                V.linear(sc, &sv);
                float nw = clampf(dpow(fmaxf(dot(bn, sn), 0.0f), 32.0f), 0.001f, 1.0f);
                float lw = fabsf(sl - bl) / phi;
                float dw = clampf(dpow(dexp(-fmaxf(dd, 0.00001f)), 2.0f), 0.0001f, 1.0f);
                float wgt = strong ? nw * dw : (dexp(-lw) * nw) * dw;
                wgt = clampf(wgt, 0.001f, 1.0f);
                float xw = aw[abs(x)], yw = aw[abs(y)];
                wgt = (xw * yw) * wgt;
                wgt = fmaxf(wgt, 0.00000001f);
                for (int c = 0; c < 4; c++) tsh[c] += ssh[c] * wgt;
                for (int c = 0; c < 2; c++) tcc[c] += scc[c] * wgt;
                tvar += (wgt * wgt) * sv;
                tw += wgt;
                if (filter_sky || filter_ao) {
                    float awt = clampf(((xw * yw) * nw) * dw, 0.000001f, 1.0f);
                    float sao[2];
                    AO.linear(sc, sao);
                    tao[0] += sao[0] * awt;
                    tao[1] += sao[1] * awt;
                    taow += awt;
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
    for (int c = 0; c < 4; c++) st(o_sh + px * 4 + c, clampf(tsh[c], -100.0f, 100.0f));
    for (int c = 0; c < 2; c++) st(o_cocg + px * 2 + c, clampf(tcc[c], -10.0f, 100.0f));
    st(o_var + px, clampf(tvar, -1.0f, 50.0f));
    st(o_aosky + px * 2 + 0, clampf(tao[0], 0.0f, 1.0f));
    st(o_aosky + px * 2 + 1, clampf(tao[1], 0.0f, 1.0f));
}

inline dim3 grid2(int W, int H) { return dim3((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8)); }
const dim3 kBlock2(32, 8);

}  // namespace

cudaError_t svgf_spatial_initial(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                                 GIIn in, GIOut out, cudaStream_t s) {
    if (fp16)
        k_spatial_initial<__half><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, (const __half*)t, face, (const __half*)in.sh, (const __half*)in.cocg, (const __half*)in.luma,
            (const __half*)in.aosky, (__half*)out.sh, (__half*)out.cocg, (__half*)out.luma, (__half*)out.aosky);
    else
        k_spatial_initial<float><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, (const float*)t, face, (const float*)in.sh, (const float*)in.cocg, (const float*)in.luma,
            (const float*)in.aosky, (float*)out.sh, (float*)out.cocg, (float*)out.luma, (float*)out.aosky);
    return cudaGetLastError();
}

cudaError_t svgf_temporal(const CamView& cam, int W, int H, int fp16, const TemporalArgs& a,
                          const void* t, const uint8_t* face, const uint8_t* block,
                          const void* prev_t, const uint8_t* prev_face, const uint8_t* prev_block,
                          GIIn cur, HistIO prev, HistIO out, cudaStream_t s) {
    if (fp16)
        k_temporal<__half><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, a, (const __half*)t, face, block, (const __half*)prev_t, prev_face, prev_block,
            (const __half*)cur.sh, (const __half*)cur.cocg, (const __half*)cur.luma, (const __half*)cur.aosky,
            (const __half*)prev.sh, (const __half*)prev.cocg, (const __half*)prev.util, (const __half*)prev.aosky,
            (__half*)out.sh, (__half*)out.cocg, (__half*)out.util, (__half*)out.aosky);
    else
        k_temporal<float><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, a, (const float*)t, face, block, (const float*)prev_t, prev_face, prev_block,
            (const float*)cur.sh, (const float*)cur.cocg, (const float*)cur.luma, (const float*)cur.aosky,
            (const float*)prev.sh, (const float*)prev.cocg, (const float*)prev.util, (const float*)prev.aosky,
            (float*)out.sh, (float*)out.cocg, (float*)out.util, (float*)out.aosky);
    return cudaGetLastError();
}

cudaError_t svgf_variance(const CamView& cam, int W, int H, int fp16, const void* t, const uint8_t* face,
                          HistIO in, FiltIO out, cudaStream_t s) {
    if (fp16)
        k_variance<__half><<<grid2(W, H), kBlock2, 0, s>>>(cam, W, H, (const __half*)t, face, (const __half*)in.sh,
                                                           (const __half*)in.cocg, (const __half*)in.util,
                                                           (__half*)out.sh, (__half*)out.cocg, (__half*)out.variance);
    else
        k_variance<float><<<grid2(W, H), kBlock2, 0, s>>>(cam, W, H, (const float*)t, face, (const float*)in.sh,
                                                          (const float*)in.cocg, (const float*)in.util,
                                                          (float*)out.sh, (float*)out.cocg, (float*)out.variance);
    return cudaGetLastError();
}

cudaError_t svgf_atrous(const CamView& cam, int W, int H, int fp16, const AtrousArgs& a,
                        const void* t, const uint8_t* face, const void* temporal_util,
                        FiltIO in, const void* in_aosky, FiltIO out, cudaStream_t s) {
    if (fp16)
        k_atrous<__half><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, a, (const __half*)t, face, (const __half*)temporal_util, (const __half*)in.sh,
            (const __half*)in.cocg, (const __half*)in.variance, (const __half*)in_aosky, (__half*)out.sh,
            (__half*)out.cocg, (__half*)out.variance, (__half*)out.aosky);
    else
        k_atrous<float><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, a, (const float*)t, face, (const float*)temporal_util, (const float*)in.sh,
            (const float*)in.cocg, (const float*)in.variance, (const float*)in_aosky, (float*)out.sh,
            (float*)out.cocg, (float*)out.variance, (float*)out.aosky);
    return cudaGetLastError();
}

}  // namespace vpt
