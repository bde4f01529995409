// The reference's non-SVGF denoiser path (USE_SVGF off, Core/Pipeline.cpp:
// 2618-2786): temporal blend (TemporalFilter.glsl, diffuse mode), a 5x5
// luminance variance (SampleVarianceCompute.glsl) and five 5x5 B3-spline
// a-trous iterations with steps 12, 8, 4, 2, 1 (AtrousSpatialFilter.glsl).
// One thread per pixel, 32x8 blocks, taps at integer offsets are fetches.
#include "kernels.cuh"

namespace vpt {

namespace {

__device__ __forceinline__ bool pixel_of(int W, int H, int* i, int* j) {
    *i = blockIdx.x * blockDim.x + threadIdx.x;
    *j = blockIdx.y * blockDim.y + threadIdx.y;
    return *i < W && *j < H;
}

// TemporalFilter.glsl main (:369-487), u_DiffuseTemporal on, u_MinimumMix 0,
// u_MaximumMix 0.96. AO passes through, the utility plane is zeroed.
template <typename S, bool kScaled>
__global__ void __launch_bounds__(256) k_plain_temporal(CamView cam, int W, int H, int Wf, int Hf, TemporalArgs a,
                                                        const S* t,
                                                        const S* prev_t, const S* c_sh, const S* c_cocg,
                                                        const S* c_aosky, const S* p_sh, const S* p_cocg, S* o_sh,
                                                        S* o_cocg, S* o_util, S* o_aosky) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const size_t px = (size_t)j * W + i;
    const v2 uv = texcoord(i, j, W, H);
    const v4 bp = position_fetch(cam, T, i, j, uv);
    float4 sh = ld4(c_sh + 4 * px);
    float2 cc = ld2(c_cocg + 2 * px);
    const float min_mix = clampf(0.0f, 0.01f, 0.9f), max_mix = clampf(0.96f, 0.1f, 0.98f);
    if (bp.w > 0.0f) {
        const v4 pr = mat_mul4(a.prev_view_proj, bp.x, bp.y, bp.z, 1.0f);
        const v2 rc = mk2((pr.x / pr.w) * 0.5f + 0.5f, (pr.y / pr.w) * 0.5f + 0.5f);
        const Bilin fp = bilin(rc, W, H);
        const Bilin fq = kScaled ? bilin(rc, Wf, Hf) : fp;
        const float4 psh = bl4(p_sh, fp);
        const float pt = bl1(prev_t, fq);
        const v3 pp = add(ray_origin(cam), muls(normalize(ray_dir_at(cam, rc)), pt));
        const float bias = 0.01f;
        if (rc.x > 0.0f + bias && rc.x < 1.0f - bias && rc.y > 0.0f + bias && rc.y < 1.0f - bias) {
            const float d = fabsf(length(sub(pp, mk3(bp.x, bp.y, bp.z))));
            if (!(d > 1.1f)) {
                float bf = dexp(-d);
                bf = clampf(bf, min_mix, max_mix);
                const float bfc = clampf(bf, 0.0f, 0.96f);
                const float2 pcc = bl2(p_cocg, fp);
                sh = make_float4(mixf(sh.x, psh.x, bfc), mixf(sh.y, psh.y, bfc), mixf(sh.z, psh.z, bfc),
                                 mixf(sh.w, psh.w, bfc));
                cc = make_float2(mixf(cc.x, pcc.x, bf), mixf(cc.y, pcc.y, bf));
            }
        }
    }
    st4(o_sh + 4 * px, sh.x, sh.y, sh.z, sh.w);
    st2(o_cocg + 2 * px, cc.x, cc.y);
    const float2 ao = ld2(c_aosky + 2 * px);
    st2(o_aosky + 2 * px, ao.x, ao.y);
    st4(o_util + 4 * px, 0.0f, 0.0f, 0.0f, 0.0f);
}

// SampleVarianceCompute.glsl: 5x5 luminance variance, REPEAT wrap.
template <typename S>
__global__ void __launch_bounds__(256) k_plain_variance(int W, int H, const S* sh, S* var) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    float tx = 0.0f, ty = 0.0f;
    int n = 0;
#pragma unroll
    for (int a = -2; a <= 2; a++) {
#pragma unroll
        for (int b = -2; b <= 2; b++) {
            const int si = wrapi(i + a, W), sj = wrapi(j + b, H);
            const float4 s = ld4(sh + 4 * ((size_t)sj * W + si));
            const float l = luminance(mk3(s.x, s.y, s.z));
            tx += l;
            ty += l * l;
            n++;
        }
    }
    const float nn = fmaxf((float)n, 1.0f);
    tx /= nn;
    ty /= nn;
    st(var + (size_t)j * W + i, fmaxf(0.0f, ty - tx * tx));
}

// AtrousSpatialFilter.glsl main (:96-220): the saturation / luminance / edge
// weights it computes are reset to 1 before use, so only the gates and the
// distance weight shape the result.
template <typename S>
__global__ void __launch_bounds__(256) k_plain_atrous(CamView cam, int W, int H, int step, const S* t,
                                                      const uint8_t* face, const uint8_t* block, const S* sh,
                                                      const S* cocg, const S* aosky, S* o_sh, S* o_cocg,
                                                      S* o_aosky) {
    int i, j;
    if (!pixel_of(W, H, &i, &j)) return;
    const Plane<S, 1> T{t, W, H};
    const float texel_x = 1.0f / (float)W, texel_y = 1.0f / (float)H;
    const float weights[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
    const size_t px = (size_t)j * W + i;
    const v2 uv = texcoord(i, j, W, H);
    const v4 bp = position_fetch(cam, T, i, j, uv);
    const v3 bn = normal_from_id(__ldg(face + px), 1.0f);
    const int bblock = min(max((int)__ldg(block + px), 0), 127);
    const bool bsky = bp.w < 0.0f;
    float tc[4] = {0.0f, 0.0f, 0.0f, 0.0f}, t2[2] = {0.0f, 0.0f}, tw = 0.0f;
    for (int tx = -2; tx <= 2; tx++) {
        const int ox = step * tx, si = i + ox;
        if (si < 0 || si >= W) continue;
#pragma unroll
        for (int ty = -2; ty <= 2; ty++) {
            const int oy = step * ty, sj = j + oy;
            if (sj < 0 || sj >= H) continue;
            const size_t sp_ = (size_t)sj * W + si;
            const v2 sc = mk2(uv.x + (float)ox * texel_x, uv.y + (float)oy * texel_y);
            const v4 pa = position_fetch(cam, T, si, sj, sc);
            const v3 na = normal_from_id(__ldg(face + sp_), 1.0f);
            const int ba = min(max((int)__ldg(block + sp_), 0), 127);
            const float err = (fabsf(pa.x - bp.x) + fabsf(pa.y - bp.y)) + fabsf(pa.z - bp.z);
            if (err < 4.25f && na.x == bn.x && na.y == bn.y && na.z == bn.z && ba == bblock && (pa.w < 0.0f) == bsky) {
                const float dw = dpow(fabsf(4.25f - err), 6.9f);
                const float wgt = (weights[tx + 2] * weights[ty + 2]) * dw;
                const float4 s4 = ld4(sh + 4 * sp_);
                const float2 s2 = ld2(cocg + 2 * sp_);
                tc[0] += s4.x * wgt;
                tc[1] += s4.y * wgt;
                tc[2] += s4.z * wgt;
                tc[3] += s4.w * wgt;
                t2[0] += s2.x * wgt;
                t2[1] += s2.y * wgt;
                tw += wgt;
            }
        }
    }
    const float d = fmaxf(tw, 0.01f);
    st4(o_sh + 4 * px, tc[0] / d, tc[1] / d, tc[2] / d, tc[3] / d);
    st2(o_cocg + 2 * px, t2[0] / d, t2[1] / d);
    const float2 ao = ld2(aosky + 2 * px);
    st2(o_aosky + 2 * px, ao.x, ao.y);
}

inline dim3 grid2(int W, int H) { return dim3((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8)); }
const dim3 kBlock2(32, 8);

template <typename S>
cudaError_t run_plain(const CamView& cam, int W, int H, const TemporalArgs& ta, const PlainDenoiseIO& io,
                      cudaStream_t s) {
    if (io.Wf != W || io.Hf != H)
        k_plain_temporal<S, true><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, io.Wf, io.Hf, ta, (const S*)io.t, (const S*)io.prev_t, (const S*)io.cur.sh,
            (const S*)io.cur.cocg, (const S*)io.cur.aosky, (const S*)io.prev.sh, (const S*)io.prev.cocg,
            (S*)io.temporal.sh, (S*)io.temporal.cocg, (S*)io.temporal.util, (S*)io.temporal.aosky);
    else
        k_plain_temporal<S, false><<<grid2(W, H), kBlock2, 0, s>>>(
            cam, W, H, io.Wf, io.Hf, ta, (const S*)io.t, (const S*)io.prev_t, (const S*)io.cur.sh,
            (const S*)io.cur.cocg, (const S*)io.cur.aosky, (const S*)io.prev.sh, (const S*)io.prev.cocg,
            (S*)io.temporal.sh, (S*)io.temporal.cocg, (S*)io.temporal.util, (S*)io.temporal.aosky);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_plain_variance<S><<<grid2(W, H), kBlock2, 0, s>>>(W, H, (const S*)io.temporal.sh, (S*)io.variance);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const S* in_sh = (const S*)io.temporal.sh;
    const S* in_cc = (const S*)io.temporal.cocg;
    const S* in_ao = (const S*)io.temporal.aosky;
    const int steps[5] = {12, 8, 4, 2, 1};   // Core/Pipeline.cpp:2712
    for (int it = 0; it < io.iterations; it++) {
        const int step = it < 5 ? steps[it] : 1;
        const FiltIO& o = io.out[it & 1];
        k_plain_atrous<S><<<grid2(W, H), kBlock2, 0, s>>>(cam, W, H, step, (const S*)io.t, io.face, io.block, in_sh,
                                                          in_cc, in_ao, (S*)o.sh, (S*)o.cocg, (S*)o.aosky);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        in_sh = (const S*)o.sh;
        in_cc = (const S*)o.cocg;
        in_ao = (const S*)o.aosky;
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t plain_denoise(const CamView& cam, int W, int H, int fp16, const TemporalArgs& ta,
                          const PlainDenoiseIO& io, cudaStream_t s) {
    return fp16 ? run_plain<__half>(cam, W, H, ta, io, s) : run_plain<float>(cam, W, H, ta, io, s);
}

}  // namespace vpt
