// High-spp ground truth of the diffuse GI over a crop of the frame, with a
// per-pixel FP64 Welford mean / M2 of the seven GI channels (SH 4, CoCg 2,
// AO). This is the only FP64 on the GPU: the sampler itself (CalculateDiffuse,
// DiffuseRayTraceFrag.glsl:535-664) runs in fp32 exactly as the diffuse pass.
//
// Work split: thread (pixel, chunk) runs samples [chunk*c, chunk*(c+1)) with a
// fresh PCG stream per (pixel, sample) and keeps its own Welford state; a
// second kernel merges the chunks of a pixel in chunk order with Chan et al.'s
// pairwise update. The order is fixed, so results are reproducible and the CPU
// restatement matches them bit for bit.
#include "gi.cuh"

namespace vpt {

namespace {

constexpr int kGtCh = 7;
constexpr int kGtRec = 1 + 2 * kGtCh;   // n, mean[7], m2[7]

__device__ __forceinline__ uint32_t gt_stream(uint32_t px, uint32_t k, uint32_t seed) {
    return pcg_hash(px + pcg_hash(k + pcg_hash(seed ^ 0x9E3779B9u)));
}

// kTex: the bounce hits sample the block textures (a.d.textured)
template <bool kTex>
__global__ void __launch_bounds__(128) k_gt_partial(GroundTruthArgs a) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int npx = a.cw * a.ch;
    if (idx >= npx * a.nchunks) return;
    const int p = idx / a.nchunks, c = idx % a.nchunks;
    const int i = a.x0 + p % a.cw, j = a.y0 + p / a.cw;
    const size_t px = (size_t)j * a.W + i;
    double n = 0.0, mean[kGtCh], m2[kGtCh];
    for (int q = 0; q < kGtCh; q++) mean[q] = m2[q] = 0.0;
    const v3 dir = normalize(ray_dir_at(a.cam, texcoord(i, j, a.W, a.H)));
    const float d = a.t[px];
    const v3 pos = add(ray_origin(a.cam), muls(dir, d));
    const v3 nrm = normal_from_id(a.face[px], 0.5f);
    const int k0 = c * a.chunk, k1 = min(a.spp, k0 + a.chunk);
    GICount cnt = {0u, 0u, 0u, 0u};
    for (int k = k0; k < k1; k++) {
        float v[kGtCh];
        float sh[4], cocg[2];
        if (d < 0.0f) {
            irradiance_to_sh(muls(sky_radiance(dir), 2.66f), nrm, sh, cocg);
            v[6] = 1.0f;
        } else {
            uint32_t rng = gt_stream((uint32_t)px, (uint32_t)k, a.seed);
            v3 odir = mk3(0.0f, 0.0f, 0.0f);
            bool sky = false;
            const v4 x = calculate_diffuse<0, kTex>(a.w, a.d, pos, nrm, &rng, &odir, &sky, &cnt);
            irradiance_to_sh(vclamp(mk3(x.x, x.y, x.z), 0.0f, 8.0f), odir, sh, cocg);
            v[6] = x.w;
        }
        v[0] = sh[0]; v[1] = sh[1]; v[2] = sh[2]; v[3] = sh[3];
        v[4] = cocg[0]; v[5] = cocg[1];
        n += 1.0;
        for (int q = 0; q < kGtCh; q++) {
            const double x = (double)v[q];
            const double delta = x - mean[q];
            mean[q] = mean[q] + delta / n;
            m2[q] = m2[q] + delta * (x - mean[q]);
        }
    }
    double* out = a.part + (size_t)idx * kGtRec;
    out[0] = n;
    for (int q = 0; q < kGtCh; q++) {
        out[1 + q] = mean[q];
        out[1 + kGtCh + q] = m2[q];
    }
}

__global__ void __launch_bounds__(128) k_gt_merge(GroundTruthArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.cw * a.ch) return;
    double n = 0.0, mean[kGtCh], m2[kGtCh];
    for (int q = 0; q < kGtCh; q++) mean[q] = m2[q] = 0.0;
    for (int c = 0; c < a.nchunks; c++) {
        const double* r = a.part + ((size_t)p * a.nchunks + c) * kGtRec;
        const double nb = r[0];
        if (nb == 0.0) continue;
        if (n == 0.0) {
            n = nb;
            for (int q = 0; q < kGtCh; q++) {
                mean[q] = r[1 + q];
                m2[q] = r[1 + kGtCh + q];
            }
            continue;
        }
        const double tot = n + nb;
        for (int q = 0; q < kGtCh; q++) {
            const double delta = r[1 + q] - mean[q];
            mean[q] = mean[q] + delta * (nb / tot);
            m2[q] = (m2[q] + r[1 + kGtCh + q]) + (delta * delta) * ((n * nb) / tot);
        }
        n = tot;
    }
    for (int q = 0; q < kGtCh; q++) {
        a.mean[(size_t)p * kGtCh + q] = mean[q];
        a.m2[(size_t)p * kGtCh + q] = m2[q];
    }
}

}  // namespace

cudaError_t ground_truth(const GroundTruthArgs& a, cudaStream_t s) {
    const int parts = a.cw * a.ch * a.nchunks;
    (a.d.textured ? k_gt_partial<true> : k_gt_partial<false>)<<<(parts + 127) / 128, 128, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_gt_merge<<<(a.cw * a.ch + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace vpt
