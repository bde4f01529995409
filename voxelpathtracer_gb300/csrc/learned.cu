// Glue between the frame planes and the learned denoiser: the 16-channel
// BF16 feature tensor the network reads, and the colour it writes back.
//
// Features of a pixel (all zero where a channel does not apply):
//   0-2   log(1 + noisy RGB)     the colour pass over the temporally accumulated GI
//   3-5   albedo                 block table entry of the hit block (RGB8 / 255)
//   6-8   normal                 the hit face's axis normal
//   9     depth                  min(hit distance, 512) / 128; 0 for sky
//   10    log(1 + variance)      the SVGF variance estimate
//   11-13 log(1 + raw RGB)       the colour pass over this frame's 1-spp GI (no
//                                temporal accumulation, so none of its reprojection blur)
//   14-15 0
// The network predicts a correction in log space: the colour plane receives
// max(exp(log(1 + noisy) + out) - 1, 0), or keeps the noisy colour where that
// is not finite.
#include <cuda_bf16.h>

#include "kernels.cuh"

namespace vpt {

namespace {

template <typename S>
__global__ void k_features(int W, int H, int x0, int y0, int w, int h, const S* color, const S* color_raw, const S* t,
                           const uint8_t* face, const uint8_t* block, const vpt_block* blocks, int n_blocks,
                           const S* var, __nv_bfloat16* out) {
    const int lx = blockIdx.x * blockDim.x + threadIdx.x, ly = blockIdx.y * blockDim.y + threadIdx.y;
    if (lx >= w || ly >= h) return;
    const int i = x0 + lx, j = y0 + ly;
    float f[16];
#pragma unroll
    for (int k = 0; k < 16; k++) f[k] = 0.0f;
    if (i >= 0 && i < W && j >= 0 && j < H) {
        const size_t px = (size_t)j * W + i;
        for (int c = 0; c < 3; c++) f[c] = log1pf(fmaxf(ld(color + px * 3 + c), 0.0f));
        const int b = block[px];
        if (b > 0 && b < n_blocks) {
            const vpt_block bb = blocks[b];
            f[3] = bb.albedo[0] / 255.0f;
            f[4] = bb.albedo[1] / 255.0f;
            f[5] = bb.albedo[2] / 255.0f;
        }
        const int fc = face[px];
        if (fc <= 5) {
            const v3 n = normal_from_id(fc, 0.0f);
            f[6] = n.x;
            f[7] = n.y;
            f[8] = n.z;
        }
        const float d = ld(t + px);
        f[9] = d > 0.0f ? fminf(d, 512.0f) / 128.0f : 0.0f;
        f[10] = log1pf(fmaxf(ld(var + px), 0.0f));
        for (int c = 0; c < 3; c++) f[11 + c] = log1pf(fmaxf(ld(color_raw + px * 3 + c), 0.0f));
    }
    __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(out + ((size_t)ly * w + lx) * 16);
#pragma unroll
    for (int k = 0; k < 8; k++) o[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
}

template <typename S>
__global__ void k_unpack(int W, int H, const float* net_out, S* color) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= W || j >= H) return;
    const size_t px = (size_t)j * W + i;
    const float4 o = *reinterpret_cast<const float4*>(net_out + px * 16);
    const float v[3] = {o.x, o.y, o.z};
    for (int c = 0; c < 3; c++) {
        const float noisy = log1pf(fmaxf(ld(color + px * 3 + c), 0.0f));
        const float r = expm1f(noisy + v[c]);
        if (isfinite(r)) st(color + px * 3 + c, fmaxf(r, 0.0f));
    }
}

}  // namespace

cudaError_t learned_features(int W, int H, int x0, int y0, int w, int h, int fp16, const void* color,
                             const void* color_raw, const void* t,
                             const uint8_t* face, const uint8_t* block, const vpt_block* blocks, int n_blocks,
                             const void* var, void* out, cudaStream_t s) {
    const dim3 b(32, 8), g((unsigned)((w + 31) / 32), (unsigned)((h + 7) / 8));
    if (fp16)
        k_features<__half><<<g, b, 0, s>>>(W, H, x0, y0, w, h, (const __half*)color, (const __half*)color_raw,
                                          (const __half*)t, face, block,
                                          blocks, n_blocks, (const __half*)var, (__nv_bfloat16*)out);
    else
        k_features<float><<<g, b, 0, s>>>(W, H, x0, y0, w, h, (const float*)color, (const float*)color_raw,
                                         (const float*)t, face, block,
                                         blocks, n_blocks, (const float*)var, (__nv_bfloat16*)out);
    return cudaGetLastError();
}

cudaError_t learned_unpack(int W, int H, int fp16, const float* net_out, void* color, cudaStream_t s) {
    const dim3 b(32, 8), g((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8));
    if (fp16) k_unpack<__half><<<g, b, 0, s>>>(W, H, net_out, (__half*)color);
    else k_unpack<float><<<g, b, 0, s>>>(W, H, net_out, (float*)color);
    return cudaGetLastError();
}

}  // namespace vpt
