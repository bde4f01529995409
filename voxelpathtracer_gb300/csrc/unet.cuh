// Launch interfaces of the learned-denoiser kernels (unet.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace vpt {

// Input of a 3x3 convolution: channels [0, C0) from p0 (at half resolution
// and nearest-upsampled when up0 = 1), channels [C0, C0 + C1) from p1 at full
// resolution (p1 unused when C1 = 0). N images of H x W (the output size).
struct ConvSrc {
    const __nv_bfloat16* p0;
    int C0;
    int up0;
    const __nv_bfloat16* p1;
    int C1;
    int N, H, W;
};

struct ConvArgs {
    ConvSrc in;
    const __nv_bfloat16* w;    // [Np][9][Cin], tap = (dy + 1) * 3 + (dx + 1)
    const float* bias;         // [Np] or null
    int Cin;                   // C0 + C1, multiple of 16, <= 256
    int Np;                    // output channels, multiple of 16, <= 256
    int relu;                  // max(0, .) after the bias
    const __nv_bfloat16* mask; // [P][Np]: output zeroed where mask <= 0 (ReLU derivative), or null
    __nv_bfloat16* out;        // [P][Np] BF16 or null
    float* out_f32;            // [P][Np] FP32 or null
    int* err;                  // nonzero after a timed-out wait (which wait), or null
    __nv_bfloat16* scratch;    // [P][Cin]: the concatenated input is assembled here when it has two sources
};

struct DwArgs {
    ConvSrc in;                // the forward input X
    const __nv_bfloat16* dy;   // [P][Np] gradient of the pre-activation output
    int Cin;                   // C0 + C1
    int Np;                    // <= 128
    int pix_per_cta;           // multiple of 128
    float* dw;                 // [Np][9][Cin] FP32, accumulated
    int* err;
};

size_t conv3x3_smem(int Cin, int Np);
size_t conv3x3_dw_smem(int Cin);
cudaError_t conv3x3(const ConvArgs& a, cudaStream_t s);
cudaError_t conv3x3_dw(const DwArgs& a, cudaStream_t s);
cudaError_t pool2(const __nv_bfloat16* in, __nv_bfloat16* out, int N, int H, int W, int C, cudaStream_t s);
cudaError_t upsum_mask(const __nv_bfloat16* g, int Cg, int off, const __nv_bfloat16* act, __nv_bfloat16* out, int N,
                       int H, int W, int C, cudaStream_t s);
cudaError_t skip_mask(const __nv_bfloat16* g, int Cg, int off, const __nv_bfloat16* gpool, const __nv_bfloat16* act,
                      __nv_bfloat16* out, int N, int H, int W, int C, cudaStream_t s);
cudaError_t mse_grad(const float* out, const float* target, __nv_bfloat16* g, long long P, float scale, double* loss,
                     cudaStream_t s);
cudaError_t bias_grad(const __nv_bfloat16* g, long long P, int C, float* db, cudaStream_t s);
cudaError_t adam(float* w, const float* grad, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                 int step, cudaStream_t s);
cudaError_t weights_bf16(const float* w, __nv_bfloat16* wf, __nv_bfloat16* wb, int Np, int Cin, cudaStream_t s);

}  // namespace vpt
