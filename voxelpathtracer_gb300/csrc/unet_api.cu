// libvpt C ABI of the learned denoiser: the raw convolution operators over
// caller device pointers, and the 3-level U-Net (32/64/96 channels, 3x3
// convolutions, ReLU, BF16 weights and activations, FP32 accumulation) with
// its forward pass, backward pass and Adam step, all on the tcgen05 kernels of
// unet.cu.
//
// Network (N images of H x W, H and W multiples of 4):
//   e1a = relu(conv(x, 16->32))           e1 = relu(conv(e1a, 32->32))     H
//   p1 = pool(e1); e2a = relu(conv(p1, 32->64)); e2 = relu(conv(e2a, 64->64))  H/2
//   p2 = pool(e2); e3a = relu(conv(p2, 64->96)); e3 = relu(conv(e3a, 96->96))  H/4
//   d2a = relu(conv([up(e3), e2], 160->64)); d2 = relu(conv(d2a, 64->64))      H/2
//   d1a = relu(conv([up(d2), e1], 96->32));  d1 = relu(conv(d1a, 32->32))      H
//   out = conv(d1, 32->16), FP32; channels 0..2 are the prediction.
// The input has 11 feature channels padded to 16. Parameters are one FP32
// vector: per layer the weights [Np][9][Cin] followed by the bias [Np].
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "unet.cuh"
#include "vpt.h"

using namespace vpt;

namespace {

using bf16 = __nv_bfloat16;

struct LayerDef {
    int cin, cout, cin_real, cout_real, relu;
};
constexpr int kLayers = 11;
const LayerDef kNet[kLayers] = {
    {16, 32, 11, 32, 1}, {32, 32, 32, 32, 1},     // e1a, e1b
    {32, 64, 32, 64, 1}, {64, 64, 64, 64, 1},     // e2a, e2b
    {64, 96, 64, 96, 1}, {96, 96, 96, 96, 1},     // e3a, e3b
    {160, 64, 160, 64, 1}, {64, 64, 64, 64, 1},   // d2a, d2b
    {96, 32, 96, 32, 1}, {32, 32, 32, 32, 1},     // d1a, d1b
    {32, 16, 32, 3, 0},                           // out
};

long long layer_offset(int l) {
    long long o = 0;
    for (int k = 0; k < l; k++) o += (long long)kNet[k].cout * 9 * kNet[k].cin + kNet[k].cout;
    return o;
}

// One error word per device for the raw operators (timed-out waits).
std::mutex g_err_mu;
int* g_err[64] = {};
int* err_word(int dev) {
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (!g_err[dev]) {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cudaMemset(p, 0, sizeof(int));
        g_err[dev] = (int*)p;
    }
    return g_err[dev];
}

vpt_status from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return VPT_OK;
    cudaGetLastError();
    if (e == cudaErrorInvalidValue) return VPT_ERR_INVALID_ARG;
    if (e == cudaErrorMemoryAllocation) return VPT_ERR_OOM;
    return VPT_ERR_CUDA;
}

}  // namespace

struct vpt_unet {
    int dev = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int maxN = 0, maxH = 0, maxW = 0;
    long long nparams = 0;
    float* params = nullptr;   // FP32 master
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int adam_step = 0;
    bf16* wf[kLayers] = {};    // forward weights
    bf16* wb[kLayers] = {};    // backward-data weights
    // activations
    bf16 *e1a, *e1, *p1, *e2a, *e2, *p2, *e3a, *e3, *d2a, *d2, *d1a, *d1;
    bf16 *cat2, *cat1;         // assembled decoder inputs [up(e3), e2] and [up(d2), e1]
    float* out = nullptr;
    // gradients
    bf16 *g_out, *g_d1, *g_d1a, *g_cat1, *g_d2, *g_d2a, *g_cat2, *g_e3, *g_e3a, *g_p2, *g_e2, *g_e2a, *g_p1, *g_e1,
        *g_e1a;
    double* loss = nullptr;
    int* errw = nullptr;
    bool weights_ready = false;
    std::vector<void*> allocs;
};

namespace {

vpt_status ufail(vpt_unet* u, vpt_status s, const char* fmt, ...) {
    if (u) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        u->err = buf;
    }
    return s;
}

#define UCK(u, call)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            cudaGetLastError();                                                                 \
            return ufail((u), e_ == cudaErrorMemoryAllocation ? VPT_ERR_OOM : VPT_ERR_CUDA,     \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);  \
        }                                                                                       \
    } while (0)

template <typename T>
vpt_status ualloc(vpt_unet* u, T** p, size_t count) {
    void* q = nullptr;
    const size_t bytes = count * sizeof(T) + 256;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ufail(u, VPT_ERR_OOM, "cudaMalloc(%zu) failed", bytes);
    }
    u->allocs.push_back(q);
    *p = (T*)q;
    return VPT_OK;
}

ConvSrc src1(const bf16* p, int C, int N, int H, int W) { return ConvSrc{p, C, 0, nullptr, 0, N, H, W}; }
ConvSrc src_cat(const bf16* low, int C0, const bf16* skip, int C1, int N, int H, int W) {
    return ConvSrc{low, C0, 1, skip, C1, N, H, W};
}

vpt_status run_conv(vpt_unet* u, int l, const ConvSrc& in, const bf16* mask, bf16* out, float* out_f32) {
    ConvArgs a;
    a.scratch = l == 6 ? u->cat2 : (l == 8 ? u->cat1 : nullptr);
    a.in = in;
    a.w = u->wf[l];
    a.bias = u->params + layer_offset(l) + (long long)kNet[l].cout * 9 * kNet[l].cin;
    a.Cin = kNet[l].cin;
    a.Np = kNet[l].cout;
    a.relu = kNet[l].relu;
    a.mask = mask;
    a.out = out;
    a.out_f32 = out_f32;
    a.err = u->errw;
    UCK(u, conv3x3(a, u->stream));
    return VPT_OK;
}

// Backward-data of layer l: gradient of its input (Cin channels) from the
// gradient `g` of its pre-activation output, times (mask > 0) when given.
vpt_status run_conv_bwd(vpt_unet* u, int l, const bf16* g, int N, int H, int W, const bf16* mask, bf16* out) {
    ConvArgs a;
    a.scratch = nullptr;
    a.in = src1(g, kNet[l].cout, N, H, W);
    a.w = u->wb[l];
    a.bias = nullptr;
    a.Cin = kNet[l].cout;
    a.Np = kNet[l].cin;
    a.relu = 0;
    a.mask = mask;
    a.out = out;
    a.out_f32 = nullptr;
    a.err = u->errw;
    UCK(u, conv3x3(a, u->stream));
    return VPT_OK;
}

vpt_status run_dw(vpt_unet* u, int l, const ConvSrc& in, const bf16* g) {
    DwArgs a;
    a.in = in;
    a.dy = g;
    a.Cin = kNet[l].cin;
    a.Np = kNet[l].cout;
    a.pix_per_cta = 4096;
    a.dw = u->grads + layer_offset(l);
    a.err = u->errw;
    UCK(u, conv3x3_dw(a, u->stream));
    const long long P = (long long)in.N * in.H * in.W;
    UCK(u, bias_grad(g, P, kNet[l].cout, u->grads + layer_offset(l) + (long long)kNet[l].cout * 9 * kNet[l].cin,
                     u->stream));
    return VPT_OK;
}

vpt_status prepare_weights(vpt_unet* u) {
    if (u->weights_ready) return VPT_OK;
    for (int l = 0; l < kLayers; l++)
        UCK(u, weights_bf16(u->params + layer_offset(l), u->wf[l], u->wb[l], kNet[l].cout, kNet[l].cin, u->stream));
    u->weights_ready = true;
    return VPT_OK;
}

vpt_status check_shape(vpt_unet* u, int N, int H, int W) {
    if (N < 1 || H < 4 || W < 4 || (H & 3) || (W & 3))
        return ufail(u, VPT_ERR_INVALID_ARG, "image batch %d x %d x %d: sizes must be multiples of 4", N, H, W);
    if ((long long)N * H * W > (long long)u->maxN * u->maxH * u->maxW)
        return ufail(u, VPT_ERR_INVALID_ARG, "image batch %d x %d x %d exceeds the capacity", N, H, W);
    return VPT_OK;
}

vpt_status forward(vpt_unet* u, const bf16* x, int N, int H, int W) {
    vpt_status s;
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    if ((s = prepare_weights(u)) != VPT_OK) return s;
    if ((s = run_conv(u, 0, src1(x, 16, N, H, W), nullptr, u->e1a, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 1, src1(u->e1a, 32, N, H, W), nullptr, u->e1, nullptr)) != VPT_OK) return s;
    UCK(u, pool2(u->e1, u->p1, N, H, W, 32, u->stream));
    if ((s = run_conv(u, 2, src1(u->p1, 32, N, H2, W2), nullptr, u->e2a, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 3, src1(u->e2a, 64, N, H2, W2), nullptr, u->e2, nullptr)) != VPT_OK) return s;
    UCK(u, pool2(u->e2, u->p2, N, H2, W2, 64, u->stream));
    if ((s = run_conv(u, 4, src1(u->p2, 64, N, H4, W4), nullptr, u->e3a, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 5, src1(u->e3a, 96, N, H4, W4), nullptr, u->e3, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 6, src_cat(u->e3, 96, u->e2, 64, N, H2, W2), nullptr, u->d2a, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 7, src1(u->d2a, 64, N, H2, W2), nullptr, u->d2, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 8, src_cat(u->d2, 64, u->e1, 32, N, H, W), nullptr, u->d1a, nullptr)) != VPT_OK) return s;
    if ((s = run_conv(u, 9, src1(u->d1a, 32, N, H, W), nullptr, u->d1, nullptr)) != VPT_OK) return s;
    return run_conv(u, 10, src1(u->d1, 32, N, H, W), nullptr, nullptr, u->out);
}

vpt_status backward(vpt_unet* u, const bf16* x, const float* target, int N, int H, int W) {
    vpt_status s;
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    const long long P = (long long)N * H * W;
    UCK(u, cudaMemsetAsync(u->grads, 0, sizeof(float) * u->nparams, u->stream));
    UCK(u, cudaMemsetAsync(u->loss, 0, sizeof(double), u->stream));
    UCK(u, mse_grad(u->out, target, u->g_out, P, 1.0f / (float)(P * 3), u->loss, u->stream));
    // out
    if ((s = run_dw(u, 10, src1(u->d1, 32, N, H, W), u->g_out)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 10, u->g_out, N, H, W, u->d1, u->g_d1)) != VPT_OK) return s;
    // d1b, d1a
    if ((s = run_dw(u, 9, src1(u->d1a, 32, N, H, W), u->g_d1)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 9, u->g_d1, N, H, W, u->d1a, u->g_d1a)) != VPT_OK) return s;
    if ((s = run_dw(u, 8, src_cat(u->d2, 64, u->e1, 32, N, H, W), u->g_d1a)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 8, u->g_d1a, N, H, W, nullptr, u->g_cat1)) != VPT_OK) return s;
    UCK(u, upsum_mask(u->g_cat1, 96, 0, u->d2, u->g_d2, N, H, W, 64, u->stream));
    // d2b, d2a
    if ((s = run_dw(u, 7, src1(u->d2a, 64, N, H2, W2), u->g_d2)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 7, u->g_d2, N, H2, W2, u->d2a, u->g_d2a)) != VPT_OK) return s;
    if ((s = run_dw(u, 6, src_cat(u->e3, 96, u->e2, 64, N, H2, W2), u->g_d2a)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 6, u->g_d2a, N, H2, W2, nullptr, u->g_cat2)) != VPT_OK) return s;
    UCK(u, upsum_mask(u->g_cat2, 160, 0, u->e3, u->g_e3, N, H2, W2, 96, u->stream));
    // e3b, e3a
    if ((s = run_dw(u, 5, src1(u->e3a, 96, N, H4, W4), u->g_e3)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 5, u->g_e3, N, H4, W4, u->e3a, u->g_e3a)) != VPT_OK) return s;
    if ((s = run_dw(u, 4, src1(u->p2, 64, N, H4, W4), u->g_e3a)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 4, u->g_e3a, N, H4, W4, nullptr, u->g_p2)) != VPT_OK) return s;
    UCK(u, skip_mask(u->g_cat2, 160, 96, u->g_p2, u->e2, u->g_e2, N, H2, W2, 64, u->stream));
    // e2b, e2a
    if ((s = run_dw(u, 3, src1(u->e2a, 64, N, H2, W2), u->g_e2)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 3, u->g_e2, N, H2, W2, u->e2a, u->g_e2a)) != VPT_OK) return s;
    if ((s = run_dw(u, 2, src1(u->p1, 32, N, H2, W2), u->g_e2a)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 2, u->g_e2a, N, H2, W2, nullptr, u->g_p1)) != VPT_OK) return s;
    UCK(u, skip_mask(u->g_cat1, 96, 64, u->g_p1, u->e1, u->g_e1, N, H, W, 32, u->stream));
    // e1b, e1a
    if ((s = run_dw(u, 1, src1(u->e1a, 32, N, H, W), u->g_e1)) != VPT_OK) return s;
    if ((s = run_conv_bwd(u, 1, u->g_e1, N, H, W, u->e1a, u->g_e1a)) != VPT_OK) return s;
    return run_dw(u, 0, src1(x, 16, N, H, W), u->g_e1a);
}

vpt_status check_err(vpt_unet* u) {
    int e = 0;
    UCK(u, cudaMemcpyAsync(&e, u->errw, sizeof(int), cudaMemcpyDeviceToHost, u->stream));
    UCK(u, cudaStreamSynchronize(u->stream));
    if (e) {
        UCK(u, cudaMemsetAsync(u->errw, 0, sizeof(int), u->stream));
        return ufail(u, VPT_ERR_DEVICE_TIMEOUT, "a tensor-core wait timed out (code %d)", e);
    }
    return VPT_OK;
}

}  // namespace

extern "C" {

vpt_status vpt_nn_conv3x3(const void* in0, int32_t c0, int32_t up0, const void* in1, int32_t c1, int32_t n, int32_t h,
                          int32_t w, const void* weight, const float* bias, int32_t cout, int32_t relu,
                          const void* mask, void* out_bf16, float* out_f32, void* stream) {
    if (!in0 || !weight || (!out_bf16 && !out_f32) || (c1 > 0 && !in1) || n < 1 || h < 1 || w < 1 || c0 < 8 ||
        c1 < 0 || (up0 != 0 && up0 != 1))
        return VPT_ERR_INVALID_ARG;
    int dev = 0;
    cudaGetDevice(&dev);
    ConvArgs a;
    a.in = ConvSrc{(const bf16*)in0, c0, up0, (const bf16*)in1, c1, n, h, w};
    a.scratch = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    if (up0 || c1 > 0) {
        // the assembled two-source input lives for this call, stream-ordered
        void* tmp = nullptr;
        if (cudaMallocAsync(&tmp, (size_t)n * h * w * (c0 + c1) * 2, st) != cudaSuccess) {
            cudaGetLastError();
            return VPT_ERR_OOM;
        }
        a.scratch = (bf16*)tmp;
    }
    a.w = (const bf16*)weight;
    a.bias = bias;
    a.Cin = c0 + c1;
    a.Np = cout;
    a.relu = relu;
    a.mask = (const bf16*)mask;
    a.out = (bf16*)out_bf16;
    a.out_f32 = out_f32;
    a.err = err_word(dev);
    const vpt_status r = from_cuda(conv3x3(a, st));
    if (a.scratch) cudaFreeAsync(a.scratch, st);
    return r;
}

vpt_status vpt_nn_conv3x3_dw(const void* in0, int32_t c0, int32_t up0, const void* in1, int32_t c1, int32_t n,
                             int32_t h, int32_t w, const void* dy, int32_t cout, float* dw, void* stream) {
    if (!in0 || !dy || !dw || (c1 > 0 && !in1) || n < 1 || h < 1 || w < 1 || c0 < 8 || c1 < 0 ||
        (up0 != 0 && up0 != 1))
        return VPT_ERR_INVALID_ARG;
    int dev = 0;
    cudaGetDevice(&dev);
    DwArgs a;
    a.in = ConvSrc{(const bf16*)in0, c0, up0, (const bf16*)in1, c1, n, h, w};
    a.dy = (const bf16*)dy;
    a.Cin = c0 + c1;
    a.Np = cout;
    a.pix_per_cta = 4096;
    a.dw = dw;
    a.err = err_word(dev);
    return from_cuda(conv3x3_dw(a, (cudaStream_t)stream));
}

vpt_status vpt_nn_status(void* stream) {
    int dev = 0;
    cudaGetDevice(&dev);
    int* w = err_word(dev);
    if (!w) return VPT_ERR_CUDA;
    int e = 0;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return VPT_ERR_CUDA;
    if (cudaMemcpy(&e, w, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return VPT_ERR_CUDA;
    if (e) {
        cudaMemset(w, 0, sizeof(int));
        return VPT_ERR_DEVICE_TIMEOUT;
    }
    return VPT_OK;
}

vpt_status vpt_unet_layer_info(int32_t layer, int32_t* cin, int32_t* cout, int32_t* cin_real, int32_t* cout_real,
                               int64_t* offset) {
    if (layer < 0 || layer >= kLayers) return VPT_ERR_INVALID_ARG;
    if (cin) *cin = kNet[layer].cin;
    if (cout) *cout = kNet[layer].cout;
    if (cin_real) *cin_real = kNet[layer].cin_real;
    if (cout_real) *cout_real = kNet[layer].cout_real;
    if (offset) *offset = layer_offset(layer);
    return VPT_OK;
}

vpt_status vpt_unet_create(vpt_unet** out, int32_t device, int32_t max_images, int32_t max_height, int32_t max_width) {
    if (!out) return VPT_ERR_INVALID_ARG;
    *out = nullptr;
    if (max_images < 1 || max_height < 4 || max_width < 4 || (max_height & 3) || (max_width & 3) ||
        (long long)max_images * max_height * max_width > (1LL << 26))
        return VPT_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return VPT_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) return VPT_ERR_INVALID_ARG;
    vpt_unet* u = new (std::nothrow) vpt_unet();
    if (!u) return VPT_ERR_OOM;
    u->dev = device;
    u->maxN = max_images;
    u->maxH = max_height;
    u->maxW = max_width;
    u->nparams = layer_offset(kLayers);
    vpt_status s = VPT_OK;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking) != cudaSuccess)
        s = VPT_ERR_CUDA;
    const size_t P = (size_t)max_images * max_height * max_width, P2 = P / 4, P4 = P / 16;
#define A(ptr, n) \
    if (s == VPT_OK) s = ualloc(u, &(ptr), (n))
    A(u->params, u->nparams);
    A(u->grads, u->nparams);
    A(u->adam_m, u->nparams);
    A(u->adam_v, u->nparams);
    for (int l = 0; l < kLayers; l++) {
        A(u->wf[l], (size_t)kNet[l].cout * 9 * kNet[l].cin);
        A(u->wb[l], (size_t)kNet[l].cout * 9 * kNet[l].cin);
    }
    A(u->e1a, P * 32); A(u->e1, P * 32); A(u->p1, P2 * 32);
    A(u->e2a, P2 * 64); A(u->e2, P2 * 64); A(u->p2, P4 * 64);
    A(u->e3a, P4 * 96); A(u->e3, P4 * 96);
    A(u->d2a, P2 * 64); A(u->d2, P2 * 64); A(u->d1a, P * 32); A(u->d1, P * 32);
    A(u->cat2, P2 * 160); A(u->cat1, P * 96);
    A(u->out, P * 16);
    A(u->g_out, P * 16); A(u->g_d1, P * 32); A(u->g_d1a, P * 32); A(u->g_cat1, P * 96);
    A(u->g_d2, P2 * 64); A(u->g_d2a, P2 * 64); A(u->g_cat2, P2 * 160);
    A(u->g_e3, P4 * 96); A(u->g_e3a, P4 * 96); A(u->g_p2, P4 * 64);
    A(u->g_e2, P2 * 64); A(u->g_e2a, P2 * 64); A(u->g_p1, P2 * 32);
    A(u->g_e1, P * 32); A(u->g_e1a, P * 32);
    A(u->loss, 1);
    A(u->errw, 1);
#undef A
    if (s == VPT_OK) {
        if (cudaMemsetAsync(u->params, 0, sizeof(float) * u->nparams, u->stream) != cudaSuccess ||
            cudaMemsetAsync(u->adam_m, 0, sizeof(float) * u->nparams, u->stream) != cudaSuccess ||
            cudaMemsetAsync(u->adam_v, 0, sizeof(float) * u->nparams, u->stream) != cudaSuccess ||
            cudaMemsetAsync(u->errw, 0, sizeof(int), u->stream) != cudaSuccess ||
            cudaStreamSynchronize(u->stream) != cudaSuccess)
            s = VPT_ERR_CUDA;
    }
    if (s != VPT_OK) {
        vpt_unet_destroy(u);
        return s;
    }
    *out = u;
    return VPT_OK;
}

vpt_status vpt_unet_destroy(vpt_unet* u) {
    if (!u) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(u->dev);
    if (u->stream) cudaStreamSynchronize(u->stream);
    for (void* p : u->allocs) cudaFree(p);
    if (u->stream) cudaStreamDestroy(u->stream);
    delete u;
    return VPT_OK;
}

const char* vpt_unet_last_error(const vpt_unet* u) { return u ? u->err.c_str() : ""; }

vpt_status vpt_unet_param_count(const vpt_unet* u, int64_t* n) {
    if (!u || !n) return VPT_ERR_INVALID_ARG;
    *n = u->nparams;
    return VPT_OK;
}

vpt_status vpt_unet_set_params(vpt_unet* u, const float* host, int64_t n) {
    if (!u) return VPT_ERR_INVALID_ARG;
    if (!host || n != u->nparams) return ufail(u, VPT_ERR_INVALID_ARG, "need %lld parameters", u->nparams);
    cudaSetDevice(u->dev);
    UCK(u, cudaMemcpyAsync(u->params, host, sizeof(float) * n, cudaMemcpyHostToDevice, u->stream));
    UCK(u, cudaMemsetAsync(u->adam_m, 0, sizeof(float) * n, u->stream));
    UCK(u, cudaMemsetAsync(u->adam_v, 0, sizeof(float) * n, u->stream));
    UCK(u, cudaStreamSynchronize(u->stream));
    u->adam_step = 0;
    u->weights_ready = false;
    return VPT_OK;
}

vpt_status vpt_unet_get_params(vpt_unet* u, float* host, int64_t n) {
    if (!u) return VPT_ERR_INVALID_ARG;
    if (!host || n != u->nparams) return ufail(u, VPT_ERR_INVALID_ARG, "need %lld parameters", u->nparams);
    cudaSetDevice(u->dev);
    UCK(u, cudaMemcpyAsync(host, u->params, sizeof(float) * n, cudaMemcpyDeviceToHost, u->stream));
    UCK(u, cudaStreamSynchronize(u->stream));
    return VPT_OK;
}

vpt_status vpt_unet_get_grads(vpt_unet* u, float* host, int64_t n) {
    if (!u) return VPT_ERR_INVALID_ARG;
    if (!host || n != u->nparams) return ufail(u, VPT_ERR_INVALID_ARG, "need %lld values", u->nparams);
    cudaSetDevice(u->dev);
    UCK(u, cudaMemcpyAsync(host, u->grads, sizeof(float) * n, cudaMemcpyDeviceToHost, u->stream));
    UCK(u, cudaStreamSynchronize(u->stream));
    return VPT_OK;
}

vpt_status vpt_unet_forward(vpt_unet* u, const void* input, int32_t n, int32_t h, int32_t w, float* out) {
    if (!u) return VPT_ERR_INVALID_ARG;
    if (!input) return ufail(u, VPT_ERR_INVALID_ARG, "input is NULL");
    vpt_status s = check_shape(u, n, h, w);
    if (s != VPT_OK) return s;
    cudaSetDevice(u->dev);
    if ((s = forward(u, (const bf16*)input, n, h, w)) != VPT_OK) return s;
    if (out)
        UCK(u, cudaMemcpyAsync(out, u->out, sizeof(float) * 16 * (size_t)n * h * w, cudaMemcpyDeviceToDevice,
                               u->stream));
    return VPT_OK;
}

vpt_status vpt_unet_output(vpt_unet* u, const float** out) {
    if (!u || !out) return VPT_ERR_INVALID_ARG;
    *out = u->out;
    return VPT_OK;
}

vpt_status vpt_unet_backward(vpt_unet* u, const void* input, const float* target, int32_t n, int32_t h, int32_t w,
                             double* loss) {
    if (!u) return VPT_ERR_INVALID_ARG;
    if (!input || !target) return ufail(u, VPT_ERR_INVALID_ARG, "input or target is NULL");
    vpt_status s = check_shape(u, n, h, w);
    if (s != VPT_OK) return s;
    cudaSetDevice(u->dev);
    if ((s = forward(u, (const bf16*)input, n, h, w)) != VPT_OK) return s;
    if ((s = backward(u, (const bf16*)input, target, n, h, w)) != VPT_OK) return s;
    if (loss) {
        double l = 0.0;
        UCK(u, cudaMemcpyAsync(&l, u->loss, sizeof(double), cudaMemcpyDeviceToHost, u->stream));
        if ((s = check_err(u)) != VPT_OK) return s;
        *loss = l / (3.0 * (double)n * h * w);
    }
    return VPT_OK;
}

vpt_status vpt_unet_adam(vpt_unet* u, float lr, float beta1, float beta2, float eps) {
    if (!u) return VPT_ERR_INVALID_ARG;
    if (!(lr > 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
        return ufail(u, VPT_ERR_INVALID_ARG, "bad Adam hyper-parameters");
    cudaSetDevice(u->dev);
    u->adam_step++;
    UCK(u, adam(u->params, u->grads, u->adam_m, u->adam_v, u->nparams, lr, beta1, beta2, eps, u->adam_step, u->stream));
    u->weights_ready = false;
    return VPT_OK;
}

vpt_status vpt_unet_synchronize(vpt_unet* u) {
    if (!u) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(u->dev);
    return check_err(u);
}

vpt_status vpt_unet_get_stream(const vpt_unet* u, void** stream) {
    if (!u || !stream) return VPT_ERR_INVALID_ARG;
    *stream = (void*)u->stream;
    return VPT_OK;
}

}  // extern "C"
