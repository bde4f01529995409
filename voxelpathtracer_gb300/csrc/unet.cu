// Kernels of the learned denoiser: 3x3 convolutions as implicit GEMMs on the
// tcgen05 tensor cores (BF16 operands, FP32 accumulation in TMEM), the weight
// gradient as a second tcgen05 GEMM over pixels, and the small elementwise
// steps around them (pooling, upsampling gradients, loss, Adam).
//
// Activations are BF16, NHWC, channels padded to a multiple of 16. A
// convolution reads up to two sources: channels [0, C0) from `p0`, optionally
// at half resolution (nearest upsampling), and channels [C0, C0 + C1) from
// `p1` at full resolution, which fuses the U-Net's upsample-and-concatenate
// into the operand staging.
//
// Forward and backward-data convolution (k_conv3x3): one CTA of 128 threads
// computes 128 consecutive pixels of one image row for all Np output
// channels: GEMM M = 128 pixels, N = Np, K = 9 taps x Cin. For each tap the
// 128 x Cin input rows and the Np x Cin weights are staged into shared memory
// (two stages, so the loads of tap t+1 overlap the MMAs of tap t), one
// thread issues Cin / 16 MMAs into the TMEM accumulator and commits them to
// the stage's mbarrier, and the epilogue reads TMEM (warp w: pixels
// 32w..32w+31), adds the bias, applies ReLU or a ReLU-derivative mask and
// stores BF16 (or FP32). Backward-data is the same kernel with the weights
// transposed and the taps flipped.
//
// Weight gradient (k_conv3x3_dw): dW[co][tap][ci] = sum_p dY[p][co] X[p+tap][ci].
// One CTA handles one tap and a range of pixels: GEMM M = 128 (co, zero
// padded), N = Cin, K = pixels, staged 128 pixels at a time by transposing
// the NHWC rows into K-major tiles; partial sums are added to FP32 dW with
// atomics.
//
// Every mbarrier wait has an iteration limit; on timeout the kernel records
// an error code, stops issuing MMAs, waits once more (bounded) and frees its
// TMEM before returning.
#include <cuda_bf16.h>

#include <algorithm>

#include "tc.cuh"
#include "unet.cuh"

namespace vpt {

namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint4 ldg16(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }

// 8 channels [c, c+8) of the (virtual) concatenated input at pixel (n, y, x);
// zero outside the image (the convolution's zero padding).
__device__ __forceinline__ uint4 load8(const ConvSrc& s, int n, int y, int x, int c) {
    if (y < 0 || y >= s.H || x < 0 || x >= s.W) return make_uint4(0u, 0u, 0u, 0u);
    if (c < s.C0) {
        const int H0 = s.H >> s.up0, W0 = s.W >> s.up0;
        const size_t px = ((size_t)n * H0 + (y >> s.up0)) * W0 + (x >> s.up0);
        return ldg16(s.p0 + px * s.C0 + c);
    }
    const size_t px = ((size_t)n * s.H + y) * s.W + x;
    return ldg16(s.p1 + px * s.C1 + (c - s.C0));
}

__host__ __device__ __forceinline__ uint32_t tmem_columns(int n) {
    uint32_t c = 32;
    while ((int)c < n) c <<= 1;
    return c;
}

__device__ __forceinline__ void unpack8(uint4 u, float* f) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float2 t = __bfloat1622float2(h[k]);
        f[2 * k] = t.x;
        f[2 * k + 1] = t.y;
    }
}
__device__ __forceinline__ uint4 pack8(const float* f) {
    uint4 u;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
    for (int k = 0; k < 4; k++) h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
    return u;
}

__global__ void __launch_bounds__(128, 1) k_conv3x3(ConvArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t s_taddr;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = blockIdx.z, y = blockIdx.y, x0 = blockIdx.x * 128;
    const int K = a.Cin, Np = a.Np, kch = K >> 3;
    const uint32_t abytes = 128u * K * 2u, bbytes = (uint32_t)Np * K * 2u, stage = abytes + bbytes;
    const uint32_t ncols = tmem_columns(Np);
    const uint32_t bar0 = tc::smem_addr(&bars[0]), bar1 = tc::smem_addr(&bars[1]);
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&s_taddr), ncols);
    if (tid == 0) {
        tc::mbar_init(bar0, 1);
        tc::mbar_init(bar1, 1);
        tc::mbar_init_fence();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = s_taddr;
    const uint32_t idesc = tc::idesc_bf16(128, Np);
    bool ok = true;
    for (int tap = 0; tap < 9; tap++) {
        const int st = tap & 1;
        const uint32_t bar = st ? bar1 : bar0;
        if (tap >= 2) ok = tc::mbar_wait(bar, (uint32_t)(((tap >> 1) - 1) & 1), a.err, 1);
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        uint8_t* sa = smem + st * stage;
        uint8_t* sb = sa + abytes;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        for (int idx = tid; idx < 128 * kch; idx += 128) {
            const int m = idx / kch, c8 = idx - m * kch;
            *reinterpret_cast<uint4*>(sa + tc::tile_offset(m, c8 * 8, K)) =
                load8(a.in, n, y + dy, x0 + m + dx, c8 * 8);
        }
        for (int idx = tid; idx < Np * kch; idx += 128) {
            const int r = idx / kch, c8 = idx - r * kch;
            *reinterpret_cast<uint4*>(sb + tc::tile_offset(r, c8 * 8, K)) =
                ldg16(a.w + ((size_t)r * 9 + tap) * K + c8 * 8);
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_addr(sa), b0 = tc::smem_addr(sb);
            const uint32_t sbo = (uint32_t)K * 16u;
            for (int k = 0; k < K / 16; k++)
                tc::mma_bf16(taddr, tc::smem_desc(a0 + 256u * k, 128u, sbo), tc::smem_desc(b0 + 256u * k, 128u, sbo),
                             idesc, (tap | k) != 0 ? 1u : 0u);
            tc::mma_commit(bar);
        }
    }
    // the commit of tap 8 (stage 0, its fifth phase) covers every MMA issued
    if (ok) ok = tc::mbar_wait(bar0, 0u, a.err, 2);
    else tc::mbar_wait(bar0, 0u, nullptr, 0);
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    const int m = warp * 32 + lane, x = x0 + m;
    const bool valid = ok && x < a.in.W;
    const size_t p = ((size_t)n * a.in.H + y) * a.in.W + x;
    for (int c0 = 0; c0 < Np; c0 += 16) {
        float v[16];
        tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (!valid) continue;
        if (a.bias) {
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] += __ldg(a.bias + c0 + k);
        }
        if (a.relu) {
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] = fmaxf(v[k], 0.0f);
        }
        if (a.mask) {
            float mk[16];
            unpack8(ldg16(a.mask + p * Np + c0), mk);
            unpack8(ldg16(a.mask + p * Np + c0 + 8), mk + 8);
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] = mk[k] > 0.0f ? v[k] : 0.0f;
        }
        if (a.out) {
            uint4* o = reinterpret_cast<uint4*>(a.out + p * Np + c0);
            o[0] = pack8(v);
            o[1] = pack8(v + 8);
        }
        if (a.out_f32) {
            float4* o = reinterpret_cast<float4*>(a.out_f32 + p * Np + c0);
#pragma unroll
            for (int k = 0; k < 4; k++) o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(taddr, ncols);
}

__global__ void __launch_bounds__(128, 1) k_conv3x3_dw(DwArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t s_taddr;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap = blockIdx.y, dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int K = 128;                         // pixels per stage
    const int N = a.Cin, Np = a.Np;
    const uint32_t abytes = 128u * K * 2u, bbytes = (uint32_t)N * K * 2u, stage = abytes + bbytes;
    const uint32_t ncols = tmem_columns(N);
    const uint32_t bar0 = tc::smem_addr(&bars[0]), bar1 = tc::smem_addr(&bars[1]);
    const long long HW = (long long)a.in.H * a.in.W, P = HW * a.in.N;
    const long long pbeg = (long long)blockIdx.x * a.pix_per_cta;
    const int chunks = (int)((min((long long)a.pix_per_cta, P - pbeg) + K - 1) / K);
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&s_taddr), ncols);
    if (tid == 0) {
        tc::mbar_init(bar0, 1);
        tc::mbar_init(bar1, 1);
        tc::mbar_init_fence();
    }
    // rows Np..127 of both A stages stay zero
    for (int s = 0; s < 2; s++) {
        uint4* za = reinterpret_cast<uint4*>(smem + s * stage);
        for (int k = tid; k < (int)(abytes / 16); k += 128) za[k] = make_uint4(0u, 0u, 0u, 0u);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = s_taddr;
    const uint32_t idesc = tc::idesc_bf16(128, N);
    bool ok = true;
    for (int c = 0; c < chunks; c++) {
        const int st = c & 1;
        const uint32_t bar = st ? bar1 : bar0;
        if (c >= 2) ok = tc::mbar_wait(bar, (uint32_t)(((c >> 1) - 1) & 1), a.err, 3);
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        uint8_t* sa = smem + st * stage;
        uint8_t* sb = sa + abytes;
        // thread tid stages pixel p (K index tid): its dY row into A, its shifted X row into B
        const long long p = pbeg + (long long)c * K + tid;
        const bool inside = p < P;
        int n = 0, y = 0, x = 0;
        if (inside) {
            n = (int)(p / HW);
            const long long r = p - (long long)n * HW;
            y = (int)(r / a.in.W);
            x = (int)(r - (long long)y * a.in.W);
        }
        bf16* A = reinterpret_cast<bf16*>(sa);
        bf16* B = reinterpret_cast<bf16*>(sb);
        for (int c8 = 0; c8 < Np; c8 += 8) {
            uint4 u = inside ? ldg16(a.dy + (size_t)p * Np + c8) : make_uint4(0u, 0u, 0u, 0u);
            const bf16* h = reinterpret_cast<const bf16*>(&u);
#pragma unroll
            for (int k = 0; k < 8; k++) A[tc::tile_offset(c8 + k, tid, K) / 2] = h[k];
        }
        for (int c8 = 0; c8 < N; c8 += 8) {
            uint4 u = inside ? load8(a.in, n, y + dy, x + dx, c8) : make_uint4(0u, 0u, 0u, 0u);
            const bf16* h = reinterpret_cast<const bf16*>(&u);
#pragma unroll
            for (int k = 0; k < 8; k++) B[tc::tile_offset(c8 + k, tid, K) / 2] = h[k];
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_addr(sa), b0 = tc::smem_addr(sb);
            const uint32_t sbo = (uint32_t)K * 16u;
            for (int k = 0; k < K / 16; k++)
                tc::mma_bf16(taddr, tc::smem_desc(a0 + 256u * k, 128u, sbo), tc::smem_desc(b0 + 256u * k, 128u, sbo),
                             idesc, (c | k) != 0 ? 1u : 0u);
            tc::mma_commit(bar);
        }
    }
    if (chunks > 0) {
        // the last commit went to stage (chunks-1)&1, its ((chunks-1)>>1)-th phase
        const int last = chunks - 1;
        const uint32_t bar = (last & 1) ? bar1 : bar0;
        const uint32_t par = (uint32_t)((last >> 1) & 1);
        if (ok) ok = tc::mbar_wait(bar, par, a.err, 4);
        else tc::mbar_wait(bar, par, nullptr, 0);
    }
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    const int co = warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (!ok || chunks == 0 || co >= Np) continue;
        float* d = a.dw + ((size_t)co * 9 + tap) * N + c0;
#pragma unroll
        for (int k = 0; k < 16; k++) atomicAdd(d + k, v[k]);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(taddr, ncols);
}

// ------------------------------------------------------------ elementwise --
// 2x2 average pooling (FP32 sum of the four BF16 values, one rounding).
__global__ void k_pool2(const bf16* in, bf16* out, int N, int H, int W, int C) {
    const int H2 = H >> 1, W2 = W >> 1, c8n = C >> 3;
    const long long total = (long long)N * H2 * W2 * c8n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % c8n);
        const long long q = i / c8n;
        const int x = (int)(q % W2), y = (int)((q / W2) % H2), n = (int)(q / ((long long)W2 * H2));
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int d = 0; d < 4; d++) {
            const size_t src = (((size_t)n * H + 2 * y + (d >> 1)) * W + 2 * x + (d & 1)) * C + c8 * 8;
            float f[8];
            unpack8(ldg16(in + src), f);
#pragma unroll
            for (int k = 0; k < 8; k++) s[k] += f[k];
        }
#pragma unroll
        for (int k = 0; k < 8; k++) s[k] *= 0.25f;
        *reinterpret_cast<uint4*>(out + (size_t)q * C + c8 * 8) = pack8(s);
    }
}

// Gradient of nearest 2x upsampling (sum of the 2x2 children) of channels
// [off, off+C) of g (Cg channels, full resolution), times (act > 0).
__global__ void k_upsum_mask(const bf16* g, int Cg, int off, const bf16* act, bf16* out, int N, int H, int W, int C) {
    const int H2 = H >> 1, W2 = W >> 1, c8n = C >> 3;
    const long long total = (long long)N * H2 * W2 * c8n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % c8n);
        const long long q = i / c8n;
        const int x = (int)(q % W2), y = (int)((q / W2) % H2), n = (int)(q / ((long long)W2 * H2));
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int d = 0; d < 4; d++) {
            const size_t src = (((size_t)n * H + 2 * y + (d >> 1)) * W + 2 * x + (d & 1)) * Cg + off + c8 * 8;
            float f[8];
            unpack8(ldg16(g + src), f);
#pragma unroll
            for (int k = 0; k < 8; k++) s[k] += f[k];
        }
        float m[8];
        unpack8(ldg16(act + (size_t)q * C + c8 * 8), m);
#pragma unroll
        for (int k = 0; k < 8; k++) s[k] = m[k] > 0.0f ? s[k] : 0.0f;
        *reinterpret_cast<uint4*>(out + (size_t)q * C + c8 * 8) = pack8(s);
    }
}

// (channels [off, off+C) of g + gpool[p/2] / 4) times (act > 0): the gradient
// of a skip tensor that feeds both a concatenation and a 2x2 pooling.
__global__ void k_skip_mask(const bf16* g, int Cg, int off, const bf16* gpool, const bf16* act, bf16* out, int N,
                            int H, int W, int C) {
    const int c8n = C >> 3;
    const long long total = (long long)N * H * W * c8n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % c8n);
        const long long q = i / c8n;
        const int x = (int)(q % W), y = (int)((q / W) % H), n = (int)(q / ((long long)W * H));
        float a[8], b[8], m[8];
        unpack8(ldg16(g + (size_t)q * Cg + off + c8 * 8), a);
        const size_t pq = ((size_t)n * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1);
        unpack8(ldg16(gpool + pq * C + c8 * 8), b);
        unpack8(ldg16(act + (size_t)q * C + c8 * 8), m);
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = m[k] > 0.0f ? a[k] + 0.25f * b[k] : 0.0f;
        *reinterpret_cast<uint4*>(out + (size_t)q * C + c8 * 8) = pack8(a);
    }
}

// Mean squared error over the first 3 of 16 output channels against the
// target (3 channels FP32); writes dL/dout as BF16 (zero in channels 3..15)
// and adds the squared-error sum to *loss.
__global__ void k_mse_grad(const float* out, const float* target, bf16* g, long long P, float scale, double* loss) {
    double acc = 0.0;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P;
         p += (long long)gridDim.x * blockDim.x) {
        float gv[16];
#pragma unroll
        for (int k = 0; k < 16; k++) gv[k] = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float d = out[p * 16 + k] - target[p * 3 + k];
            acc += (double)d * d;
            gv[k] = 2.0f * d * scale;
        }
        uint4* o = reinterpret_cast<uint4*>(g + p * 16);
        o[0] = pack8(gv);
        o[1] = pack8(gv + 8);
    }
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// Sum over pixels of a BF16 gradient: the bias gradient.
__global__ void k_bias_grad(const bf16* g, long long P, int C, float* db) {
    const int c = threadIdx.x % C;
    const int lanes = blockDim.x / C;
    float acc = 0.0f;
    for (long long p = (long long)blockIdx.x * lanes + threadIdx.x / C; p < P; p += (long long)gridDim.x * lanes)
        acc += __bfloat162float(g[p * C + c]);
    if (threadIdx.x < lanes * C) atomicAdd(db + c, acc);
}

// Adam on the FP32 master parameters; also writes the BF16 forward weights
// and the tap-flipped, transposed BF16 weights of the backward-data conv.
__global__ void k_adam(float* w, const float* grad, float* m, float* v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// BF16 copies of one layer's FP32 weights [Np][9][Cin]: forward layout and
// the backward-data layout [Cin][9][Np] with the taps flipped.
__global__ void k_weights_bf16(const float* w, bf16* wf, bf16* wb, int Np, int Cin) {
    const int total = Np * 9 * Cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int ci = i % Cin, tap = (i / Cin) % 9, co = i / (9 * Cin);
        const bf16 h = __float2bfloat16_rn(w[i]);
        wf[i] = h;
        wb[((size_t)ci * 9 + (8 - tap)) * Np + co] = h;
    }
}

}  // namespace

size_t conv3x3_smem(int Cin, int Np) { return 2u * (128u * Cin * 2u + (size_t)Np * Cin * 2u); }
size_t conv3x3_dw_smem(int Cin) { return 2u * (128u * 128u * 2u + (size_t)Cin * 128u * 2u); }

cudaError_t conv3x3(const ConvArgs& a, cudaStream_t s) {
    if (a.Cin != a.in.C0 + a.in.C1 || a.Cin % 16 || a.Cin < 16 || a.Cin > 256 || a.Np % 16 || a.Np < 16 ||
        a.Np > 256 || (a.in.up0 && ((a.in.H | a.in.W) & 1)) || (a.in.C0 % 8) || (a.in.C1 % 8))
        return cudaErrorInvalidValue;
    const size_t sm = conv3x3_smem(a.Cin, a.Np);
    if (sm > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.in.W + 127) / 128), (unsigned)a.in.H, (unsigned)a.in.N);
    k_conv3x3<<<grid, 128, sm, s>>>(a);
    return cudaGetLastError();
}

cudaError_t conv3x3_dw(const DwArgs& a, cudaStream_t s) {
    if (a.Cin != a.in.C0 + a.in.C1 || a.Cin % 16 || a.Cin < 16 || a.Cin > 256 || a.Np % 8 || a.Np < 8 ||
        a.Np > 128 || a.pix_per_cta < 128 || a.pix_per_cta % 128 || (a.in.up0 && ((a.in.H | a.in.W) & 1)))
        return cudaErrorInvalidValue;
    const size_t sm = conv3x3_dw_smem(a.Cin);
    cudaError_t e = cudaFuncSetAttribute(k_conv3x3_dw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const long long P = (long long)a.in.N * a.in.H * a.in.W;
    dim3 grid((unsigned)((P + a.pix_per_cta - 1) / a.pix_per_cta), 9);
    k_conv3x3_dw<<<grid, 128, sm, s>>>(a);
    return cudaGetLastError();
}

static unsigned ew_grid(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16); }

cudaError_t pool2(const bf16* in, bf16* out, int N, int H, int W, int C, cudaStream_t s) {
    k_pool2<<<ew_grid((long long)N * (H / 2) * (W / 2) * (C / 8)), 256, 0, s>>>(in, out, N, H, W, C);
    return cudaGetLastError();
}
cudaError_t upsum_mask(const bf16* g, int Cg, int off, const bf16* act, bf16* out, int N, int H, int W, int C,
                       cudaStream_t s) {
    k_upsum_mask<<<ew_grid((long long)N * (H / 2) * (W / 2) * (C / 8)), 256, 0, s>>>(g, Cg, off, act, out, N, H, W, C);
    return cudaGetLastError();
}
cudaError_t skip_mask(const bf16* g, int Cg, int off, const bf16* gpool, const bf16* act, bf16* out, int N, int H,
                      int W, int C, cudaStream_t s) {
    k_skip_mask<<<ew_grid((long long)N * H * W * (C / 8)), 256, 0, s>>>(g, Cg, off, gpool, act, out, N, H, W, C);
    return cudaGetLastError();
}
cudaError_t mse_grad(const float* out, const float* target, bf16* g, long long P, float scale, double* loss,
                     cudaStream_t s) {
    k_mse_grad<<<ew_grid(P), 256, 0, s>>>(out, target, g, P, scale, loss);
    return cudaGetLastError();
}
cudaError_t bias_grad(const bf16* g, long long P, int C, float* db, cudaStream_t s) {
    const int per = 256 / C;
    k_bias_grad<<<ew_grid(P / per + 1), per * C, 0, s>>>(g, P, C, db);
    return cudaGetLastError();
}
cudaError_t adam(float* w, const float* grad, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                 int step, cudaStream_t s) {
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    k_adam<<<ew_grid(n), 256, 0, s>>>(w, grad, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}
cudaError_t weights_bf16(const float* w, bf16* wf, bf16* wb, int Np, int Cin, cudaStream_t s) {
    k_weights_bf16<<<ew_grid((long long)Np * 9 * Cin), 256, 0, s>>>(w, wf, wb, Np, Cin);
    return cudaGetLastError();
}

}  // namespace vpt
