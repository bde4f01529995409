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
// Forward and backward-data convolution (k_conv3x3): GEMM M = 128 pixels of
// one image row, N = Np output channels, K = 9 taps x Cin, in persistent
// warp-specialised CTAs: a TMA producer fills a ring of shared-memory stages
// (one (tap, channel chunk) each; TMA's zero fill is the convolution's
// padding), one thread issues the tcgen05 MMAs into double-buffered TMEM
// accumulators, and four epilogue warps add the bias, apply ReLU or a
// ReLU-derivative mask and store BF16 (or FP32) while the next tile's MMAs
// run. Backward-data is the same kernel with the weights transposed and the
// taps flipped. A two-source input is assembled into a scratch tensor first.
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

#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <mutex>

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


constexpr int kConvStages = 8;   // most shared-memory stages of (tap, channel chunk) operand tiles

// Persistent, warp-specialised forward / backward-data convolution with TMA.
// Operands sit in shared memory as TMA writes them: a box of (KC channels,
// R rows) is R rows of KC * 2 bytes (64 or 32) with the 64- or 32-byte
// swizzle, which the tensor core reads through a swizzled K-major descriptor
// (8-row atoms 8 * KC * 2 bytes apart; a K step of 16 channels advances the
// start by 32 bytes).
//   warp 0      one lane: loads the weights of all 9 taps once (when they fit,
//               `w_resident`), then for each (tap, channel chunk) stage of each
//               tile issues the TMA box of the 128 input pixels x + dx of row
//               y + dy (zero outside the image) - and the chunk's weights when
//               they are not resident - into a ring of S <= kConvStages, announcing
//               the bytes on the stage's `full` barrier.
//   warp 1      one lane issues the stage's tcgen05 MMAs into one of two TMEM
//               accumulators and releases the stage with a commit to `empty`;
//               after a tile's last stage it commits `acc_full`.
//   warps 2-5   epilogue: wait `acc_full`, read their 32 TMEM lanes, add bias,
//               apply ReLU / mask, store, arrive on `acc_empty`, overlapping the
//               next tile's MMAs in the other accumulator.
// CTAs loop over 128-pixel row tiles (x fastest, so neighbouring CTAs share
// input rows in L2).
// Two-source inputs (`split` > 0: channels [0, split) from a half-resolution
// tensor upsampled by nearest neighbour, the rest from a full-resolution one)
// are staged without assembling the concatenation: a tile's 128 accumulator
// rows are its 64 even pixels, then its 64 odd ones. For tap dx the even
// pixels x0 + 2m read input column x0 + 2m + dx, i.e. half-resolution column
// m0 + m + floor(dx / 2) and full-resolution pixel (m0 + m + floor(dx / 2),
// parity dx & 1); the odd ones the same with dx + 1. So each half is one
// 64-pixel box: from `tm_in` (the half-resolution tensor) or from `tm_in2`
// (the full-resolution tensor as (channel, parity, x / 2, y, image)), and the
// epilogue stores row r to pixel x0 + 2 (r % 64) + r / 64.
constexpr int kConvThreads = 192;
__global__ void __launch_bounds__(kConvThreads, 1)
    k_conv3x3(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_w,
              const __grid_constant__ CUtensorMap tm_in2, ConvArgs a, int KC, int ntiles, int tiles_x, int w_resident,
              int box_w, int S, int split) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[kConvStages], empty[kConvStages], acc_full[2], acc_empty[2], wbar;
    __shared__ uint32_t s_taddr;
    __shared__ volatile int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = a.Cin, Np = a.Np, H = a.in.H, W = a.in.W;
    const int nkc = K / KC, nit = 9 * nkc;
    const uint32_t wbytes = w_resident ? 9u * K * Np * 2u : 0u;
    const uint32_t abytes = 128u * KC * 2u, bbytes = w_resident ? 0u : (uint32_t)Np * KC * 2u;
    const uint32_t stage = abytes + bbytes;
    const uint32_t rb = (uint32_t)KC * 2u;          // bytes of one operand row
    const uint32_t nblk = (uint32_t)Np * rb;        // bytes of one Np x KC weight block
    // bytes one stage's boxes deliver (a box is box_w <= 128 pixels wide; rows
    // past it hold stale data that only feeds accumulator rows the epilogue skips)
    const uint32_t stage_tx = (split > 0 ? 128u : (uint32_t)box_w) * rb + bbytes;
    const uint32_t ncols = tmem_columns(2 * Np);
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&s_taddr), ncols);
    if (tid == 0) {
        for (int k = 0; k < kConvStages; k++) {
            tc::mbar_init(tc::smem_addr(&full[k]), 1);
            tc::mbar_init(tc::smem_addr(&empty[k]), 1);
        }
        for (int k = 0; k < 2; k++) {
            tc::mbar_init(tc::smem_addr(&acc_full[k]), 1);
            tc::mbar_init(tc::smem_addr(&acc_empty[k]), 128);
        }
        tc::mbar_init(tc::smem_addr(&wbar), 1);
        s_abort = 0;
        tc::mbar_init_fence();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = s_taddr;
    const uint32_t wbase = tc::smem_addr(smem), ring = wbase + wbytes;

    if (warp == 0) {
        // ---------------------------------------------------------- producer
        if (lane == 0) {
            if (w_resident) {
                // block (tap, chunk c) of Np rows x KC channels at (tap * nkc + c) * nblk
                tc::mbar_expect_tx(tc::smem_addr(&wbar), wbytes);
                for (int tap = 0; tap < 9; tap++)
                    for (int c = 0; c < nkc; c++)
                        tc::tma_load_3d(wbase + (uint32_t)(tap * nkc + c) * nblk, &tm_w, c * KC, tap, 0,
                                        tc::smem_addr(&wbar));
            }
            int j = 0;
            for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
                const int xb = tile % tiles_x, ry = tile / tiles_x;
                const int y = ry % H, n = ry / H, x0 = xb * 128;
                bool ok = true;
                for (int it = 0; it < nit; it++, j++) {
                    const int st = j % S;
                    if (j >= S &&
                        !tc::mbar_wait_or_abort(tc::smem_addr(&empty[st]), (uint32_t)(((j / S) - 1) & 1),
                                                a.err, 1, &s_abort)) {
                        ok = false;
                        break;
                    }
                    const int tap = it / nkc, c0 = (it - tap * nkc) * KC;
                    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
                    const uint32_t sa = ring + st * stage, sb = sa + abytes;
                    const uint32_t bar = tc::smem_addr(&full[st]);
                    tc::mbar_expect_tx(bar, stage_tx);
                    if (split > 0) {
                        const int m0 = x0 >> 1, e = dx >> 1, o = (dx + 1) >> 1;   // floor(dx / 2), floor((dx + 1) / 2)
                        if (c0 < split) {
                            tc::tma_load_4d(sa, &tm_in, c0, m0 + e, (y + dy) >> 1, n, bar);
                            tc::tma_load_4d(sa + 64u * rb, &tm_in, c0, m0 + o, (y + dy) >> 1, n, bar);
                        } else {
                            tc::tma_load_5d(sa, &tm_in2, c0 - split, dx & 1, m0 + e, y + dy, n, bar);
                            tc::tma_load_5d(sa + 64u * rb, &tm_in2, c0 - split, (dx + 1) & 1, m0 + o, y + dy, n, bar);
                        }
                    } else {
                        tc::tma_load_4d(sa, &tm_in, c0, x0 + dx, y + dy, n, bar);
                    }
                    if (!w_resident) tc::tma_load_3d(sb, &tm_w, c0, tap, 0, bar);
                }
                if (!ok) break;
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issue
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, Np);
            const uint64_t adesc0 = tc::smem_desc_sw(ring, rb), wdesc0 = tc::smem_desc_sw(wbase, rb);
            int j = 0, tcount = 0;
            bool ok = !w_resident || tc::mbar_wait_or_abort(tc::smem_addr(&wbar), 0u, a.err, 5, &s_abort);
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, tcount++) {
                const int buf = tcount & 1;
                if (tcount >= 2 &&
                    !tc::mbar_wait_or_abort(tc::smem_addr(&acc_empty[buf]), (uint32_t)(((tcount >> 1) - 1) & 1),
                                            a.err, 2, &s_abort))
                    break;
                tc::fence_after_sync();
                const uint32_t d = taddr + (uint32_t)(buf * Np);
                for (int it = 0; it < nit; it++, j++) {
                    const int st = j % S;
                    if (!tc::mbar_wait_or_abort(tc::smem_addr(&full[st]), (uint32_t)((j / S) & 1), a.err, 3,
                                                &s_abort)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const int tap = it / nkc, c = it - tap * nkc;
                    // descriptors differ only in the start-address field (address >> 4)
                    const uint64_t ad = adesc0 + ((st * stage) >> 4);
                    const uint64_t bd = w_resident ? wdesc0 + (((uint32_t)(tap * nkc + c) * nblk) >> 4)
                                                   : adesc0 + ((st * stage + abytes) >> 4);
                    for (int k = 0; k < KC / 16; k++)
                        tc::mma_bf16(d, ad + (uint64_t)(2u * k), bd + (uint64_t)(2u * k), idesc, (it | k) != 0 ? 1u : 0u);
                    tc::mma_commit(tc::smem_addr(&empty[st]));
                }
                if (ok) tc::mma_commit(tc::smem_addr(&acc_full[buf]));
            }
        }
        __syncwarp();
    } else {
        // ---------------------------------------------------------- epilogue
        const int q = warp & 3;                 // TMEM lane quarter of this warp
        const int m = q * 32 + lane;
        int tcount = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, tcount++) {
            const int buf = tcount & 1;
            if (!tc::mbar_wait_or_abort(tc::smem_addr(&acc_full[buf]), (uint32_t)((tcount >> 1) & 1), a.err, 4,
                                        &s_abort))
                break;
            tc::fence_after_sync();
            const int xb = tile % tiles_x, ry = tile / tiles_x;
            const int y = ry % H, n = ry / H, x = xb * 128 + (split > 0 ? 2 * (m & 63) + (m >> 6) : m);
            const bool valid = x < W;
            const size_t p = ((size_t)n * H + y) * W + x;
            for (int c0 = 0; c0 < Np; c0 += 16) {
                float v[16];
                tc::tmem_ld16(taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * Np + c0), v);
                if (!valid) continue;
                if (a.bias) {
                    const float4* bb = reinterpret_cast<const float4*>(a.bias + c0);
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const float4 b4 = __ldg(bb + k);
                        v[4 * k] += b4.x;
                        v[4 * k + 1] += b4.y;
                        v[4 * k + 2] += b4.z;
                        v[4 * k + 3] += b4.w;
                    }
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
            tc::mbar_arrive(tc::smem_addr(&acc_empty[buf]));
        }
    }
    // on an abort, give copies and MMAs still in flight a bounded moment before TMEM is freed
    if (s_abort && warp == 1 && lane == 0) {
        for (int k = 0; k < kConvStages; k++) {
            tc::mbar_wait(tc::smem_addr(&full[k]), 0u, nullptr, 0);
            tc::mbar_wait(tc::smem_addr(&empty[k]), 0u, nullptr, 0);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(taddr, ncols);
}

// 16-byte global -> shared copy; src_bytes 0 writes zeros.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
// One arrival on the mbarrier (not counted in its expected arrivals) once
// every cp.async this thread issued before has landed.
__device__ __forceinline__ void cp_async_arrive(uint32_t bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

constexpr int kRowBufs = 6;       // most resident input rows per CTA
constexpr int kRowThreads = 288;  // 4 loader warps, 1 MMA warp, 4 epilogue warps

// Row-resident convolution for layers whose weights fit in shared memory.
// A CTA walks down vertical strips (a 128-pixel column tile, R output rows);
// every input row segment x0-1 .. x0+128 is fetched once into a ring of
// `nb` row buffers and serves three output rows and all three dx taps: the
// tap (dy, dx) operand of output row y is row buffer (y + dy) read through a
// descriptor that starts dx + 1 pixels in. A row buffer holds the segment as
// K/8 blocks of 130 pixels x 8 channels (16 bytes a pixel), i.e. the
// canonical K-major layout without swizzle (SBO = 128, LBO = 2080), in which a
// one-pixel shift is a 16-byte start offset.
//   warps 0-3   loaders: one thread issues a TMA box per input row (a 5-D
//               map of the NHWC input ordered channel-in-group, pixel, group,
//               row, image, so the box arrives in the row buffer's layout;
//               zero outside the image) on the buffer's `row_full` barrier;
//               for images narrower than the box and for two-source inputs
//               (the decoder's upsample-and-concatenate, whose half-resolution
//               pixels appear twice in a row) the four warps issue 16-byte
//               cp.async copies from the sources instead.
//   warp 4      one lane: 9 taps x K/16 MMAs per output row into one of two
//               TMEM accumulators, commits `acc_full`, and releases input row
//               y - 1 (its last use) with a commit to `row_empty`.
//   warps 5-8   epilogue, as in k_conv3x3.
__global__ void __launch_bounds__(kRowThreads, 1)
    k_conv3x3_rows(const __grid_constant__ CUtensorMap tm_w, const __grid_constant__ CUtensorMap tm_in, ConvArgs a,
                   int R, int nstrips, int tiles_x, int nb, int tma_rows) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t row_full[kRowBufs], row_empty[kRowBufs], acc_full[2], acc_empty[2], wbar;
    __shared__ uint32_t s_taddr;
    __shared__ volatile int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = a.Cin, Np = a.Np, H = a.in.H, W = a.in.W, G = K / 8;
    const int strips_y = (H + R - 1) / R;
    const uint32_t wbytes = 9u * K * Np * 2u;
    const uint32_t nblk = (uint32_t)Np * 16u;        // one Np x 8-channel weight block
    const uint32_t rowb = ((uint32_t)G * 2080u + 127u) & ~127u;   // one row buffer, 128-byte aligned
    const uint32_t ncols = tmem_columns(2 * Np);
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&s_taddr), ncols);
    if (tid == 0) {
        for (int k = 0; k < kRowBufs; k++) {
            tc::mbar_init(tc::smem_addr(&row_full[k]), tma_rows ? 1 : 128);
            tc::mbar_init(tc::smem_addr(&row_empty[k]), 1);
        }
        for (int k = 0; k < 2; k++) {
            tc::mbar_init(tc::smem_addr(&acc_full[k]), 1);
            tc::mbar_init(tc::smem_addr(&acc_empty[k]), 128);
        }
        tc::mbar_init(tc::smem_addr(&wbar), 1);
        s_abort = 0;
        tc::mbar_init_fence();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = s_taddr;
    const uint32_t wbase = tc::smem_addr(smem), rbase = wbase + wbytes;
    const bf16* in = a.in.p0;

    if (warp < 4) {
        // ---------------------------------------------------------- loaders
        if (tid == 0) {
            tc::mbar_expect_tx(tc::smem_addr(&wbar), wbytes);
            for (int tap = 0; tap < 9; tap++)
                for (int g = 0; g < G; g++)
                    tc::tma_load_3d(wbase + (uint32_t)(tap * G + g) * nblk, &tm_w, g * 8, tap, 0, tc::smem_addr(&wbar));
        }
        int L = 0;
        bool ok = true;
        // one TMA box per input row (8 channels x 130 pixels x K/8 groups, zero
        // outside the image), issued by one thread; else 16-byte cp.async by
        // the four loader warps
        const bool loader = !tma_rows || tid == 0;
        for (int strip = blockIdx.x; strip < nstrips && ok && loader; strip += gridDim.x) {
            const int xb = strip % tiles_x, rest = strip / tiles_x;
            const int ys = (rest % strips_y) * R, n = rest / strips_y;
            const int ye = min(ys + R, H);
            const int x0 = xb * 128;
            for (int yy = ys - 1; yy <= ye; yy++, L++) {
                const int b = L % nb;
                if (L >= nb &&
                    !tc::mbar_wait_or_abort(tc::smem_addr(&row_empty[b]), (uint32_t)(((L / nb) - 1) & 1), a.err, 6,
                                            &s_abort)) {
                    ok = false;
                    break;
                }
                const uint32_t dst = rbase + (uint32_t)b * rowb;
                if (tma_rows) {
                    tc::mbar_expect_tx(tc::smem_addr(&row_full[b]), (uint32_t)G * 2080u);
                    tc::tma_load_5d(dst, &tm_in, 0, x0 - 1, 0, yy, n, tc::smem_addr(&row_full[b]));
                    continue;
                }
                const bool yin = yy >= 0 && yy < H;
                const int C0 = a.in.C0, C1 = a.in.C1, up = a.in.up0;
                const int W0 = W >> up, yc = yin ? yy : 0;
                const bf16* row0 = in + ((size_t)n * (H >> up) + (yc >> up)) * W0 * C0;
                const bf16* row1 = C1 > 0 ? a.in.p1 + ((size_t)n * H + yc) * W * C1 : in;
                // 16-byte chunk q = pixel p (x0 - 1 + p) x group g: channels [0, C0)
                // from the first source (at x >> up), the rest from the second
                for (int q = tid; q < 130 * G; q += 128) {
                    const int pp = q / G, g = q - pp * G;
                    const int x = x0 - 1 + pp, c = g * 8;
                    const bool inside = yin && x >= 0 && x < W;
                    const void* src = c < C0 ? (const void*)(row0 + (size_t)(x >> up) * C0 + c)
                                             : (const void*)(row1 + (size_t)x * C1 + (c - C0));
                    cp_async16(dst + (uint32_t)g * 2080u + (uint32_t)pp * 16u, inside ? src : (const void*)in,
                               inside ? 16u : 0u);
                }
                cp_async_arrive(tc::smem_addr(&row_full[b]));
            }
        }
        if (!tma_rows) cp_async_wait_all();
    } else if (warp == 4) {
        // ---------------------------------------------------------- MMA issue
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, Np);
            const uint64_t adesc0 = tc::smem_desc(rbase, 2080u, 128u), bdesc0 = tc::smem_desc(wbase, nblk, 128u);
            const uint32_t bstep = (2u * nblk) >> 4;           // 16 channels of weights
            const int ksteps = K / 16;
            bool ok = tc::mbar_wait_or_abort(tc::smem_addr(&wbar), 0u, a.err, 7, &s_abort);
            int L = 0, tcount = 0;
            for (int strip = blockIdx.x; strip < nstrips && ok; strip += gridDim.x) {
                const int rest = strip / tiles_x;
                const int ys = (rest % strips_y) * R;
                const int ye = min(ys + R, H);
                const int rows = ye - ys;
                for (int k = 0; k < rows && ok; k++, tcount++) {
                    // input rows y-1, y, y+1 are loads L+k, L+k+1, L+k+2
                    for (int d = 0; d < 3 && ok; d++) {
                        const int Ld = L + k + d;
                        ok = tc::mbar_wait_or_abort(tc::smem_addr(&row_full[Ld % nb]), (uint32_t)((Ld / nb) & 1), a.err,
                                                    8, &s_abort);
                    }
                    const int buf = tcount & 1;
                    if (ok && tcount >= 2)
                        ok = tc::mbar_wait_or_abort(tc::smem_addr(&acc_empty[buf]), (uint32_t)(((tcount >> 1) - 1) & 1),
                                                    a.err, 9, &s_abort);
                    if (!ok) break;
                    tc::fence_proxy_async();
                    tc::fence_after_sync();
                    const uint32_t d = taddr + (uint32_t)(buf * Np);
                    // descriptors differ only in their start-address field (bits 0-13,
                    // address >> 4): step them by integer offsets, no rebuilding per MMA
                    uint32_t acc = 0u;
                    for (int dy = 0; dy < 3; dy++) {
                        const uint64_t arow = adesc0 + (((uint32_t)((L + k + dy) % nb) * rowb) >> 4);
                        for (int dx = 0; dx < 3; dx++) {
                            const uint64_t ad = arow + (uint32_t)dx;             // one pixel = 16 bytes
                            const uint64_t bd = bdesc0 + (((uint32_t)((dy * 3 + dx) * G) * nblk) >> 4);
                            for (int kk = 0; kk < ksteps; kk++) {
                                tc::mma_bf16(d, ad + (uint64_t)(260u * kk), bd + (uint64_t)(bstep * kk), idesc, acc);
                                acc = 1u;
                            }
                        }
                    }
                    tc::mma_commit(tc::smem_addr(&acc_full[buf]));
                    tc::mma_commit(tc::smem_addr(&row_empty[(L + k) % nb]));   // input row y-1 is done
                }
                if (!ok) break;
                // the strip's last two input rows
                tc::mma_commit(tc::smem_addr(&row_empty[(L + rows) % nb]));
                tc::mma_commit(tc::smem_addr(&row_empty[(L + rows + 1) % nb]));
                L += rows + 2;
            }
        }
        __syncwarp();
    } else {
        // ---------------------------------------------------------- epilogue
        const int q = warp & 3;
        const int m = q * 32 + lane;
        int tcount = 0;
        bool ok = true;
        for (int strip = blockIdx.x; strip < nstrips && ok; strip += gridDim.x) {
            const int xb = strip % tiles_x, rest = strip / tiles_x;
            const int ys = (rest % strips_y) * R, n = rest / strips_y;
            const int ye = min(ys + R, H);
            const int x = xb * 128 + m;
            const bool valid = x < W;
            for (int y = ys; y < ye; y++, tcount++) {
                const int buf = tcount & 1;
                if (!tc::mbar_wait_or_abort(tc::smem_addr(&acc_full[buf]), (uint32_t)((tcount >> 1) & 1), a.err, 10,
                                            &s_abort)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const size_t p = ((size_t)n * H + y) * W + x;
                for (int c0 = 0; c0 < Np; c0 += 16) {
                    float v[16];
                    tc::tmem_ld16(taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * Np + c0), v);
                    if (!valid) continue;
                    if (a.bias) {
                        const float4* bb = reinterpret_cast<const float4*>(a.bias + c0);
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const float4 b4 = __ldg(bb + k);
                            v[4 * k] += b4.x;
                            v[4 * k + 1] += b4.y;
                            v[4 * k + 2] += b4.z;
                            v[4 * k + 3] += b4.w;
                        }
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
                        for (int k = 0; k < 4; k++)
                            o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
                    }
                }
                tc::fence_before_sync();
                tc::mbar_arrive(tc::smem_addr(&acc_empty[buf]));
            }
        }
    }
    if (s_abort && warp == 4 && lane == 0) {
        for (int k = 0; k < kRowBufs; k++) {
            tc::mbar_wait(tc::smem_addr(&row_full[k]), 0u, nullptr, 0);
            tc::mbar_wait(tc::smem_addr(&row_empty[k]), 0u, nullptr, 0);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(taddr, ncols);
}

// The two-source input of a decoder convolution, assembled: channels [0, C0)
// nearest-upsampled from the half-size p0, channels [C0, C0 + C1) from p1.
__global__ void k_upcat(ConvSrc s, bf16* out) {
    const int C = s.C0 + s.C1, c8n = C >> 3;
    const long long total = (long long)s.N * s.H * s.W * c8n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % c8n);
        const long long q = i / c8n;
        const int x = (int)(q % s.W), y = (int)((q / s.W) % s.H), n = (int)(q / ((long long)s.W * s.H));
        *reinterpret_cast<uint4*>(out + (size_t)q * C + c8 * 8) = load8(s, n, y, x, c8 * 8);
    }
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

static unsigned ew_grid(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        cudaGetLastError();
    });
    return fn;
}

// BF16 tensor map of `rank` dims (innermost first), boxes of `box`, zero fill,
// with the shared-memory swizzle `swz`.
static bool make_map(CUtensorMap* m, const void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                     const cuuint32_t* box, CUtensorMapSwizzle swz) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Channel chunk of one pipeline stage and whether all 9 taps of weights stay
// in shared memory, within the shared-memory budget.
// The ring has as many stages (3..kConvStages) as fit a 52 KB budget, which
// leaves room for four CTAs per SM.
struct ConvPlan {
    int kc, resident, stages;
    size_t smem;
};
static ConvPlan conv_plan(int Cin, int Np) {
    ConvPlan p;
    p.kc = Cin % 32 == 0 ? 32 : 16;
    const size_t wbytes = 9u * (size_t)Cin * Np * 2u;
    p.resident = wbytes <= 80u * 1024u;
    const size_t stage = 128u * p.kc * 2u + (p.resident ? 0u : (size_t)Np * p.kc * 2u);
    const size_t fixed = p.resident ? wbytes : 0u, budget = 52u * 1024u;
    long long s = budget > fixed ? (long long)((budget - fixed) / stage) : 0;
    p.stages = (int)std::max(3LL, std::min((long long)kConvStages, s));
    p.smem = fixed + (size_t)p.stages * stage;
    return p;
}

size_t conv3x3_smem(int Cin, int Np) { return conv_plan(Cin, Np).smem; }

// Persistent CTAs per SM for a conv: limited by shared memory and by TMEM
// (two accumulators of Np columns each, 512 columns per SM).
static int conv_ctas_per_sm(int Np, size_t smem) {
    const int by_tmem = 512 / (int)tmem_columns(2 * Np);
    const int by_smem = (int)((220u * 1024u) / (smem + 2048u));
    // up to four resident CTAs (measured on the 1080p inference: 1.85 / 1.77 /
    // 1.75 ms with at most 2 / 3 / 4 and the stage budget below)
    return std::max(1, std::min(std::min(by_tmem, by_smem), 4));
}

size_t conv3x3_dw_smem(int Cin) { return 2u * (128u * 128u * 2u + (size_t)Cin * 128u * 2u); }

cudaError_t conv3x3(const ConvArgs& a, cudaStream_t s) {
    if (a.Cin != a.in.C0 + a.in.C1 || a.Cin % 16 || a.Cin < 16 || a.Cin > 256 || a.Np % 16 || a.Np < 16 ||
        a.Np > 256 || (a.in.up0 && ((a.in.H | a.in.W) & 1)) || (a.in.C0 % 8) || (a.in.C1 % 8) || !a.w)
        return cudaErrorInvalidValue;
    const long long P = (long long)a.in.N * a.in.H * a.in.W;
    const bool two = a.in.up0 || a.in.C1 > 0;
    const bf16* src = a.in.p0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int tiles_x = (a.in.W + 127) / 128;
    // row-resident kernel when the weights and at least four input rows fit
    {
        const size_t wbytes = 9u * (size_t)a.Cin * a.Np * 2u, rowb = ((size_t)(a.Cin / 8) * 2080u + 127u) & ~(size_t)127u;
        const size_t budget = 200u * 1024u;
        if (wbytes <= 80u * 1024u && wbytes + 4u * rowb <= budget) {
            // the most resident CTAs per SM, up to three (measured: 1080p
            // inference 2.49 / 2.01 / 1.85 / 1.89 ms with 1 / 2 / 3 / 4), with
            // 4..6 row buffers each, then the most buffers for that count
            const int tmem_cap = 512 / (int)tmem_columns(2 * a.Np);
            int per_sm = 1, nb = (int)std::min<size_t>(kRowBufs, (budget - wbytes) / rowb);
            for (int p = std::min(3, tmem_cap); p >= 2; p--) {
                const size_t room = (220u * 1024u) / (size_t)p;
                if (room < wbytes + 4u * rowb + 2048u) continue;
                per_sm = p;
                nb = (int)std::min<size_t>(kRowBufs, (room - 2048u - wbytes) / rowb);
                break;
            }
            const size_t sm = wbytes + (size_t)nb * rowb;
            const int ctas = sms * per_sm;
            const long long cols = (long long)tiles_x * a.in.N;
            // strips of R rows: about four per CTA, at least 4 rows each
            int R = (int)std::max<long long>(4, ((long long)a.in.H * cols + 4LL * ctas - 1) / (4LL * ctas));
            R = std::min(R, a.in.H);
            const long long nstrips = cols * ((a.in.H + R - 1) / R);
            if (nstrips > (1LL << 30)) return cudaErrorInvalidValue;
            CUtensorMap tm_w8;
            const cuuint64_t dw8[3] = {(cuuint64_t)a.Cin, 9u, (cuuint64_t)a.Np};
            const cuuint64_t sw8[2] = {(cuuint64_t)a.Cin * 2u, (cuuint64_t)a.Cin * 2u * 9u};
            const cuuint32_t bw8[3] = {8u, 1u, (cuuint32_t)a.Np};
            if (!make_map(&tm_w8, a.w, 3, dw8, sw8, bw8, CU_TENSOR_MAP_SWIZZLE_NONE)) return cudaErrorInvalidValue;
            // a two-source input is read from its sources by the cp.async loaders
            ConvArgs b = a;
            if (!two) b.in = ConvSrc{src, a.Cin, 0, nullptr, 0, a.in.N, a.in.H, a.in.W};
            // input rows as a 5-D map ordered (channel in group, pixel, group,
            // row, image) so that one box lands in the row buffer's K-major
            // layout: K/8 blocks of 130 pixels x 16 bytes
            CUtensorMap tm_rows;
            const int G = a.Cin / 8;
            const cuuint64_t dr[5] = {8u, (cuuint64_t)a.in.W, (cuuint64_t)G, (cuuint64_t)a.in.H, (cuuint64_t)a.in.N};
            const cuuint64_t sr[4] = {(cuuint64_t)a.Cin * 2u, 16u, (cuuint64_t)a.Cin * 2u * a.in.W,
                                      (cuuint64_t)a.Cin * 2u * a.in.W * a.in.H};
            const cuuint32_t br[5] = {8u, 130u, (cuuint32_t)G, 1u, 1u};
            // (images narrower than the box keep the cp.async loaders)
            const bool tma_rows =
                !two && a.in.W >= 130 && make_map(&tm_rows, src, 5, dr, sr, br, CU_TENSOR_MAP_SWIZZLE_NONE);
            if (!tma_rows) std::memset(&tm_rows, 0, sizeof tm_rows);
            if ((e = cudaFuncSetAttribute(k_conv3x3_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) !=
                cudaSuccess)
                return e;
            const int grid = (int)std::min<long long>(nstrips, ctas);
            k_conv3x3_rows<<<grid, kRowThreads, sm, s>>>(tm_w8, tm_rows, b, R, (int)nstrips, tiles_x, nb,
                                                         tma_rows ? 1 : 0);
            return cudaGetLastError();
        }
    }
    const ConvPlan plan = conv_plan(a.Cin, a.Np);
    if (plan.smem > 200u * 1024u) return cudaErrorInvalidValue;
    // a decoder input (half-resolution source first, then a full-resolution
    // one) is staged from its sources in even / odd pixel order when both
    // split at chunk boundaries and a row holds a whole 64-pixel half box;
    // otherwise it is assembled into a scratch tensor first
    const bool split = two && a.in.up0 && a.in.C1 > 0 && a.in.C0 % plan.kc == 0 && a.in.C1 % plan.kc == 0 &&
                       a.in.W >= 128;
    if (two && !split) {
        if (!a.scratch) return cudaErrorInvalidValue;
        k_upcat<<<ew_grid(P * (a.Cin / 8)), 256, 0, s>>>(a.in, a.scratch);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        src = a.scratch;
    }
    CUtensorMap tm_in, tm_w, tm_in2;
    std::memset(&tm_in2, 0, sizeof tm_in2);
    const cuuint64_t din[4] = {(cuuint64_t)a.Cin, (cuuint64_t)a.in.W, (cuuint64_t)a.in.H, (cuuint64_t)a.in.N};
    const cuuint64_t sin[3] = {(cuuint64_t)a.Cin * 2u, (cuuint64_t)a.Cin * 2u * a.in.W,
                               (cuuint64_t)a.Cin * 2u * a.in.W * a.in.H};
    const int box_w = a.in.W < 128 ? a.in.W : 128;
    const cuuint32_t kc = (cuuint32_t)plan.kc;
    const CUtensorMapSwizzle swz = plan.kc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
    const cuuint32_t bin[4] = {kc, (cuuint32_t)box_w, 1u, 1u};
    const cuuint64_t dw[3] = {(cuuint64_t)a.Cin, 9u, (cuuint64_t)a.Np};
    const cuuint64_t sw[2] = {(cuuint64_t)a.Cin * 2u, (cuuint64_t)a.Cin * 2u * 9u};
    const cuuint32_t bw[3] = {kc, 1u, (cuuint32_t)a.Np};
    if (!make_map(&tm_w, a.w, 3, dw, sw, bw, swz)) return cudaErrorInvalidValue;
    ConvArgs b = a;
    if (split) {
        const int C0 = a.in.C0, C1 = a.in.C1, W2 = a.in.W / 2, H2 = a.in.H / 2;
        const cuuint64_t dl[4] = {(cuuint64_t)C0, (cuuint64_t)W2, (cuuint64_t)H2, (cuuint64_t)a.in.N};
        const cuuint64_t sl[3] = {(cuuint64_t)C0 * 2u, (cuuint64_t)C0 * 2u * W2, (cuuint64_t)C0 * 2u * W2 * H2};
        const cuuint32_t bl[4] = {kc, 64u, 1u, 1u};
        const cuuint64_t dp[5] = {(cuuint64_t)C1, 2u, (cuuint64_t)W2, (cuuint64_t)a.in.H, (cuuint64_t)a.in.N};
        const cuuint64_t sp[4] = {(cuuint64_t)C1 * 2u, (cuuint64_t)C1 * 4u, (cuuint64_t)C1 * 2u * a.in.W,
                                  (cuuint64_t)C1 * 2u * a.in.W * a.in.H};
        const cuuint32_t bp[5] = {kc, 1u, 64u, 1u, 1u};
        if (!make_map(&tm_in, a.in.p0, 4, dl, sl, bl, swz) || !make_map(&tm_in2, a.in.p1, 5, dp, sp, bp, swz))
            return cudaErrorInvalidValue;
    } else {
        if (!make_map(&tm_in, src, 4, din, sin, bin, swz)) return cudaErrorInvalidValue;
        b.in = ConvSrc{src, a.Cin, 0, nullptr, 0, a.in.N, a.in.H, a.in.W};
    }
    if ((e = cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem)) !=
        cudaSuccess)
        return e;
    const long long ntiles = (long long)tiles_x * a.in.H * a.in.N;
    if (ntiles > (1LL << 30)) return cudaErrorInvalidValue;
    const int grid = (int)std::min<long long>(ntiles, (long long)sms * conv_ctas_per_sm(a.Np, plan.smem));
    k_conv3x3<<<grid, kConvThreads, plan.smem, s>>>(tm_in, tm_w, tm_in2, b, plan.kc, (int)ntiles, tiles_x,
                                                     plan.resident, box_w, plan.stages, split ? a.in.C0 : 0);
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
