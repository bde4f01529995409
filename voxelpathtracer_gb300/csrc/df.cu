// Manhattan distance field (World::GenerateDistanceField, Core/World.cpp:69-113;
// ManhattanDistanceX/Y/Z.comp).
//
// The reference runs three dependent sweeps with one thread per row/column and
// image load/store. Its result is min(min(254, X+Y+Z), L1 distance to the
// nearest non-air voxel); these kernels produce the same bytes.
//
// Vectorised path (X a multiple of 16 up to 1024, lines along y and z up to
// 1536 voxels, both volumes 16-byte aligned: every benchmark world):
//   x: k_df_x16 -- each lane owns one 16-byte segment of a row (one 128-bit
//      load), finds the nearest solid voxel left and right of each byte from
//      its own segment and a shuffle scan over the row's lanes, and writes the
//      16 distances with one 128-bit store: one read and one write per voxel;
//   y, z: k_df_sweep_tile -- a CTA stages a tile of 16..64 consecutive x by
//      the whole line along y (or z) in shared memory with 128-bit loads,
//      computes the line transform there with all its threads (4 columns per
//      thread as two 16-bit lanes per register, each line split into
//      segments joined by their end values; min(d_prev + 1, d) is one DPX
//      add-min per lane pair), and writes the tile back with 128-bit stores:
//      one read and one write per voxel per sweep, all global accesses
//      independent of one another.
// Generic path (any X, any alignment): one warp per row with warp shuffles
// for x; one thread per column with the running value in a register for y, z.
#include <algorithm>

#include "kernels.cuh"

namespace vpt {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__global__ void __launch_bounds__(256) k_df_x(const uint8_t* __restrict__ vox, uint8_t* __restrict__ df, int X,
                                              int rows, int maxd) {
    int row = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (row >= rows) return;   // whole warp
    const uint8_t* v = vox + (size_t)row * X;
    uint8_t* d = df + (size_t)row * X;
    const int chunk = (X + 31) >> 5;
    const int x0 = min(lane * chunk, X), x1 = min(x0 + chunk, X);
    const int NEG = -(1 << 24), POS = 1 << 24;
    int first = POS, last = NEG;
    for (int x = x0; x < x1; x++) {
        if (v[x]) {
            if (first == POS) first = x;
            last = x;
        }
    }
    int incl = last;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int t = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl = max(incl, t);
    }
    int left = __shfl_up_sync(kFull, incl, 1);
    if (lane == 0) left = NEG;
    int incr = first;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int t = __shfl_down_sync(kFull, incr, off);
        if (lane + off < 32) incr = min(incr, t);
    }
    int right = __shfl_down_sync(kFull, incr, 1);
    if (lane == 31) right = POS;
    // forward: distance to the nearest solid at or left of x
    int l = left;
    for (int x = x0; x < x1; x++) {
        if (v[x]) l = x;
        d[x] = (uint8_t)min(maxd, x - l);
    }
    // backward: combine with the nearest solid at or right of x
    int r = right;
    for (int x = x1 - 1; x >= x0; x--) {
        if (v[x]) r = x;
        int dv = min((int)d[x], min(maxd, r - x));
        d[x] = (uint8_t)dv;
    }
}

// Sweep along an axis with `stride`, n samples, starting at `base`.
__device__ __forceinline__ void sweep(uint8_t* base, size_t stride, int n) {
    int prev = base[0];
    for (int k = 1; k < n; k++) {
        uint8_t* p = base + (size_t)k * stride;
        int cur = *p;
        if (prev < cur) {   // ManhattanDistanceY.comp:105-109
            cur = prev + 1;
            *p = (uint8_t)cur;
        }
        prev = cur;
    }
    prev = base[(size_t)(n - 1) * stride];
    for (int k = n - 2; k >= 0; k--) {
        uint8_t* p = base + (size_t)k * stride;
        int cur = *p;
        if (prev < cur) {
            cur = prev + 1;
            *p = (uint8_t)cur;
        }
        prev = cur;
    }
}

__global__ void __launch_bounds__(128) k_df_y(uint8_t* df, int X, int Y) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int z = blockIdx.y;
    if (x >= X) return;
    sweep(df + (size_t)z * X * Y + x, (size_t)X, Y);
}

__global__ void __launch_bounds__(128) k_df_z(uint8_t* df, int X, int Y, int Z) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= X) return;
    sweep(df + (size_t)y * X + x, (size_t)X * Y, Z);
}

// ------------------------------------------------- vectorised full build --
// x sweep, X % 16 == 0 and X <= 1024. A row of X bytes is S = X / 16
// segments; L lanes (a power of two >= S, at most 32) work on one row, each on
// kSegs = ceil(S / L) consecutive segments held in registers, so a warp holds
// 32 / L rows. Each warp does kGroups such row groups, with the loads of all
// of them issued before any is processed (more bytes in flight).
constexpr int kGroups = 4;

// The distances of one row group's segments v (row `row`, this lane's
// segments from s0); every lane of the warp calls it.
template <int kSegs>
__device__ __forceinline__ void x_row(const uint4 (&v)[kSegs], uint4* __restrict__ df, int S, int L, int l, int s0,
                                      int row, bool live, int maxd) {
    const int NEG = -(1 << 24), POS = 1 << 24;
    // nearest solid at or left of / at or right of each byte, first within the lane
    int first = POS, last = NEG;
#pragma unroll
    for (int k = kSegs - 1; k >= 0; k--) {
        const unsigned w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
        for (int b = 15; b >= 0; b--)
            if ((w[b >> 2] >> (8 * (b & 3))) & 0xffu) first = (s0 + k) * 16 + b;
    }
#pragma unroll
    for (int k = 0; k < kSegs; k++) {
        const unsigned w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
        for (int b = 0; b < 16; b++)
            if ((w[b >> 2] >> (8 * (b & 3))) & 0xffu) last = (s0 + k) * 16 + b;
    }
    // inclusive max-scan of `last` towards the right, min-scan of `first` towards the left, within the row
    int incl = last, incr = first;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        if (off >= L) break;
        const int a = __shfl_up_sync(kFull, incl, off, L);   // every lane of the warp gets here
        const int b = __shfl_down_sync(kFull, incr, off, L);
        if (l >= off) incl = max(incl, a);
        if (l + off < L) incr = min(incr, b);
    }
    int left = __shfl_up_sync(kFull, incl, 1, L);
    int right = __shfl_down_sync(kFull, incr, 1, L);
    if (l == 0) left = NEG;
    if (l == L - 1) right = POS;
    // right-to-left pass: distance to the nearest solid at or right of x
    unsigned char dr[kSegs * 16];
#pragma unroll
    for (int k = kSegs - 1; k >= 0; k--) {
        const unsigned w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
        for (int b = 15; b >= 0; b--) {
            const int x = (s0 + k) * 16 + b;
            if ((w[b >> 2] >> (8 * (b & 3))) & 0xffu) right = x;
            dr[k * 16 + b] = (unsigned char)min(maxd, right - x);
        }
    }
    // left-to-right pass, combined and packed
#pragma unroll
    for (int k = 0; k < kSegs; k++) {
        const unsigned w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
        unsigned o[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int b = 0; b < 16; b++) {
            const int x = (s0 + k) * 16 + b;
            if ((w[b >> 2] >> (8 * (b & 3))) & 0xffu) left = x;
            const unsigned d = (unsigned)min((int)dr[k * 16 + b], min(maxd, x - left));
            o[b >> 2] |= d << (8 * (b & 3));
        }
        if (live && s0 + k < S) df[(size_t)row * S + s0 + k] = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

template <int kSegs>
__global__ void __launch_bounds__(256) k_df_x16(const uint4* __restrict__ vox, uint4* __restrict__ df, int S,
                                                int L, int rows, int maxd) {
    const int lane = threadIdx.x & 31;
    const int rows_per_warp = 32 / L;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int sub = lane / L, l = lane % L;                 // row within the group, lane within the row
    // segments [s0, s0 + kSegs) of a row belong to this lane
    const int s0 = l * kSegs;
    int row[kGroups];
    bool live[kGroups];
    uint4 v[kGroups][kSegs];
#pragma unroll
    for (int g = 0; g < kGroups; g++) {
        row[g] = (kGroups * warp + g) * rows_per_warp + sub;
        live[g] = row[g] < rows;
#pragma unroll
        for (int k = 0; k < kSegs; k++)
            v[g][k] = (live[g] && s0 + k < S) ? __ldg(vox + (size_t)row[g] * S + s0 + k) : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int g = 0; g < kGroups; g++) x_row<kSegs>(v[g], df, S, L, l, s0, row[g], live[g], maxd);
}

// y or z sweep over a tile: x in [x0, x0 + w) (w a multiple of 16, at most
// kTile) and the whole line of n samples `stride` bytes apart, starting at
// byte base = blockIdx.y * outer + x0. The tile sits in shared memory, row r
// at r * w. The line's result is min over j of d[j] + |r - j| (the forward
// then backward min(d, d_prev + 1) sweeps of ManhattanDistanceY/Z.comp), so
// the 128 threads split it: G = w / 4 column groups (4 columns per thread, as
// two 16-bit lanes per register) times P = 128 / G segments of m rows each
// (m odd, so the segments of one warp fall in different shared-memory
// banks). Each thread
//   1. reduces its segment to the distance it passes on at either end
//      (min of d[j] + distance to the segment's last / first row);
//   2. chains those over the segments before / after it into the forward
//      value just before its segment and the backward value just after it;
//   3. runs the forward sweep over its segment seeded with the first and the
//      backward sweep over the forward values seeded with the second, which
//      leaves the exact line result in its rows.
constexpr int kTile = 64;
constexpr unsigned kInf2 = 0x3fff3fffu;   // "no voxel yet" in both 16-bit lanes; + 1536 cannot overflow

__device__ __forceinline__ unsigned lo_pair(unsigned w) { return __byte_perm(w, 0u, 0x4140); }   // bytes 0, 1
__device__ __forceinline__ unsigned hi_pair(unsigned w) { return __byte_perm(w, 0u, 0x4342); }   // bytes 2, 3
__device__ __forceinline__ unsigned pack_pairs(unsigned lo, unsigned hi) { return __byte_perm(lo, hi, 0x6420); }

__global__ void __launch_bounds__(128) k_df_sweep_tile(uint8_t* __restrict__ df, int X, int n, size_t stride,
                                                       size_t outer) {
    extern __shared__ __align__(16) uint8_t tile[];
    __shared__ unsigned s_carry[4][128];   // per thread: forward-end lo / hi, backward-start lo / hi
    const int x0 = blockIdx.x * kTile;
    const int w = min(kTile, X - x0);
    const int q = w >> 4;   // 16-byte words per row
    uint8_t* base = df + (size_t)blockIdx.y * outer + x0;
    // four independent 128-bit loads in flight per thread before they are stored
    const int nq = n * q;
    for (int k0 = threadIdx.x; k0 < nq; k0 += 4 * blockDim.x) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int k = k0 + u * blockDim.x;
            if (k < nq) {
                const int r = k / q, c = k - r * q;
                v[u] = *reinterpret_cast<const uint4*>(base + (size_t)r * stride + 16 * c);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int k = k0 + u * blockDim.x;
            if (k < nq) {
                const int r = k / q, c = k - r * q;
                reinterpret_cast<uint4*>(tile + (size_t)r * w)[c] = v[u];
            }
        }
    }
    __syncthreads();
    const int G = w >> 2;                   // column groups (words per row)
    const int P = blockDim.x / G;           // segments
    const int g = threadIdx.x % G, sg = threadIdx.x / G;
    const int m = ((n + P - 1) / P) | 1;
    const int a = min(n, sg * m), b = min(n, a + m);
    unsigned* col = reinterpret_cast<unsigned*>(tile) + g;
    // 1. the segment's own contribution at its ends
    unsigned fl = kInf2, fh = kInf2, bl = kInf2, bh = kInf2;
    for (int r = a; r < b; r++) {
        const unsigned cw = col[(size_t)r * G];
        const unsigned to_end = (unsigned)(b - 1 - r) * 0x00010001u, to_start = (unsigned)(r - a) * 0x00010001u;
        fl = __viaddmin_u16x2(lo_pair(cw), to_end, fl);
        fh = __viaddmin_u16x2(hi_pair(cw), to_end, fh);
        bl = __viaddmin_u16x2(lo_pair(cw), to_start, bl);
        bh = __viaddmin_u16x2(hi_pair(cw), to_start, bh);
    }
    s_carry[0][threadIdx.x] = fl;
    s_carry[1][threadIdx.x] = fh;
    s_carry[2][threadIdx.x] = bl;
    s_carry[3][threadIdx.x] = bh;
    __syncthreads();
    // 2. forward value before row a, backward value after row b - 1
    unsigned Fl = kInf2, Fh = kInf2, Bl = kInf2, Bh = kInf2;
    for (int k = 0; k < sg; k++) {
        const int ka = min(n, k * m);
        const unsigned len = (unsigned)(min(n, ka + m) - ka) * 0x00010001u;
        Fl = __viaddmin_u16x2(Fl, len, s_carry[0][k * G + g]);
        Fh = __viaddmin_u16x2(Fh, len, s_carry[1][k * G + g]);
    }
    for (int k = P - 1; k > sg; k--) {
        const int ka = min(n, k * m);
        const unsigned len = (unsigned)(min(n, ka + m) - ka) * 0x00010001u;
        Bl = __viaddmin_u16x2(Bl, len, s_carry[2][k * G + g]);
        Bh = __viaddmin_u16x2(Bh, len, s_carry[3][k * G + g]);
    }
    // 3. the seeded sweeps (ManhattanDistanceY.comp:105-109: d = min(d, d_prev + 1))
    const unsigned one = 0x00010001u;
    for (int r = a; r < b; r++) {
        const unsigned cw = col[(size_t)r * G];
        Fl = __viaddmin_u16x2(Fl, one, lo_pair(cw));
        Fh = __viaddmin_u16x2(Fh, one, hi_pair(cw));
        col[(size_t)r * G] = pack_pairs(Fl, Fh);
    }
    for (int r = b - 1; r >= a; r--) {
        const unsigned cw = col[(size_t)r * G];
        Bl = __viaddmin_u16x2(Bl, one, lo_pair(cw));
        Bh = __viaddmin_u16x2(Bh, one, hi_pair(cw));
        col[(size_t)r * G] = pack_pairs(Bl, Bh);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nq; k += blockDim.x) {
        const int r = k / q, c = k - r * q;
        *reinterpret_cast<uint4*>(base + (size_t)r * stride + 16 * c) =
            reinterpret_cast<const uint4*>(tile + (size_t)r * w)[c];
    }
}

// ------------------------------------------------------ incremental update --
// An edit of the voxels in box E changes the field only within L1 distance
// maxd of E, inside the box O = E grown by maxd on every side. Over the sweep
// box B = O grown by one more voxel (clipped to the world), the field is
// recomputed from initial values: 0 for solid voxels, maxd for other voxels
// of O, and the old (still exact) value for the ring B \ O; the three
// separable min(d, d_prev + 1) sweeps of that initialisation yield
// min over sources p of init(p) + |v - p|_1, which is the exact capped L1
// distance everywhere in B (every init is an upper bound of the true value,
// and any shortest path to a solid outside B leaves B through the exact ring).
struct Box3 {
    int x0, y0, z0, x1, y1, z1;   // [x0, x1) x [y0, y1) x [z0, z1)
};

__global__ void __launch_bounds__(256) k_dfu_init(const uint8_t* __restrict__ vox, uint8_t* __restrict__ df, int X,
                                                  int Y, Box3 b, Box3 o, int maxd) {
    const int w = b.x1 - b.x0, h = b.y1 - b.y0;
    const long long n = (long long)w * h * (b.z1 - b.z0);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = b.x0 + (int)(i % w), y = b.y0 + (int)((i / w) % h), z = b.z0 + (int)(i / ((long long)w * h));
        const size_t v = (size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z);
        const bool in_o = x >= o.x0 && x < o.x1 && y >= o.y0 && y < o.y1 && z >= o.z0 && z < o.z1;
        if (vox[v]) df[v] = 0;
        else if (in_o) df[v] = (uint8_t)maxd;
    }
}

// axis 0: x lines over (y, z); 1: y lines over (x, z); 2: z lines over (x, y)
__global__ void __launch_bounds__(128) k_dfu_sweep(uint8_t* df, int X, int Y, Box3 b, int axis) {
    const int w = b.x1 - b.x0, h = b.y1 - b.y0, d = b.z1 - b.z0;
    const int na = axis == 0 ? h : w, nb = axis == 2 ? h : d;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)na * nb) return;
    const int ia = (int)(idx % na), ib = (int)(idx / na);
    size_t base;
    if (axis == 0) {
        base = (size_t)b.x0 + (size_t)X * ((size_t)(b.y0 + ia) + (size_t)Y * (b.z0 + ib));
        sweep(df + base, 1, w);
    } else if (axis == 1) {
        base = (size_t)(b.x0 + ia) + (size_t)X * ((size_t)b.y0 + (size_t)Y * (b.z0 + ib));
        sweep(df + base, (size_t)X, h);
    } else {
        base = (size_t)(b.x0 + ia) + (size_t)X * ((size_t)(b.y0 + ib) + (size_t)Y * b.z0);
        sweep(df + base, (size_t)X * Y, d);
    }
}

}  // namespace

cudaError_t df_update(const uint8_t* vox, uint8_t* df, int X, int Y, int Z, int ex0, int ey0, int ez0, int ex1,
                      int ey1, int ez1, cudaStream_t s, int* launches) {
    const int maxd = min(254, X + Y + Z);
    Box3 o{max(ex0 - maxd, 0), max(ey0 - maxd, 0), max(ez0 - maxd, 0), min(ex1 + maxd, X), min(ey1 + maxd, Y),
           min(ez1 + maxd, Z)};
    Box3 b{max(o.x0 - 1, 0), max(o.y0 - 1, 0), max(o.z0 - 1, 0), min(o.x1 + 1, X), min(o.y1 + 1, Y), min(o.z1 + 1, Z)};
    const long long n = (long long)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
    k_dfu_init<<<(unsigned)std::min<long long>((n + 255) / 256, 152LL * 32), 256, 0, s>>>(vox, df, X, Y, b, o, maxd);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int w = b.x1 - b.x0, h = b.y1 - b.y0, d = b.z1 - b.z0;
    const long long lines[3] = {(long long)h * d, (long long)w * d, (long long)w * h};
    for (int axis = 0; axis < 3; axis++) {
        k_dfu_sweep<<<(unsigned)((lines[axis] + 127) / 128), 128, 0, s>>>(df, X, Y, b, axis);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (launches) *launches += 4;
    return cudaSuccess;
}

namespace {

constexpr int kSweepSmemMax = 96 * 1024;   // shared memory of one sweep tile: lines of up to 1536 voxels

template <int kSegs>
cudaError_t launch_x16(const uint8_t* vox, uint8_t* df, int X, int rows, int maxd, cudaStream_t s) {
    const int S = X / 16;
    int L = 1;
    while (L < S && L < 32) L <<= 1;
    const int rows_per_warp = kGroups * (32 / L);
    const long long threads = (long long)(rows + rows_per_warp - 1) / rows_per_warp * 32;
    k_df_x16<kSegs><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        reinterpret_cast<const uint4*>(vox), reinterpret_cast<uint4*>(df), S, L, rows, maxd);
    return cudaGetLastError();
}

cudaError_t launch_sweep_tile(uint8_t* df, int X, int n, size_t stride, size_t outer, int lines, cudaStream_t s) {
    const size_t smem = (size_t)n * kTile;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) {   // lines longer than 768 voxels: opt in to more shared memory (current device)
        e = cudaFuncSetAttribute(k_df_sweep_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, kSweepSmemMax);
        if (e != cudaSuccess) return e;
    }
    k_df_sweep_tile<<<dim3((unsigned)((X + kTile - 1) / kTile), (unsigned)lines), 128, smem, s>>>(df, X, n, stride,
                                                                                                  outer);
    return cudaGetLastError();
}

}  // namespace

cudaError_t df_build(const uint8_t* vox, uint8_t* df, int X, int Y, int Z, cudaStream_t s, int* launches) {
    const int maxd = min(254, X + Y + Z);   // ManhattanDistanceX.comp:51
    const int rows = Y * Z;
    const bool vec = X % 16 == 0 && X <= 16 * 32 * 2 && ((uintptr_t)vox & 15u) == 0 && ((uintptr_t)df & 15u) == 0 &&
                     (size_t)std::max(Y, Z) * kTile <= (size_t)kSweepSmemMax;
    if (vec) {
        cudaError_t e =
            X <= 16 * 32 ? launch_x16<1>(vox, df, X, rows, maxd, s) : launch_x16<2>(vox, df, X, rows, maxd, s);
        if (e != cudaSuccess) return e;
        // y lines: for each z, X * Y bytes; z lines: for each y, stride X * Y
        if ((e = launch_sweep_tile(df, X, Y, (size_t)X, (size_t)X * Y, Z, s)) != cudaSuccess) return e;
        if ((e = launch_sweep_tile(df, X, Z, (size_t)X * Y, (size_t)X, Y, s)) != cudaSuccess) return e;
        if (launches) *launches += 3;
        return cudaSuccess;
    }
    k_df_x<<<(unsigned)((rows + 7) / 8), 256, 0, s>>>(vox, df, X, rows, maxd);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_df_y<<<dim3((unsigned)((X + 127) / 128), (unsigned)Z), 128, 0, s>>>(df, X, Y);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_df_z<<<dim3((unsigned)((X + 127) / 128), (unsigned)Y), 128, 0, s>>>(df, X, Y, Z);
    if (launches) *launches += 3;
    return cudaGetLastError();
}

}  // namespace vpt
