// Manhattan distance field (World::GenerateDistanceField, Core/World.cpp:69-113;
// ManhattanDistanceX/Y/Z.comp).
//
// The reference runs three dependent sweeps with one thread per row/column and
// image load/store. Its result is min(min(254, X+Y+Z), L1 distance to the
// nearest non-air voxel); these kernels produce the same bytes:
//   x: one warp per row, segmented nearest-solid search with warp shuffles;
//   y, z: one thread per column, forward/backward min(d, d_prev + 1) sweeps
//         with the running value in a register; a warp covers 32 consecutive
//         x, so every row access is one coalesced 32-byte sector.
// The x sweep reads the volume and writes the field once; the y and z sweeps
// read the field twice and write it at most twice (L2-resident for <= 256^3).
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

}  // namespace

cudaError_t df_build(const uint8_t* vox, uint8_t* df, int X, int Y, int Z, cudaStream_t s, int* launches) {
    const int maxd = min(254, X + Y + Z);   // ManhattanDistanceX.comp:51
    const int rows = Y * Z;
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
