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
