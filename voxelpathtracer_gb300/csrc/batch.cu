// Batched multi-world tracing: one persistent launch over the ray tiles of
// many worlds of different sizes, and the brick re-layout of the distance
// field that the launch can trace through.
//
// The reference renders one world per process (Core/Pipeline.cpp drives one
// World's passes a frame); here each batch entry is one such world with its
// own voxel volume, distance field, block table, camera and ray tile. Work is
// split into 8x4-pixel tiles; a warp takes `tiles_per_grab` consecutive queue
// entries with one atomic, finds each tile's world by binary search over the
// tile prefix sums (in shared memory) and runs the primary, sun-shadow and
// diffuse passes of pixel_passes.cuh for its 32 pixels. Results are the same
// bits as the per-world pass kernels. The queue is one counter the host zeroes
// before the launch; no thread waits on another, so the kernel cannot stall.
#include "pixel_passes.cuh"

namespace vpt {

namespace {

// Last world whose first tile is <= tile (worlds with no tiles are skipped over).
__device__ __forceinline__ int world_of(const int* s_begin, int n_worlds, int tile) {
    int lo = 0, hi = n_worlds - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_begin[mid] <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Primary, sun-shadow and diffuse passes of one 8x4 tile, one pixel per lane.
template <int B>
__device__ __forceinline__ void batch_tile(const BatchLaunch& a, const BatchFrame& fr, const BatchWorld& bw,
                                           int local, int lane) {
    const int i = (local % bw.tiles_x) * 8 + (lane & 7);
    const int j = (local / bw.tiles_x) * 4 + (lane >> 3);
    const bool valid = i < bw.W && j < bw.H;
    unsigned psteps = 0, srays = 0, ssteps = 0;
    GICount cnt = {0u, 0u, 0u, 0u};
    if (valid) {
        const WorldView w = bw.w;
        const CamView& cam = bw.cam;
        const size_t px = (size_t)j * bw.W + i;
        float d;
        int face;
        psteps = primary_pixel<B>(w, cam, bw.W, bw.H, i, j, fr.primary_max_steps, px, bw.t, bw.face, bw.block, bw.hit,
                                  bw.steps, &d, &face);
        bw.shadow[px] = shadow_pixel<B>(w, cam, bw.W, bw.H, i, j, fr.shadow_max_steps,
                                        mk3(fr.sun[0], fr.sun[1], fr.sun[2]), d, face, &srays, &ssteps);
        diffuse_pixel<B>(w, cam, bw.W, bw.H, i, j, fr.d, px, d, face, bw.sh, bw.cocg, bw.luma, bw.aosky, &cnt);
    }
    if (a.stats) {
        count_rays(a.stats, kRayPrimary, valid ? 1u : 0u, psteps);
        count_rays(a.stats, kRayShadow, srays, ssteps);
        count_rays(a.stats, kRayDiffuse, cnt.diffuse_rays, cnt.diffuse_steps);
        count_rays(a.stats, kRayBounceShadow, cnt.shadow_rays, cnt.shadow_steps);
    }
}

// Two tiles of one world, two pixels per lane: the primary rays and then the
// sun-shadow rays of both pixels are traced interleaved (two gathers in
// flight per lane), the diffuse samples one pixel after the other. The same
// bits as two batch_tile calls.
template <int B>
__device__ __forceinline__ void batch_tile_pair(const BatchLaunch& a, const BatchFrame& fr, const BatchWorld& bw,
                                                int local0, int lane) {
    int i[2], j[2];
    bool valid[2];
    for (int k = 0; k < 2; k++) {
        const int local = local0 + k;
        i[k] = (local % bw.tiles_x) * 8 + (lane & 7);
        j[k] = (local / bw.tiles_x) * 4 + (lane >> 3);
        valid[k] = i[k] < bw.W && j[k] < bw.H;
    }
    const WorldView w = bw.w;
    const CamView& cam = bw.cam;
    float d[2] = {-1.0f, -1.0f};
    int face[2] = {kFaceMiss, kFaceMiss};
    unsigned psteps[2] = {0u, 0u}, srays = 0, ssteps = 0;
    GICount cnt = {0u, 0u, 0u, 0u};
    primary_pixel2<B>(w, cam, bw.W, bw.H, i, j, valid, fr.primary_max_steps, bw.t, bw.face, bw.block, bw.hit, bw.steps,
                      d, face, psteps);
    uint8_t sh[2];
    shadow_pixel2<B>(w, cam, bw.W, bw.H, i, j, valid, fr.shadow_max_steps, mk3(fr.sun[0], fr.sun[1], fr.sun[2]), d,
                     face, sh, &srays, &ssteps);
    for (int k = 0; k < 2; k++) {
        if (!valid[k]) continue;
        const size_t px = (size_t)j[k] * bw.W + i[k];
        bw.shadow[px] = sh[k];
        diffuse_pixel<B>(w, cam, bw.W, bw.H, i[k], j[k], fr.d, px, d[k], face[k], bw.sh, bw.cocg, bw.luma, bw.aosky,
                         &cnt);
    }
    if (a.stats) {
        count_rays(a.stats, kRayPrimary, (valid[0] ? 1u : 0u) + (valid[1] ? 1u : 0u), psteps[0] + psteps[1]);
        count_rays(a.stats, kRayShadow, srays, ssteps);
        count_rays(a.stats, kRayDiffuse, cnt.diffuse_rays, cnt.diffuse_steps);
        count_rays(a.stats, kRayBounceShadow, cnt.shadow_rays, cnt.shadow_steps);
    }
}

// kRays: pixels (rays of a pass) per lane, 1 or 2; a warp takes
// tiles_per_grab * kRays tiles per queue access. kWide: blocks of up to 512
// threads, three per SM (40 registers a thread); otherwise up to 256
// threads, four per SM (64 registers, far fewer spills of the diffuse path's
// state).
template <int B, int kRays, bool kWide>
__global__ void __launch_bounds__(kWide ? 512 : 256, kWide ? 3 : 4) k_batch_trace(BatchLaunch a) {
    __shared__ int s_begin[kBatchMaxWorlds + 1];
    for (int k = threadIdx.x; k <= a.n_worlds; k += blockDim.x) s_begin[k] = a.tile_begin[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const BatchFrame& fr = *a.frame;
    const int grab = a.tiles_per_grab * kRays;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.queue, grab);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= a.n_tiles) break;
        const int end = min(base + grab, a.n_tiles);
        for (int tile = base; tile < end;) {
            const int lo = world_of(s_begin, a.n_worlds, tile);
            if (kRays == 2 && tile + 1 < end && world_of(s_begin, a.n_worlds, tile + 1) == lo) {
                batch_tile_pair<B>(a, fr, a.worlds[lo], tile - s_begin[lo], lane);
                tile += 2;
            } else {
                batch_tile<B>(a, fr, a.worlds[lo], tile - s_begin[lo], lane);
                tile += 1;
            }
        }
    }
}

// One pass of the tile queue for the phased launch: kPass 0 primary, 1 sun
// shadow, 2 diffuse, each pass a persistent kernel of its own (the three
// passes' code never competes for one SM's instruction cache). The shadow
// and diffuse passes read the hit distance and face the primary pass stored,
// as the per-pass kernels do; outputs and ray counts are batch_tile's.
template <int B, int kPass>
__device__ __forceinline__ void batch_pass_tile(const BatchLaunch& a, const BatchFrame& fr, const BatchWorld& bw,
                                                int local, int lane) {
    const int i = (local % bw.tiles_x) * 8 + (lane & 7);
    const int j = (local / bw.tiles_x) * 4 + (lane >> 3);
    const bool valid = i < bw.W && j < bw.H;
    unsigned n0 = 0, s0 = 0;
    GICount cnt = {0u, 0u, 0u, 0u};
    if (valid) {
        const WorldView w = bw.w;
        const CamView& cam = bw.cam;
        const size_t px = (size_t)j * bw.W + i;
        if (kPass == 0) {
            float d;
            int face;
            s0 = primary_pixel<B>(w, cam, bw.W, bw.H, i, j, fr.primary_max_steps, px, bw.t, bw.face, bw.block, bw.hit,
                                  bw.steps, &d, &face);
            n0 = 1;
        } else if (kPass == 1) {
            bw.shadow[px] = shadow_pixel<B>(w, cam, bw.W, bw.H, i, j, fr.shadow_max_steps,
                                            mk3(fr.sun[0], fr.sun[1], fr.sun[2]), __ldg(bw.t + px),
                                            __ldg(bw.face + px), &n0, &s0);
        } else {
            diffuse_pixel<B>(w, cam, bw.W, bw.H, i, j, fr.d, px, __ldg(bw.t + px), __ldg(bw.face + px), bw.sh, bw.cocg,
                             bw.luma, bw.aosky, &cnt);
        }
    }
    if (a.stats) {
        if (kPass == 0) count_rays(a.stats, kRayPrimary, n0, s0);
        if (kPass == 1) count_rays(a.stats, kRayShadow, n0, s0);
        if (kPass == 2) {
            count_rays(a.stats, kRayDiffuse, cnt.diffuse_rays, cnt.diffuse_steps);
            count_rays(a.stats, kRayBounceShadow, cnt.shadow_rays, cnt.shadow_steps);
        }
    }
}

template <int B, int kPass, bool kWide>
__global__ void __launch_bounds__(kWide ? 512 : 256, kWide ? 3 : 4) k_batch_pass(BatchLaunch a) {
    __shared__ int s_begin[kBatchMaxWorlds + 1];
    for (int k = threadIdx.x; k <= a.n_worlds; k += blockDim.x) s_begin[k] = a.tile_begin[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const BatchFrame& fr = *a.frame;
    int* queue = a.queue + kPass;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(queue, a.tiles_per_grab);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= a.n_tiles) break;
        const int end = min(base + a.tiles_per_grab, a.n_tiles);
        for (int tile = base; tile < end; tile++) {
            const int lo = world_of(s_begin, a.n_worlds, tile);
            batch_pass_tile<B, kPass>(a, fr, a.worlds[lo], tile - s_begin[lo], lane);
        }
    }
}

template <int B>
__global__ void __launch_bounds__(256) k_df_bricks(const uint8_t* __restrict__ df, uint8_t* __restrict__ out, int X,
                                                   int Y, int Z, int bx, int by, size_t total) {
    const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= total) return;
    constexpr int L = B == 4 ? 2 : 3;
    const size_t brick = o >> (3 * L);
    const int r = (int)(o & ((size_t)B * B * B - 1));
    const int x = (int)(brick % (size_t)bx) * B + (r & (B - 1));
    const int y = (int)((brick / (size_t)bx) % (size_t)by) * B + ((r >> L) & (B - 1));
    const int z = (int)(brick / ((size_t)bx * by)) * B + (r >> (2 * L));
    // padding outside the volume is never read (the traversal tests the volume first)
    out[o] = (x < X && y < Y && z < Z) ? df[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)] : 0;
}

template <int B, int kRays>
int max_blocks_for(int block_threads) {
    int n = 0;
    const cudaError_t e = block_threads > 256
                              ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_trace<B, kRays, true>,
                                                                              block_threads, 0)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_trace<B, kRays, false>,
                                                                              block_threads, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// The three pass kernels of the phased launch, each with the grid that fills
// every SM to its own occupancy limit (or `blocks`).
template <int B, bool kWide>
cudaError_t launch_passes(const BatchLaunch& a, int block_threads, int blocks, int sms, cudaStream_t s,
                          const BatchSide* side) {
    using K = void (*)(BatchLaunch);
    const K ks[3] = {k_batch_pass<B, 0, kWide>, k_batch_pass<B, 1, kWide>, k_batch_pass<B, 2, kWide>};
    for (int p = 0; p < 3; p++) {
        cudaStream_t st = s;
        if (side && p == 1) {   // the shadow pass on the side stream, beside the diffuse pass
            if (cudaEventRecord(side->fork, s) != cudaSuccess || cudaStreamWaitEvent(side->side, side->fork, 0) != cudaSuccess)
                return cudaErrorInvalidValue;
            st = side->side;
        }
        int g = blocks;
        if (g <= 0) {
            int n = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ks[p], block_threads, 0) != cudaSuccess) {
                cudaGetLastError();
                return cudaErrorInvalidConfiguration;
            }
            g = n * sms;
        }
        if (g <= 0) return cudaErrorInvalidConfiguration;
        ks[p]<<<g, block_threads, 0, st>>>(a);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (side && p == 1 && cudaEventRecord(side->join, side->side) != cudaSuccess) return cudaErrorInvalidValue;
    }
    if (side && cudaStreamWaitEvent(s, side->join, 0) != cudaSuccess) return cudaErrorInvalidValue;
    return cudaSuccess;
}

}  // namespace

int batch_max_blocks(int df_brick, int block_threads, int rays_per_lane, int device) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    const bool two = rays_per_lane == 2;
    const int per_sm = df_brick == 4 ? (two ? max_blocks_for<4, 2>(block_threads) : max_blocks_for<4, 1>(block_threads))
                       : df_brick == 8 ? (two ? max_blocks_for<8, 2>(block_threads) : max_blocks_for<8, 1>(block_threads))
                                       : (two ? max_blocks_for<0, 2>(block_threads) : max_blocks_for<0, 1>(block_threads));
    return per_sm * sms;
}

cudaError_t batch_trace(const BatchLaunch& a, int df_brick, int block_threads, int rays_per_lane, int blocks,
                        int phased, cudaStream_t s, const BatchSide* side) {
    if (a.n_worlds < 1 || a.n_worlds > kBatchMaxWorlds || block_threads < 32 || block_threads > 512 ||
        (block_threads & 31) || a.tiles_per_grab < 1 || (rays_per_lane != 1 && rays_per_lane != 2) ||
        (phased && rays_per_lane != 1))
        return cudaErrorInvalidValue;
    int dev = 0;
    cudaGetDevice(&dev);
    if (phased) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return cudaErrorInvalidValue;
        const bool wide = block_threads > 256;
        switch (df_brick) {
            case 0: return wide ? launch_passes<0, true>(a, block_threads, blocks, sms, s, side)
                                : launch_passes<0, false>(a, block_threads, blocks, sms, s, side);
            case 4: return wide ? launch_passes<4, true>(a, block_threads, blocks, sms, s, side)
                                : launch_passes<4, false>(a, block_threads, blocks, sms, s, side);
            case 8: return wide ? launch_passes<8, true>(a, block_threads, blocks, sms, s, side)
                                : launch_passes<8, false>(a, block_threads, blocks, sms, s, side);
            default: return cudaErrorInvalidValue;
        }
    }
    if (blocks <= 0) blocks = batch_max_blocks(df_brick, block_threads, rays_per_lane, dev);
    if (blocks <= 0) return cudaErrorInvalidConfiguration;
    const bool two = rays_per_lane == 2;
    using K = void (*)(BatchLaunch);
    // [brick 0 / 4 / 8][one / two rays][narrow / wide blocks]
    const K table[3][2][2] = {
        {{k_batch_trace<0, 1, false>, k_batch_trace<0, 1, true>}, {k_batch_trace<0, 2, false>, k_batch_trace<0, 2, true>}},
        {{k_batch_trace<4, 1, false>, k_batch_trace<4, 1, true>}, {k_batch_trace<4, 2, false>, k_batch_trace<4, 2, true>}},
        {{k_batch_trace<8, 1, false>, k_batch_trace<8, 1, true>}, {k_batch_trace<8, 2, false>, k_batch_trace<8, 2, true>}}};
    const int bi = df_brick == 0 ? 0 : (df_brick == 4 ? 1 : (df_brick == 8 ? 2 : -1));
    if (bi < 0) return cudaErrorInvalidValue;
    table[bi][two ? 1 : 0][block_threads > 256 ? 1 : 0]<<<blocks, block_threads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t df_to_bricks(const uint8_t* df, uint8_t* out, int X, int Y, int Z, int brick, cudaStream_t s) {
    if (brick != 4 && brick != 8) return cudaErrorInvalidValue;
    const int bx = (X + brick - 1) / brick, by = (Y + brick - 1) / brick, bz = (Z + brick - 1) / brick;
    const size_t total = (size_t)bx * by * bz * brick * brick * brick;
    const unsigned grid = (unsigned)((total + 255) / 256);
    if (brick == 4) k_df_bricks<4><<<grid, 256, 0, s>>>(df, out, X, Y, Z, bx, by, total);
    else k_df_bricks<8><<<grid, 256, 0, s>>>(df, out, X, Y, Z, bx, by, total);
    return cudaGetLastError();
}

}  // namespace vpt
