// libvpt C ABI of the world batch: device buffers per world, the launch
// tables of the persistent kernel, its CUDA-graph replay, the per-world plain
// path it is compared against, and the launch-shape autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "vpt.h"

using namespace vpt;

namespace {

struct HostWorld {
    int X = 0, Y = 0, Z = 0, W = 0, H = 0;
    uint8_t* vox = nullptr;
    uint8_t* df = nullptr;          // x-fastest
    uint8_t* df_brick[2] = {};      // 4^3 and 8^3 brick layouts (built on demand)
    vpt_block* blocks = nullptr;
    int n_blocks = 0;
    float* t = nullptr;
    uint8_t* face = nullptr;
    uint8_t* block = nullptr;
    int32_t* hit = nullptr;
    uint16_t* steps = nullptr;
    uint8_t* shadow = nullptr;
    float* sh = nullptr;
    float* cocg = nullptr;
    float* luma = nullptr;
    float* aosky = nullptr;
    vpt_camera cam{};
    bool have_cam = false;
};

int brick_slot(int brick) { return brick == 4 ? 0 : 1; }

}  // namespace

struct vpt_batch {
    vpt_batch_config cfg{};
    int dev = 0;
    cudaStream_t stream = nullptr;
    BatchSide side{nullptr, nullptr, nullptr};   // the phased launch's shadow stream
    std::string err;
    std::vector<HostWorld> worlds;
    bool df_valid = false;
    bool brick_valid[2] = {false, false};
    vpt_batch_tuning tuning{};
    // launch tables (device) and the per-frame constants
    BatchWorld* d_worlds = nullptr;
    int* d_tile_begin = nullptr;
    BatchFrame* d_frame = nullptr;
    BatchFrame* h_frame = nullptr;  // pinned staging of *d_frame
    cudaEvent_t frame_copied = nullptr;
    int* d_queue = nullptr;
    Counters* counters = nullptr;
    bool stats = false;
    bool tables_valid = false;
    int tables_brick = -1;
    int n_tiles = 0;
    // graph of [zero queue, persistent launch]
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    bool graph_stats = false;
    uint64_t launches = 0;
    std::vector<void*> allocs;
};

namespace {

vpt_status bfail(vpt_batch* b, vpt_status s, const char* fmt, ...) {
    if (b) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        b->err = buf;
    }
    return s;
}

#define BCK(b, call)                                                                           \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? VPT_ERR_OOM : VPT_ERR_CUDA,    \
                         "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

vpt_status balloc(vpt_batch* b, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return bfail(b, e == cudaErrorMemoryAllocation ? VPT_ERR_OOM : VPT_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                     cudaGetErrorString(e));
    }
    b->allocs.push_back(*p);
    return VPT_OK;
}

CamView cam_of(const vpt_camera& c) {
    CamView v;
    memcpy(v.inv_view, c.inv_view, sizeof v.inv_view);
    memcpy(v.inv_proj, c.inv_proj, sizeof v.inv_proj);
    v.pos[0] = c.position[0];
    v.pos[1] = c.position[1];
    v.pos[2] = c.position[2];
    return v;
}

WorldView view_of(const HostWorld& h, int brick) {
    WorldView w;
    w.vox = h.vox;
    w.df = brick == 0 ? h.df : h.df_brick[brick_slot(brick)];
    w.X = h.X;
    w.Y = h.Y;
    w.Z = h.Z;
    w.blocks = h.blocks;
    w.n_blocks = h.n_blocks;
    w.bx = brick ? (h.X + brick - 1) / brick : 0;
    w.by = brick ? (h.Y + brick - 1) / brick : 0;
    return w;
}

vpt_status check_ready(vpt_batch* b) {
    if (b->worlds.empty()) return bfail(b, VPT_ERR_STATE, "the batch holds no world");
    if (!b->df_valid) return bfail(b, VPT_ERR_STATE, "distance fields not built (call vpt_batch_build_df)");
    for (size_t k = 0; k < b->worlds.size(); k++)
        if (!b->worlds[k].have_cam) return bfail(b, VPT_ERR_STATE, "world %zu has no camera", k);
    return VPT_OK;
}

vpt_status ensure_bricks(vpt_batch* b, int brick) {
    if (brick == 0) return VPT_OK;
    const int slot = brick_slot(brick);
    if (b->brick_valid[slot]) return VPT_OK;
    for (HostWorld& h : b->worlds) {
        if (!h.df_brick[slot]) {
            const size_t n = (size_t)((h.X + brick - 1) / brick) * ((h.Y + brick - 1) / brick) *
                             ((h.Z + brick - 1) / brick) * brick * brick * brick;
            vpt_status s = balloc(b, (void**)&h.df_brick[slot], n);
            if (s != VPT_OK) return s;
        }
        BCK(b, df_to_bricks(h.df, h.df_brick[slot], h.X, h.Y, h.Z, brick, b->stream));
        b->launches += 1;
    }
    b->brick_valid[slot] = true;
    b->tables_valid = false;
    return VPT_OK;
}

// Uploads the world table and the tile prefix sums for the given layout.
vpt_status build_tables(vpt_batch* b, int brick) {
    vpt_status s = ensure_bricks(b, brick);
    if (s != VPT_OK) return s;
    if (b->tables_valid && b->tables_brick == brick) return VPT_OK;
    const int n = (int)b->worlds.size();
    std::vector<BatchWorld> hw(n);
    std::vector<int> begin(n + 1);
    long long tiles = 0;
    for (int k = 0; k < n; k++) {
        const HostWorld& h = b->worlds[k];
        BatchWorld& d = hw[k];
        d.w = view_of(h, brick);
        d.cam = cam_of(h.cam);
        d.W = h.W;
        d.H = h.H;
        d.tiles_x = (h.W + 7) / 8;
        d.tile_begin = (int)tiles;
        begin[k] = (int)tiles;
        tiles += (long long)d.tiles_x * ((h.H + 3) / 4);
        d.t = h.t;
        d.face = h.face;
        d.block = h.block;
        d.hit = h.hit;
        d.steps = h.steps;
        d.shadow = h.shadow;
        d.sh = h.sh;
        d.cocg = h.cocg;
        d.luma = h.luma;
        d.aosky = h.aosky;
    }
    if (tiles > (1LL << 30)) return bfail(b, VPT_ERR_INVALID_ARG, "batch too large: %lld tiles", tiles);
    begin[n] = (int)tiles;
    BCK(b, cudaMemcpyAsync(b->d_worlds, hw.data(), sizeof(BatchWorld) * n, cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(b->d_tile_begin, begin.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));   // the host vectors go out of scope
    b->n_tiles = (int)tiles;
    b->tables_valid = true;
    b->tables_brick = brick;
    b->graph_valid = false;
    return VPT_OK;
}

vpt_status stage_frame(vpt_batch* b, const vpt_frame* f) {
    BCK(b, cudaEventSynchronize(b->frame_copied));   // the previous copy has read the staging buffer
    BatchFrame& fr = *b->h_frame;
    fr.primary_max_steps = b->cfg.primary_max_steps;
    fr.shadow_max_steps = b->cfg.shadow_max_steps;
    fr.sun[0] = f->sun_dir[0];
    fr.sun[1] = f->sun_dir[1];
    fr.sun[2] = f->sun_dir[2];
    fr.d.diffuse_max_steps = b->cfg.diffuse_max_steps;
    fr.d.bounce_shadow_max_steps = b->cfg.bounce_shadow_max_steps;
    fr.d.bounces = b->cfg.bounces;
    fr.d.spp = b->cfg.spp;
    fr.d.frame_index = f->frame_index;
    fr.d.seed = f->seed;
    fr.d.lighting = gi_lighting(f);
    BCK(b, cudaMemcpyAsync(b->d_frame, b->h_frame, sizeof(BatchFrame), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaEventRecord(b->frame_copied, b->stream));
    return VPT_OK;
}

BatchLaunch launch_args(vpt_batch* b) {
    BatchLaunch a;
    a.worlds = b->d_worlds;
    a.tile_begin = b->d_tile_begin;
    a.frame = b->d_frame;
    a.n_worlds = (int)b->worlds.size();
    a.n_tiles = b->n_tiles;
    a.tiles_per_grab = b->tuning.tiles_per_grab;
    a.queue = b->d_queue;
    a.stats = b->stats ? b->counters : nullptr;
    return a;
}

vpt_status ensure_side(vpt_batch* b) {
    // each handle created once; a call after a failed creation retries the missing ones
    if (!b->side.side) {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        BCK(b, cudaStreamCreateWithPriority(&b->side.side, cudaStreamNonBlocking, hi));
    }
    if (!b->side.fork) BCK(b, cudaEventCreateWithFlags(&b->side.fork, cudaEventDisableTiming));
    if (!b->side.join) BCK(b, cudaEventCreateWithFlags(&b->side.join, cudaEventDisableTiming));
    return VPT_OK;
}

vpt_status launch_persistent(vpt_batch* b) {
    BCK(b, cudaMemsetAsync(b->d_queue, 0, 3 * sizeof(int), b->stream));
    if (b->tuning.phased) {
        const vpt_status st = ensure_side(b);
        if (st != VPT_OK) return st;
    }
    BCK(b, batch_trace(launch_args(b), b->tuning.df_brick, b->tuning.block_threads, b->tuning.rays_per_lane,
                       b->tuning.blocks, b->tuning.phased, b->stream, b->tuning.phased ? &b->side : nullptr));
    b->launches += b->tuning.phased ? 3 : 1;
    return VPT_OK;
}

vpt_status launch_graph(vpt_batch* b) {
    if (!b->graph_valid || b->graph_stats != b->stats) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        if (b->tuning.phased) {
            const vpt_status st = ensure_side(b);
            if (st != VPT_OK) return st;
        }
        BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e1 = cudaMemsetAsync(b->d_queue, 0, 3 * sizeof(int), b->stream);
        cudaError_t e2 = batch_trace(launch_args(b), b->tuning.df_brick, b->tuning.block_threads, b->tuning.rays_per_lane,
                                     b->tuning.blocks, b->tuning.phased, b->stream,
                                     b->tuning.phased ? &b->side : nullptr);
        cudaError_t e3 = cudaStreamEndCapture(b->stream, &g);
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return bfail(b, VPT_ERR_CUDA, "graph capture failed: %s / %s / %s", cudaGetErrorString(e1),
                         cudaGetErrorString(e2), cudaGetErrorString(e3));
        }
        cudaError_t e4 = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e4 != cudaSuccess) {
            b->graph = nullptr;
            return bfail(b, VPT_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e4));
        }
        b->graph_valid = true;
        b->graph_stats = b->stats;
    }
    BCK(b, cudaGraphLaunch(b->graph, b->stream));
    b->launches += b->tuning.phased ? 3 : 1;
    return VPT_OK;
}

vpt_status launch_per_world(vpt_batch* b, const vpt_frame* f) {
    DiffuseArgs a;
    a.diffuse_max_steps = b->cfg.diffuse_max_steps;
    a.bounce_shadow_max_steps = b->cfg.bounce_shadow_max_steps;
    a.bounces = b->cfg.bounces;
    a.spp = b->cfg.spp;
    a.frame_index = f->frame_index;
    a.seed = f->seed;
    a.lighting = gi_lighting(f);
    Counters* st = b->stats ? b->counters : nullptr;
    for (HostWorld& h : b->worlds) {
        const WorldView w = view_of(h, 0);
        const CamView cam = cam_of(h.cam);
        BCK(b, trace_primary(w, cam, h.W, h.H, b->cfg.primary_max_steps, 0,
                             GBufferOut{h.t, h.face, h.block, h.hit, h.steps}, st, b->stream));
        BCK(b, trace_shadow(w, cam, h.W, h.H, b->cfg.shadow_max_steps, f->sun_dir, 0, h.t, h.face, h.shadow, st,
                            b->stream));
        BCK(b, trace_diffuse(w, cam, h.W, h.H, a, 0, h.t, h.face, GIOut{h.sh, h.cocg, h.luma, h.aosky}, st,
                             b->stream));
        b->launches += 3;
    }
    return VPT_OK;
}

bool valid_tuning(const vpt_batch_tuning& t) {
    return t.block_threads >= 64 && t.block_threads <= 512 && (t.block_threads & 31) == 0 && t.tiles_per_grab >= 1 &&
           t.tiles_per_grab <= 16 && (t.df_brick == 0 || t.df_brick == 4 || t.df_brick == 8) && t.blocks >= 0 &&
           (t.rays_per_lane == 1 || t.rays_per_lane == 2) && (t.phased == 0 || (t.phased == 1 && t.rays_per_lane == 1));
}

}  // namespace

extern "C" {

vpt_status vpt_batch_default_config(vpt_batch_config* cfg) {
    if (!cfg) return VPT_ERR_INVALID_ARG;
    memset(cfg, 0, sizeof *cfg);
    cfg->device = 0;
    cfg->max_worlds = 64;
    cfg->primary_max_steps = 350;
    cfg->shadow_max_steps = 350;
    cfg->diffuse_max_steps = 48;
    cfg->bounce_shadow_max_steps = 128;
    cfg->bounces = 1;
    cfg->spp = 1;
    return VPT_OK;
}

vpt_status vpt_batch_create(vpt_batch** out, const vpt_batch_config* cfg) {
    if (!out || !cfg) return VPT_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->max_worlds < 1 || cfg->max_worlds > kBatchMaxWorlds || cfg->primary_max_steps < 0 ||
        cfg->shadow_max_steps < 0 || cfg->diffuse_max_steps < 0 || cfg->bounce_shadow_max_steps < 0 ||
        cfg->bounces < 0 || cfg->bounces > 8 || cfg->spp < 1 || cfg->spp > 32)
        return VPT_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return VPT_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) return VPT_ERR_INVALID_ARG;
    vpt_batch* b = new (std::nothrow) vpt_batch();
    if (!b) return VPT_ERR_OOM;
    b->cfg = *cfg;
    b->dev = cfg->device;
    b->tuning.block_threads = 256;
    b->tuning.tiles_per_grab = 1;
    b->tuning.df_brick = 0;
    b->tuning.blocks = 0;
    b->tuning.rays_per_lane = 1;
    vpt_status s = VPT_OK;
    if (cudaSetDevice(b->dev) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->frame_copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost((void**)&b->h_frame, sizeof(BatchFrame)) != cudaSuccess)
        s = VPT_ERR_CUDA;
    if (s == VPT_OK) s = balloc(b, (void**)&b->d_worlds, sizeof(BatchWorld) * cfg->max_worlds);
    if (s == VPT_OK) s = balloc(b, (void**)&b->d_tile_begin, sizeof(int) * (cfg->max_worlds + 1));
    if (s == VPT_OK) s = balloc(b, (void**)&b->d_frame, sizeof(BatchFrame));
    if (s == VPT_OK) s = balloc(b, (void**)&b->d_queue, 256);
    if (s == VPT_OK) s = balloc(b, (void**)&b->counters, sizeof(Counters));
    if (s == VPT_OK && cudaMemsetAsync(b->counters, 0, sizeof(Counters), b->stream) != cudaSuccess) s = VPT_ERR_CUDA;
    if (s == VPT_OK && cudaEventRecord(b->frame_copied, b->stream) != cudaSuccess) s = VPT_ERR_CUDA;
    if (s != VPT_OK) {
        vpt_batch_destroy(b);
        return s;
    }
    *out = b;
    return VPT_OK;
}

vpt_status vpt_batch_destroy(vpt_batch* b) {
    if (!b) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(b->dev);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->side.side) cudaStreamSynchronize(b->side.side);
    if (b->side.fork) cudaEventDestroy(b->side.fork);
    if (b->side.join) cudaEventDestroy(b->side.join);
    if (b->side.side) cudaStreamDestroy(b->side.side);
    for (void* p : b->allocs) cudaFree(p);
    if (b->h_frame) cudaFreeHost(b->h_frame);
    if (b->frame_copied) cudaEventDestroy(b->frame_copied);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return VPT_OK;
}

const char* vpt_batch_last_error(const vpt_batch* b) { return b ? b->err.c_str() : ""; }

vpt_status vpt_batch_add_world(vpt_batch* b, const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z,
                               const vpt_block* table, int32_t n_blocks, int32_t width, int32_t height,
                               int32_t* world_id) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (!voxels || !table) return bfail(b, VPT_ERR_INVALID_ARG, "voxels or block table is NULL");
    if ((int)b->worlds.size() >= b->cfg.max_worlds)
        return bfail(b, VPT_ERR_INVALID_ARG, "batch is full (%d worlds)", b->cfg.max_worlds);
    if (X < 1 || Y < 1 || Z < 1 || X > 1024 || Y > 1024 || Z > 1024)
        return bfail(b, VPT_ERR_INVALID_ARG, "bad world dimensions %d x %d x %d", X, Y, Z);
    if (n_blocks < 1 || n_blocks > 256) return bfail(b, VPT_ERR_INVALID_ARG, "block table must have 1..256 entries");
    if (width < 1 || height < 1 || width > 4096 || height > 4096)
        return bfail(b, VPT_ERR_INVALID_ARG, "bad ray tile %d x %d", width, height);
    cudaSetDevice(b->dev);
    HostWorld h;
    h.X = X; h.Y = Y; h.Z = Z; h.W = width; h.H = height;
    const size_t nv = (size_t)X * Y * Z, np = (size_t)width * height;
    vpt_status s;
#define A(ptr, bytes) \
    if ((s = balloc(b, (void**)&(ptr), (bytes))) != VPT_OK) return s
    A(h.vox, nv);
    A(h.df, nv);
    A(h.blocks, 256 * sizeof(vpt_block));
    A(h.t, np * 4);
    A(h.face, np);
    A(h.block, np);
    A(h.hit, np * 12);
    A(h.steps, np * 2);
    A(h.shadow, np);
    A(h.sh, np * 16);
    A(h.cocg, np * 8);
    A(h.luma, np * 4);
    A(h.aosky, np * 8);
#undef A
    h.n_blocks = n_blocks;
    BCK(b, cudaMemcpyAsync(h.vox, voxels, nv, cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemsetAsync(h.blocks, 0, 256 * sizeof(vpt_block), b->stream));
    BCK(b, cudaMemcpyAsync(h.blocks, table, (size_t)n_blocks * sizeof(vpt_block), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    b->worlds.push_back(h);
    b->df_valid = false;
    b->brick_valid[0] = b->brick_valid[1] = false;
    b->tables_valid = false;
    b->graph_valid = false;
    if (world_id) *world_id = (int32_t)b->worlds.size() - 1;
    return VPT_OK;
}

vpt_status vpt_batch_set_camera(vpt_batch* b, int32_t world, const vpt_camera* cam) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (!cam || world < 0 || world >= (int)b->worlds.size())
        return bfail(b, VPT_ERR_INVALID_ARG, "bad world index %d or NULL camera", world);
    b->worlds[world].cam = *cam;
    b->worlds[world].have_cam = true;
    b->tables_valid = false;   // the table holds the cameras
    return VPT_OK;
}

vpt_status vpt_batch_build_df(vpt_batch* b) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (b->worlds.empty()) return bfail(b, VPT_ERR_STATE, "the batch holds no world");
    cudaSetDevice(b->dev);
    for (HostWorld& h : b->worlds) {
        int launches = 0;
        BCK(b, df_build(h.vox, h.df, h.X, h.Y, h.Z, b->stream, &launches));
        b->launches += (uint64_t)launches;
    }
    b->df_valid = true;
    b->brick_valid[0] = b->brick_valid[1] = false;
    b->tables_valid = false;
    vpt_status s = ensure_bricks(b, b->tuning.df_brick);
    if (s != VPT_OK) return s;
    BCK(b, cudaStreamSynchronize(b->stream));
    return VPT_OK;
}

vpt_status vpt_batch_read_df(vpt_batch* b, int32_t world, uint8_t* host, size_t bytes) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (world < 0 || world >= (int)b->worlds.size() || !host) return bfail(b, VPT_ERR_INVALID_ARG, "bad arguments");
    const HostWorld& h = b->worlds[world];
    const size_t n = (size_t)h.X * h.Y * h.Z;
    if (bytes != n) return bfail(b, VPT_ERR_INVALID_ARG, "need %zu bytes, got %zu", n, bytes);
    if (!b->df_valid) return bfail(b, VPT_ERR_STATE, "distance fields not built");
    cudaSetDevice(b->dev);
    BCK(b, cudaMemcpyAsync(host, h.df, n, cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return VPT_OK;
}

vpt_status vpt_batch_set_tuning(vpt_batch* b, const vpt_batch_tuning* t) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (!t || !valid_tuning(*t)) return bfail(b, VPT_ERR_INVALID_ARG, "bad batch tuning");
    if (t->block_threads != b->tuning.block_threads || t->tiles_per_grab != b->tuning.tiles_per_grab ||
        t->df_brick != b->tuning.df_brick || t->blocks != b->tuning.blocks)
        b->graph_valid = false;
    b->tuning = *t;
    return VPT_OK;
}

vpt_status vpt_batch_get_tuning(const vpt_batch* b, vpt_batch_tuning* t) {
    if (!b || !t) return VPT_ERR_INVALID_ARG;
    *t = b->tuning;
    return VPT_OK;
}

vpt_status vpt_batch_trace(vpt_batch* b, const vpt_frame* f, int32_t mode) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (!f) return bfail(b, VPT_ERR_INVALID_ARG, "frame is NULL");
    if (mode != VPT_BATCH_GRAPH && mode != VPT_BATCH_PERSISTENT && mode != VPT_BATCH_PER_WORLD)
        return bfail(b, VPT_ERR_INVALID_ARG, "bad batch mode %d", mode);
    vpt_status s = check_ready(b);
    if (s != VPT_OK) return s;
    cudaSetDevice(b->dev);
    if (mode == VPT_BATCH_PER_WORLD) return launch_per_world(b, f);
    if ((s = build_tables(b, b->tuning.df_brick)) != VPT_OK) return s;
    if ((s = stage_frame(b, f)) != VPT_OK) return s;
    return mode == VPT_BATCH_GRAPH ? launch_graph(b) : launch_persistent(b);
}

vpt_status vpt_batch_autotune(vpt_batch* b, const vpt_frame* f, int32_t reps, vpt_batch_tune_record* records,
                              int32_t max_records, int32_t* n_records) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (!f || reps < 1 || reps > 100 || max_records < 0 || (max_records > 0 && !records))
        return bfail(b, VPT_ERR_INVALID_ARG, "bad autotune arguments");
    vpt_status s = check_ready(b);
    if (s != VPT_OK) return s;
    cudaSetDevice(b->dev);
    const bool stats = b->stats;
    b->stats = false;
    const vpt_batch_tuning start = b->tuning;
    vpt_batch_tuning best = start;
    float best_ms = -1.0f;
    int n = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    const int threads[3] = {128, 256, 512}, grabs[3] = {1, 2, 4}, bricks[3] = {0, 4, 8}, rays[2] = {1, 2};
    // one or two rays per lane in the one-kernel launch, and the phased launch (one ray per lane)
    for (int ri = 0; ri < 3 && s == VPT_OK; ri++)
    for (int bi = 0; bi < 3 && s == VPT_OK; bi++) {
        for (int ti = 0; ti < 3 && s == VPT_OK; ti++) {
            for (int gi = 0; gi < 3 && s == VPT_OK; gi++) {
                vpt_batch_tuning t = start;
                t.df_brick = bricks[bi];
                t.block_threads = threads[ti];
                t.tiles_per_grab = grabs[gi];
                t.rays_per_lane = ri < 2 ? rays[ri] : 1;
                t.phased = ri == 2 ? 1 : 0;
                t.blocks = 0;
                b->tuning = t;
                b->graph_valid = false;
                if ((s = build_tables(b, t.df_brick)) != VPT_OK) break;
                if ((s = stage_frame(b, f)) != VPT_OK) break;
                if ((s = launch_persistent(b)) != VPT_OK) break;   // warm-up
                std::vector<float> ms;
                for (int r = 0; r < reps && s == VPT_OK; r++) {
                    cudaEventRecord(e0, b->stream);
                    s = launch_persistent(b);
                    cudaEventRecord(e1, b->stream);
                    if (s != VPT_OK) break;
                    if (cudaEventSynchronize(e1) != cudaSuccess) { s = bfail(b, VPT_ERR_CUDA, "autotune launch failed"); break; }
                    float m = 0.0f;
                    cudaEventElapsedTime(&m, e0, e1);
                    ms.push_back(m);
                }
                if (s != VPT_OK) break;
                std::sort(ms.begin(), ms.end());
                const float med = ms[ms.size() / 2];
                if (n < max_records) {
                    records[n].tuning = t;
                    records[n].ms = med;
                    records[n].pad = 0.0f;
                }
                n++;
                if (best_ms < 0.0f || med < best_ms) {
                    best_ms = med;
                    best = t;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->stats = stats;
    b->tuning = s == VPT_OK ? best : start;
    b->graph_valid = false;
    if (n_records) *n_records = std::min(n, max_records);
    if (s != VPT_OK) return s;
    BCK(b, cudaStreamSynchronize(b->stream));
    return VPT_OK;
}

vpt_status vpt_batch_read_plane(vpt_batch* b, int32_t world, int32_t plane, void* host, size_t bytes) {
    if (!b) return VPT_ERR_INVALID_ARG;
    if (world < 0 || world >= (int)b->worlds.size() || !host)
        return bfail(b, VPT_ERR_INVALID_ARG, "bad world index %d or NULL destination", world);
    const HostWorld& h = b->worlds[world];
    const size_t np = (size_t)h.W * h.H;
    const void* src = nullptr;
    size_t n = 0;
    switch (plane) {
        case VPT_PLANE_T: src = h.t; n = np * 4; break;
        case VPT_PLANE_FACE: src = h.face; n = np; break;
        case VPT_PLANE_BLOCK: src = h.block; n = np; break;
        case VPT_PLANE_HIT: src = h.hit; n = np * 12; break;
        case VPT_PLANE_STEPS: src = h.steps; n = np * 2; break;
        case VPT_PLANE_SHADOW: src = h.shadow; n = np; break;
        case VPT_PLANE_GI_SH: src = h.sh; n = np * 16; break;
        case VPT_PLANE_GI_COCG: src = h.cocg; n = np * 8; break;
        case VPT_PLANE_GI_LUMA: src = h.luma; n = np * 4; break;
        case VPT_PLANE_GI_AOSKY: src = h.aosky; n = np * 8; break;
        default: return bfail(b, VPT_ERR_INVALID_ARG, "plane %d is not a batch plane", plane);
    }
    if (bytes != n) return bfail(b, VPT_ERR_INVALID_ARG, "plane %d needs %zu bytes, got %zu", plane, n, bytes);
    cudaSetDevice(b->dev);
    BCK(b, cudaMemcpyAsync(host, src, n, cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return VPT_OK;
}

vpt_status vpt_batch_world_info(const vpt_batch* b, int32_t world, int32_t dims[3], int32_t tile[2]) {
    if (!b || world < 0 || world >= (int)b->worlds.size()) return VPT_ERR_INVALID_ARG;
    const HostWorld& h = b->worlds[world];
    if (dims) { dims[0] = h.X; dims[1] = h.Y; dims[2] = h.Z; }
    if (tile) { tile[0] = h.W; tile[1] = h.H; }
    return VPT_OK;
}

vpt_status vpt_batch_count(const vpt_batch* b, int32_t* n) {
    if (!b || !n) return VPT_ERR_INVALID_ARG;
    *n = (int32_t)b->worlds.size();
    return VPT_OK;
}

vpt_status vpt_batch_synchronize(vpt_batch* b) {
    if (!b) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(b->dev);
    BCK(b, cudaStreamSynchronize(b->stream));
    return VPT_OK;
}

vpt_status vpt_batch_set_stats(vpt_batch* b, int32_t enabled) {
    if (!b) return VPT_ERR_INVALID_ARG;
    b->stats = enabled != 0;
    return VPT_OK;
}

vpt_status vpt_batch_read_stats(vpt_batch* b, vpt_stats* out) {
    if (!b || !out) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(b->dev);
    Counters c;
    BCK(b, cudaMemcpyAsync(&c, b->counters, sizeof c, cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaMemsetAsync(b->counters, 0, sizeof(Counters), b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    for (int k = 0; k < 6; k++) {
        out->rays[k] = c.rays[k];
        out->steps[k] = c.steps[k];
    }
    return VPT_OK;
}

vpt_status vpt_batch_launch_count(const vpt_batch* b, uint64_t* out) {
    if (!b || !out) return VPT_ERR_INVALID_ARG;
    *out = b->launches;
    return VPT_OK;
}

vpt_status vpt_batch_get_stream(const vpt_batch* b, void** stream) {
    if (!b || !stream) return VPT_ERR_INVALID_ARG;
    *stream = (void*)b->stream;
    return VPT_OK;
}

}  // extern "C"
