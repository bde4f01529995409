// libvpt C ABI: context, device buffers, pass sequencing and instrumentation.
// The per-frame pass order and the ping-pong history follow Core/Pipeline.cpp
// (initial trace :1959-2016, diffuse :2169-2281, SVGF :2284-2615, shadow
// :2790-2850, colour :3603-3821, swaps :1775-1788 and :1970-1971).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "textures.cuh"
#include "vpt.h"

using namespace vpt;

namespace {

enum GB { GB_T = 0, GB_FACE, GB_BLOCK, GB_HIT, GB_STEPS, GB_N };
enum GI { GI_SH = 0, GI_COCG, GI_LUMA, GI_AOSKY, GI_N };
enum HI { HI_SH = 0, HI_COCG, HI_UTIL, HI_AOSKY, HI_N };
enum FI { FI_SH = 0, FI_COCG, FI_VAR, FI_AOSKY, FI_N };

struct PlaneMeta {
    int channels;
    int typed;    // 1: storage type (f32/f16); 0: fixed dtype below
    int dtype;
    int gi;       // 1: on the GI grid; 0: at the G-buffer's resolution
};

PlaneMeta plane_meta(int plane) {
    switch (plane) {
        case VPT_PLANE_T: case VPT_PLANE_PREV_T: return {1, 1, 0, 0};
        case VPT_PLANE_FACE: case VPT_PLANE_BLOCK: case VPT_PLANE_SHADOW:
        case VPT_PLANE_PREV_FACE: case VPT_PLANE_PREV_BLOCK: return {1, 0, VPT_DTYPE_U8, 0};
        case VPT_PLANE_HIT: return {3, 0, VPT_DTYPE_I32, 0};
        case VPT_PLANE_STEPS: return {1, 0, VPT_DTYPE_U16, 0};
        case VPT_PLANE_GI_SH: case VPT_PLANE_PRE_SH: case VPT_PLANE_TEMP_SH: case VPT_PLANE_HIST_SH:
        case VPT_PLANE_VAR_SH: case VPT_PLANE_DEN_SH: return {4, 1, 0, 1};
        case VPT_PLANE_TEMP_UTIL: case VPT_PLANE_HIST_UTIL: return {4, 1, 0, 1};
        case VPT_PLANE_GI_COCG: case VPT_PLANE_PRE_COCG: case VPT_PLANE_TEMP_COCG: case VPT_PLANE_HIST_COCG:
        case VPT_PLANE_VAR_COCG: case VPT_PLANE_DEN_COCG: return {2, 1, 0, 1};
        case VPT_PLANE_GI_AOSKY: case VPT_PLANE_PRE_AOSKY: case VPT_PLANE_TEMP_AOSKY: case VPT_PLANE_HIST_AOSKY:
        case VPT_PLANE_DEN_AOSKY: return {2, 1, 0, 1};
        case VPT_PLANE_GI_LUMA: case VPT_PLANE_PRE_LUMA: case VPT_PLANE_VAR_VARIANCE:
        case VPT_PLANE_DEN_VARIANCE: return {1, 1, 0, 1};
        case VPT_PLANE_COLOR: return {3, 1, 0, 0};
        case VPT_PLANE_SPEC: case VPT_PLANE_SPEC_OUT: case VPT_PLANE_SPEC_DEN: return {4, 1, 0, 1};
        case VPT_PLANE_SPEC_HIT: case VPT_PLANE_SPEC_MASK: case VPT_PLANE_SPEC_ACC:
        case VPT_PLANE_SPEC_STABLE_HIT: return {1, 1, 0, 1};
        case VPT_PLANE_GB_ALBEDO: case VPT_PLANE_GB_NORMAL: return {3, 1, 0, 0};
        case VPT_PLANE_GB_PBR: return {4, 1, 0, 0};
        case VPT_PLANE_GB_AO: return {1, 1, 0, 0};
        default: return {0, 0, -1, 0};
    }
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case VPT_DTYPE_F32: case VPT_DTYPE_I32: return 4;
        case VPT_DTYPE_F16: case VPT_DTYPE_U16: return 2;
        case VPT_DTYPE_U8: return 1;
        default: return 0;
    }
}

}  // namespace

struct vpt_ctx {
    vpt_config cfg{};
    int dev = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int fp16 = 0;
    size_t npx = 0;
    // GI grid: gd times coarser than the G-buffer, gw x gh = ngi texels; the
    // G-buffer read at its texel centres (t, face, block), refreshed before
    // the GI passes; with gd == 1 these point at the G-buffer itself
    int gd = 1, gw = 0, gh = 0;
    size_t ngi = 0;
    void* view[3] = {};
    // world
    uint8_t* vox = nullptr;
    uint8_t* df = nullptr;
    int X = 0, Y = 0, Z = 0;
    bool df_valid = false;
    vpt_block* blocks = nullptr;
    int n_blocks = 0;
    // planes
    void* gbuf[2][GB_N] = {};
    uint8_t* shadow = nullptr;
    void* gi[GI_N] = {};
    void* pre[GI_N] = {};
    void* hist[2][HI_N] = {};
    void* var[FI_N] = {};
    void* den[2][FI_N] = {};
    void* color = nullptr;
    // reflection planes on the GI grid: traced radiance (4 ch) and emissive
    // mask, hit distance (this / last frame), the temporal output (4 ch) and
    // stabilised hit distance (this / last frame), accumulation factor, and
    // the first hit-distance blur pass's output
    void* rspec = nullptr;
    void* rmask = nullptr;
    void* rhit[2] = {};
    void* rout[2] = {};
    void* rstable[2] = {};
    void* racc = nullptr;
    void* rhit_tmp = nullptr;
    void* rden1 = nullptr;   // x pass of the reflection denoiser
    void* rden = nullptr;    // y pass: what the colour pass reads with reflection_denoise
    int cur = 0;        // index of this frame's G-buffer / temporal output
    int den_last = 0;   // den set holding the last a-trous output
    // cameras
    vpt_camera cam{};
    bool have_cam = false;
    vpt_camera prev_cam{};
    bool have_prev = false;
    // fused trace: work queue counter and launch-shape knobs
    int* queue = nullptr;
    vpt_tuning tuning{};
    // instrumentation
    Counters* counters = nullptr;
    bool stats = false;
    bool profiling = false;
    cudaEvent_t ev[VPT_PASS_COUNT][2] = {};
    bool ev_used[VPT_PASS_COUNT] = {};
    uint64_t launches = 0;
    std::vector<void*> allocs;
    std::vector<float> host_staging;
    // learned denoiser: full-frame feature tensor, the colour shaded from the
    // raw 1-spp GI, and the cross-stream events
    void* feat = nullptr;
    void* color_raw = nullptr;
    cudaEvent_t ev_net[2] = {};
    // block textures: each array's texels with all mip levels, the per-block
    // layer ids, the sRGB decode table, and the textured G-buffer planes
    // (albedo 3, normal 3, PBR 4, AO 1 channels)
    uint8_t* tex[4] = {};
    TexArray tex_arr[4] = {};
    int* tex_ids = nullptr;
    float* srgb = nullptr;    // 256 sRGB decodes, then 256 values byte / 255
    int tex_grass[10] = {};
    bool textured = false;
    void* gbt[4] = {};
    bool gbt_valid = false;   // the textured planes belong to this frame's G-buffer
    // double-buffered readback (vpt_render_frame_async): copy stream, the
    // copy's completion event, and an fp32 staging plane for fp16 storage
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_color = nullptr, ev_copy = nullptr;
    bool copy_pending = false;
    void* color_stage = nullptr;
    // the sun-shadow pass overlapped with the diffuse trace and SVGF
    // (vpt_tuning.overlap_shadow): its stream, the fork and join events, and
    // whether a forked shadow pass has not been joined yet
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool shadow_forked = false;
    // the temporal pass's history gather queued on the side stream by
    // trace_all (split_temporal), with the arguments it used
    void* tsum = nullptr;
    cudaEvent_t ev_tgather = nullptr;
    bool tgather_pending = false;
    TemporalArgs tgather_args;
};

namespace {

vpt_status fail(vpt_ctx* c, vpt_status s, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return s;
}

#define CK(ctx, call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? VPT_ERR_OOM : VPT_ERR_CUDA,  \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

vpt_status dalloc(vpt_ctx* c, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(c, e == cudaErrorMemoryAllocation ? VPT_ERR_OOM : VPT_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    c->allocs.push_back(*p);
    return VPT_OK;
}

CamView cam_view(const vpt_camera& c) {
    CamView v;
    memcpy(v.inv_view, c.inv_view, sizeof v.inv_view);
    memcpy(v.inv_proj, c.inv_proj, sizeof v.inv_proj);
    v.pos[0] = c.position[0];
    v.pos[1] = c.position[1];
    v.pos[2] = c.position[2];
    return v;
}

WorldView world_view(const vpt_ctx* c) {
    WorldView w;
    w.vox = c->vox;
    w.df = c->df;
    w.X = c->X;
    w.Y = c->Y;
    w.Z = c->Z;
    w.blocks = c->blocks;
    w.n_blocks = c->n_blocks;
    return w;
}

void* plane_ptr(vpt_ctx* c, int plane) {
    int cur = c->cur, prv = 1 - c->cur;
    switch (plane) {
        case VPT_PLANE_T: return c->gbuf[cur][GB_T];
        case VPT_PLANE_FACE: return c->gbuf[cur][GB_FACE];
        case VPT_PLANE_BLOCK: return c->gbuf[cur][GB_BLOCK];
        case VPT_PLANE_HIT: return c->gbuf[cur][GB_HIT];
        case VPT_PLANE_STEPS: return c->gbuf[cur][GB_STEPS];
        case VPT_PLANE_SHADOW: return c->shadow;
        case VPT_PLANE_GI_SH: return c->gi[GI_SH];
        case VPT_PLANE_GI_COCG: return c->gi[GI_COCG];
        case VPT_PLANE_GI_LUMA: return c->gi[GI_LUMA];
        case VPT_PLANE_GI_AOSKY: return c->gi[GI_AOSKY];
        case VPT_PLANE_PRE_SH: return c->pre[GI_SH];
        case VPT_PLANE_PRE_COCG: return c->pre[GI_COCG];
        case VPT_PLANE_PRE_LUMA: return c->pre[GI_LUMA];
        case VPT_PLANE_PRE_AOSKY: return c->pre[GI_AOSKY];
        case VPT_PLANE_TEMP_SH: return c->hist[cur][HI_SH];
        case VPT_PLANE_TEMP_COCG: return c->hist[cur][HI_COCG];
        case VPT_PLANE_TEMP_UTIL: return c->hist[cur][HI_UTIL];
        case VPT_PLANE_TEMP_AOSKY: return c->hist[cur][HI_AOSKY];
        case VPT_PLANE_HIST_SH: return c->hist[prv][HI_SH];
        case VPT_PLANE_HIST_COCG: return c->hist[prv][HI_COCG];
        case VPT_PLANE_HIST_UTIL: return c->hist[prv][HI_UTIL];
        case VPT_PLANE_HIST_AOSKY: return c->hist[prv][HI_AOSKY];
        case VPT_PLANE_PREV_T: return c->gbuf[prv][GB_T];
        case VPT_PLANE_PREV_FACE: return c->gbuf[prv][GB_FACE];
        case VPT_PLANE_PREV_BLOCK: return c->gbuf[prv][GB_BLOCK];
        case VPT_PLANE_VAR_SH: return c->var[FI_SH];
        case VPT_PLANE_VAR_COCG: return c->var[FI_COCG];
        case VPT_PLANE_VAR_VARIANCE: return c->var[FI_VAR];
        case VPT_PLANE_DEN_SH: return c->den[c->den_last][FI_SH];
        case VPT_PLANE_DEN_COCG: return c->den[c->den_last][FI_COCG];
        case VPT_PLANE_DEN_VARIANCE: return c->den[c->den_last][FI_VAR];
        case VPT_PLANE_DEN_AOSKY: return c->den[c->den_last][FI_AOSKY];
        case VPT_PLANE_COLOR: return c->color;
        case VPT_PLANE_SPEC: return c->rspec;
        case VPT_PLANE_SPEC_HIT: return c->rhit[cur];
        case VPT_PLANE_SPEC_MASK: return c->rmask;
        case VPT_PLANE_SPEC_OUT: return c->rout[cur];
        case VPT_PLANE_SPEC_ACC: return c->racc;
        case VPT_PLANE_SPEC_STABLE_HIT: return c->rstable[cur];
        case VPT_PLANE_SPEC_DEN: return c->rden;
        case VPT_PLANE_GB_ALBEDO: return c->gbt[0];
        case VPT_PLANE_GB_NORMAL: return c->gbt[1];
        case VPT_PLANE_GB_PBR: return c->gbt[2];
        case VPT_PLANE_GB_AO: return c->gbt[3];
        default: return nullptr;
    }
}

size_t plane_bytes(const vpt_ctx* c, int plane, int* channels, int* dtype) {
    PlaneMeta m = plane_meta(plane);
    if (m.channels == 0) return 0;
    int dt = m.typed ? (c->fp16 ? VPT_DTYPE_F16 : VPT_DTYPE_F32) : m.dtype;
    if (channels) *channels = m.channels;
    if (dtype) *dtype = dt;
    return (m.gi ? c->ngi : c->npx) * (size_t)m.channels * dtype_size(dt);
}

vpt_status alloc_planes(vpt_ctx* c) {
    const size_t nf = c->npx, n = c->ngi, es = c->fp16 ? 2 : 4;
    vpt_status s;
#define A(ptr, bytes) \
    if ((s = dalloc(c, (void**)&(ptr), (bytes))) != VPT_OK) return s
    for (int k = 0; k < 2; k++) {
        A(c->gbuf[k][GB_T], nf * es);
        A(c->gbuf[k][GB_FACE], nf);
        A(c->gbuf[k][GB_BLOCK], nf);
        A(c->gbuf[k][GB_HIT], nf * 12);
        A(c->gbuf[k][GB_STEPS], nf * 2);
        A(c->hist[k][HI_SH], n * 4 * es);
        A(c->hist[k][HI_COCG], n * 2 * es);
        A(c->hist[k][HI_UTIL], n * 4 * es);
        A(c->hist[k][HI_AOSKY], n * 2 * es);
        A(c->den[k][FI_SH], n * 4 * es);
        A(c->den[k][FI_COCG], n * 2 * es);
        A(c->den[k][FI_VAR], n * es);
        A(c->den[k][FI_AOSKY], n * 2 * es);
    }
    A(c->shadow, nf);
    if (c->gd > 1) {
        A(c->view[0], n * es);
        A(c->view[1], n);
        A(c->view[2], n);
    }
    A(c->gi[GI_SH], n * 4 * es);
    A(c->gi[GI_COCG], n * 2 * es);
    A(c->gi[GI_LUMA], n * es);
    A(c->gi[GI_AOSKY], n * 2 * es);
    A(c->pre[GI_SH], n * 4 * es);
    A(c->pre[GI_COCG], n * 2 * es);
    A(c->pre[GI_LUMA], n * es);
    A(c->pre[GI_AOSKY], n * 2 * es);
    A(c->var[FI_SH], n * 4 * es);
    A(c->var[FI_COCG], n * 2 * es);
    A(c->var[FI_VAR], n * es);
    c->var[FI_AOSKY] = nullptr;
    A(c->color, nf * 3 * es);
    if (c->cfg.reflection_spp > 0) {
        A(c->rspec, n * 4 * es);
        A(c->rmask, n * es);
        A(c->racc, n * es);
        A(c->rhit_tmp, n * es);
        A(c->rden1, n * 4 * es);
        A(c->rden, n * 4 * es);
        for (int k = 0; k < 2; k++) {
            A(c->rhit[k], n * es);
            A(c->rout[k], n * 4 * es);
            A(c->rstable[k], n * es);
        }
    }
    A(c->counters, sizeof(Counters));
    A(c->queue, 256);
#undef A
    return VPT_OK;
}

// Fills the previous-frame G-buffer with "miss" and zeroes the history, the
// state the first frame reprojects from.
vpt_status clear_history(vpt_ctx* c) {
    const size_t n = c->npx, ng = c->ngi, es = c->fp16 ? 2 : 4;
    int prv = 1 - c->cur;
    std::vector<uint8_t> minus_one(n * es);
    if (c->fp16) {
        __half h = __float2half(-1.0f);
        for (size_t k = 0; k < n; k++) memcpy(&minus_one[k * 2], &h, 2);
    } else {
        float f = -1.0f;
        for (size_t k = 0; k < n; k++) memcpy(&minus_one[k * 4], &f, 4);
    }
    CK(c, cudaMemcpyAsync(c->gbuf[prv][GB_T], minus_one.data(), n * es, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemsetAsync(c->gbuf[prv][GB_FACE], kFaceMiss, n, c->stream));
    CK(c, cudaMemsetAsync(c->gbuf[prv][GB_BLOCK], 0, n, c->stream));
    CK(c, cudaMemsetAsync(c->hist[prv][HI_SH], 0, ng * 4 * es, c->stream));
    CK(c, cudaMemsetAsync(c->hist[prv][HI_COCG], 0, ng * 2 * es, c->stream));
    CK(c, cudaMemsetAsync(c->hist[prv][HI_UTIL], 0, ng * 4 * es, c->stream));
    CK(c, cudaMemsetAsync(c->hist[prv][HI_AOSKY], 0, ng * 2 * es, c->stream));
    if (c->cfg.reflection_spp > 0) {
        CK(c, cudaMemsetAsync(c->rhit[prv], 0, ng * es, c->stream));
        CK(c, cudaMemsetAsync(c->rout[prv], 0, ng * 4 * es, c->stream));
        CK(c, cudaMemsetAsync(c->rstable[prv], 0, ng * es, c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));
    c->have_prev = false;
    return VPT_OK;
}

void pass_begin(vpt_ctx* c, int pass, cudaStream_t st = nullptr) {
    if (c->profiling) {
        cudaEventRecord(c->ev[pass][0], st ? st : c->stream);
        c->ev_used[pass] = true;
    }
}
void pass_end(vpt_ctx* c, int pass, cudaStream_t st = nullptr) {
    if (c->profiling) cudaEventRecord(c->ev[pass][1], st ? st : c->stream);
}

vpt_status shadow_run(vpt_ctx* c, const vpt_frame* f, cudaStream_t st);

// Makes the context stream wait for a sun-shadow pass forked onto the side
// stream (before anything that reads the shadow plane).
vpt_status join_shadow(vpt_ctx* c) {
    if (!c->shadow_forked) return VPT_OK;
    c->shadow_forked = false;
    if (cudaStreamWaitEvent(c->stream, c->ev_join, 0) != cudaSuccess) {
        cudaGetLastError();
        return VPT_ERR_CUDA;
    }
    return VPT_OK;
}

vpt_status check_world(vpt_ctx* c) {
    if (!c->vox) return fail(c, VPT_ERR_STATE, "no world uploaded");
    if (!c->df_valid) return fail(c, VPT_ERR_STATE, "distance field not built (call vpt_build_df)");
    if (!c->blocks) return fail(c, VPT_ERR_STATE, "no block table set");
    return VPT_OK;
}

vpt_status check_frame(vpt_ctx* c, const vpt_frame* f) {
    if (!f) return fail(c, VPT_ERR_INVALID_ARG, "frame is NULL");
    if (!c->have_cam) return fail(c, VPT_ERR_STATE, "no primary trace this frame");
    return VPT_OK;
}

// Refreshes the GI-grid reading of this frame's G-buffer (a no-op when the
// grids coincide). Called by every pass that reads it, so planes written by
// the caller between passes are picked up.
vpt_status refresh_view(vpt_ctx* c) {
    const int cur = c->cur;
    if (c->gd == 1) {
        c->view[0] = c->gbuf[cur][GB_T];
        c->view[1] = c->gbuf[cur][GB_FACE];
        c->view[2] = c->gbuf[cur][GB_BLOCK];
        return VPT_OK;
    }
    CK(c, gi_view(c->cfg.width, c->cfg.height, c->gw, c->gh, c->fp16, c->gbuf[cur][GB_T],
                  (const uint8_t*)c->gbuf[cur][GB_FACE], (const uint8_t*)c->gbuf[cur][GB_BLOCK], c->view[0],
                  (uint8_t*)c->view[1], (uint8_t*)c->view[2], c->stream));
    c->launches += 1;
    return VPT_OK;
}

}  // namespace

extern "C" {

const char* vpt_status_string(vpt_status s) {
    switch (s) {
        case VPT_OK: return "ok";
        case VPT_ERR_INVALID_ARG: return "invalid argument";
        case VPT_ERR_OOM: return "out of memory";
        case VPT_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case VPT_ERR_CUDA: return "CUDA error";
        case VPT_ERR_STATE: return "call out of order";
        case VPT_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

int vpt_abi_version(void) { return VPT_ABI_VERSION; }

vpt_status vpt_default_config(vpt_config* cfg) {
    if (!cfg) return VPT_ERR_INVALID_ARG;
    memset(cfg, 0, sizeof *cfg);
    cfg->width = 1920;
    cfg->height = 1080;
    cfg->primary_max_steps = 350;
    cfg->shadow_max_steps = 350;
    cfg->diffuse_max_steps = 48;
    cfg->bounce_shadow_max_steps = 128;
    cfg->bounces = 1;
    cfg->spp = 1;
    cfg->storage = VPT_STORAGE_F32;
    cfg->atrous_iterations = 5;
    cfg->resolution_scale = 1.0f;
    cfg->gi_divisor = 1;
    cfg->reflection_spp = 0;
    cfg->reflection_max_steps = 64;
    cfg->reflection_shadow_max_steps = 150;
    cfg->reflection_temporal = 1;
    cfg->reflection_denoise = 1;
    cfg->color_phi_bias = 3.325f;
    cfg->device = 0;
    return VPT_OK;
}

vpt_status vpt_default_frame(vpt_frame* f) {
    if (!f) return VPT_ERR_INVALID_ARG;
    memset(f, 0, sizeof *f);
    // a morning sun: normalize(0.3, 0.8, 0.5)
    float sx = 0.3f, sy = 0.8f, sz = 0.5f;
    float l = sqrtf((sx * sx + sy * sy) + sz * sz);
    f->sun_dir[0] = sx / l;
    f->sun_dir[1] = sy / l;
    f->sun_dir[2] = sz / l;
    f->time = 1.0f;
    f->sun_radiance[0] = 5.2f;
    f->sun_radiance[1] = 4.9f;
    f->sun_radiance[2] = 4.4f;
    f->moon_radiance[0] = 0.05f;
    f->moon_radiance[1] = 0.06f;
    f->moon_radiance[2] = 0.09f;
    f->frame_index = 0;
    f->seed = 0;
    f->gi_sun_strength = 1.0f;
    f->gi_sky_strength = 1.125f;
    f->diffuse_light_intensity = 1.25f;
    f->temporal = 1;
    return VPT_OK;
}

vpt_status vpt_create(vpt_ctx** out, const vpt_config* cfg) {
    if (!out || !cfg) return VPT_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->width <= 0 || cfg->height <= 0 || cfg->width > 16384 || cfg->height > 16384) return VPT_ERR_INVALID_ARG;
    if (cfg->storage != VPT_STORAGE_F32 && cfg->storage != VPT_STORAGE_F16) return VPT_ERR_INVALID_ARG;
    if (cfg->primary_max_steps < 0 || cfg->shadow_max_steps < 0 || cfg->diffuse_max_steps < 0 ||
        cfg->bounce_shadow_max_steps < 0 || cfg->bounces < 0 || cfg->bounces > 8 || cfg->spp < 1 ||
        cfg->spp > 32 || cfg->atrous_iterations < 0 || cfg->atrous_iterations > 8 ||
        (cfg->denoiser != VPT_DENOISER_SVGF && cfg->denoiser != VPT_DENOISER_ATROUS))
        return VPT_ERR_INVALID_ARG;
    const int gd = cfg->gi_divisor <= 1 ? 1 : cfg->gi_divisor;
    if (cfg->gi_divisor < 0 || gd > 16 || cfg->width % gd != 0 || cfg->height % gd != 0) return VPT_ERR_INVALID_ARG;
    if (cfg->reflection_spp < 0 || cfg->reflection_spp > 16 || cfg->reflection_max_steps < 0 ||
        cfg->reflection_shadow_max_steps < 0)
        return VPT_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return VPT_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) return VPT_ERR_INVALID_ARG;
    vpt_ctx* c = new (std::nothrow) vpt_ctx();
    if (!c) return VPT_ERR_OOM;
    c->cfg = *cfg;
    c->dev = cfg->device;
    c->tuning.refill_threshold = 16;
    c->tuning.trace_blocks = 0;
    c->tuning.overlap_shadow = 1;
    c->tuning.split_temporal = 0;
    c->fp16 = cfg->storage == VPT_STORAGE_F16;
    c->npx = (size_t)cfg->width * (size_t)cfg->height;
    c->gd = gd;
    c->gw = cfg->width / gd;
    c->gh = cfg->height / gd;
    c->ngi = (size_t)c->gw * (size_t)c->gh;
    vpt_status s = VPT_OK;
    if (cudaSetDevice(c->dev) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        s = VPT_ERR_CUDA;
    }
    if (s == VPT_OK) s = alloc_planes(c);
    if (s == VPT_OK) {
        for (int p = 0; p < VPT_PASS_COUNT && s == VPT_OK; p++)
            for (int k = 0; k < 2; k++)
                if (cudaEventCreate(&c->ev[p][k]) != cudaSuccess) s = VPT_ERR_CUDA;
    }
    if (s == VPT_OK && cudaMemsetAsync(c->counters, 0, sizeof(Counters), c->stream) != cudaSuccess) s = VPT_ERR_CUDA;
    if (s == VPT_OK) s = clear_history(c);
    if (s != VPT_OK) {
        vpt_destroy(c);
        return s;
    }
    *out = c;
    return VPT_OK;
}

vpt_status vpt_destroy(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : c->allocs) cudaFree(p);
    if (c->vox) cudaFree(c->vox);
    if (c->df) cudaFree(c->df);
    for (int p = 0; p < VPT_PASS_COUNT; p++)
        for (int k = 0; k < 2; k++)
            if (c->ev[p][k]) cudaEventDestroy(c->ev[p][k]);
    for (int k = 0; k < 2; k++)
        if (c->ev_net[k]) cudaEventDestroy(c->ev_net[k]);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    if (c->ev_color) cudaEventDestroy(c->ev_color);
    if (c->ev_copy) cudaEventDestroy(c->ev_copy);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->side_stream) cudaStreamSynchronize(c->side_stream);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_tgather) cudaEventDestroy(c->ev_tgather);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return VPT_OK;
}

const char* vpt_last_error(const vpt_ctx* c) { return c ? c->err.c_str() : ""; }

vpt_status vpt_upload_world(vpt_ctx* c, const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!voxels) return fail(c, VPT_ERR_INVALID_ARG, "voxels is NULL");
    if (X <= 0 || Y <= 0 || Z <= 0 || X > 2048 || Y > 2048 || Z > 2048 || (size_t)X * Y * Z > ((size_t)1 << 31))
        return fail(c, VPT_ERR_INVALID_ARG, "bad world dimensions %d x %d x %d", X, Y, Z);
    cudaSetDevice(c->dev);
    size_t n = (size_t)X * Y * Z;
    if (c->vox == nullptr || (size_t)c->X * c->Y * c->Z != n) {
        if (c->vox) { cudaFree(c->vox); cudaFree(c->df); }
        c->vox = nullptr;
        c->df = nullptr;
        void* a = nullptr;
        void* b = nullptr;
        cudaError_t e1 = cudaMalloc(&a, n);
        cudaError_t e2 = e1 == cudaSuccess ? cudaMalloc(&b, n) : e1;
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            if (a) cudaFree(a);
            return fail(c, VPT_ERR_OOM, "world allocation of %zu bytes failed", 2 * n);
        }
        c->vox = (uint8_t*)a;
        c->df = (uint8_t*)b;
    }
    c->X = X;
    c->Y = Y;
    c->Z = Z;
    c->df_valid = false;
    CK(c, cudaMemcpyAsync(c->vox, voxels, n, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return VPT_OK;
}

vpt_status vpt_set_block_table(vpt_ctx* c, const vpt_block* table, int32_t n) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!table || n <= 0 || n > 256) return fail(c, VPT_ERR_INVALID_ARG, "block table must have 1..256 entries");
    cudaSetDevice(c->dev);
    if (!c->blocks) {
        void* p = nullptr;
        vpt_status s = dalloc(c, &p, 256 * sizeof(vpt_block));
        if (s != VPT_OK) return s;
        c->blocks = (vpt_block*)p;
    }
    CK(c, cudaMemcpyAsync(c->blocks, table, (size_t)n * sizeof(vpt_block), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    c->n_blocks = n;
    return VPT_OK;
}

namespace {
// K of StopRay (InitialRayTraceFrag.glsl:421): 1 / (2 tan(fov / (2 W))) with the
// vertical fov 2 atan(1 / proj[1][1]), in double precision
float alpha_k(float proj11, int width) {
    const double fov = 2.0 * std::atan(1.0 / (double)proj11);
    return (float)(1.0 / (std::tan(fov / (2.0 * (double)width)) * 2.0));
}

BlockTexView tex_view(const vpt_ctx* c) {
    BlockTexView tv;
    tv.albedo = c->tex_arr[0];
    tv.normal = c->tex_arr[1];
    tv.pbr = c->tex_arr[2];
    tv.emissive = c->tex_arr[3];
    tv.ids = c->tex_ids;
    for (int k = 0; k < 10; k++) tv.grass[k] = c->tex_grass[k];
    tv.srgb = c->srgb;
    tv.unorm = c->srgb ? c->srgb + 256 : nullptr;
    return tv;
}

void dfree(vpt_ctx* c, void** p) {
    if (!*p) return;
    for (size_t k = 0; k < c->allocs.size(); k++)
        if (c->allocs[k] == *p) {
            c->allocs.erase(c->allocs.begin() + (long)k);
            break;
        }
    cudaFree(*p);
    *p = nullptr;
}
}  // namespace

vpt_status vpt_set_block_textures(vpt_ctx* c, const vpt_block_textures* t) {
    if (!c) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    CK(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 4; k++) dfree(c, (void**)&c->tex[k]);
    dfree(c, (void**)&c->tex_ids);
    dfree(c, (void**)&c->srgb);
    c->textured = false;
    c->gbt_valid = false;
    if (!t) return VPT_OK;
    const int S = t->size;
    if (S < 1 || S > 1024 || (S & (S - 1)))
        return fail(c, VPT_ERR_INVALID_ARG, "texture size must be a power of two in 1..1024");
    const uint8_t* src[4] = {t->albedo, t->normal, t->pbr, t->emissive};
    const int layers[4] = {t->albedo_layers, t->normal_layers, t->pbr_layers, t->emissive ? t->emissive_layers : 0};
    const int chans[4] = {4, 4, 4, 1};
    for (int k = 0; k < 3; k++)
        if (!src[k] || layers[k] < 1 || layers[k] > 4096)
            return fail(c, VPT_ERR_INVALID_ARG, "albedo, normal and PBR arrays need 1..4096 layers");
    if (t->emissive && (layers[3] < 1 || layers[3] > 4096))
        return fail(c, VPT_ERR_INVALID_ARG, "the emissive array needs 1..4096 layers");
    int levels = 1;
    while ((S >> (levels - 1)) > 1) levels++;
    vpt_status st;
    for (int k = 0; k < 4; k++) {
        TexArray& a = c->tex_arr[k];
        a = TexArray{};
        if (!src[k]) continue;
        a.layers = layers[k];
        a.channels = chans[k];
        a.size = S;
        a.levels = levels;
        long long off = 0;
        for (int l = 0; l < levels; l++) {
            a.level_off[l] = off;
            off += (long long)a.layers * (S >> l) * (S >> l);
        }
        if ((st = dalloc(c, (void**)&c->tex[k], (size_t)off * a.channels)) != VPT_OK) return st;
        a.texels = c->tex[k];
        CK(c, cudaMemcpyAsync(c->tex[k], src[k], (size_t)a.layers * S * S * a.channels, cudaMemcpyHostToDevice,
                              c->stream));
        for (int l = 0; l + 1 < levels; l++) CK(c, tex_build_mip(a, l, c->tex[k], c->stream));
        c->launches += (uint64_t)(levels - 1);
    }
    // layer ids [albedo | normal | PBR | emissive] and the sRGB decode of a byte
    // (IEC 61966-2-1: c / 12.92 up to 0.04045, else ((c + 0.055) / 1.055)^2.4)
    std::vector<int> ids(640);
    for (int b = 0; b < 128; b++) {
        ids[b] = t->albedo_id[b];
        ids[128 + b] = t->normal_id[b];
        ids[256 + b] = t->pbr_id[b];
        ids[384 + b] = t->emissive_id[b];
        ids[512 + b] = t->transparent[b] ? 1 : 0;
    }
    std::vector<float> lut(512);
    for (int v = 0; v < 256; v++) {
        const float x = (float)v / 255.0f;
        lut[v] = x <= 0.04045f ? x / 12.92f : dpow((x + 0.055f) / 1.055f, 2.4f);
        lut[256 + v] = x;
    }
    if ((st = dalloc(c, (void**)&c->tex_ids, ids.size() * sizeof(int))) != VPT_OK) return st;
    if ((st = dalloc(c, (void**)&c->srgb, lut.size() * sizeof(float))) != VPT_OK) return st;
    CK(c, cudaMemcpyAsync(c->tex_ids, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->srgb, lut.data(), lut.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    for (int k = 0; k < 10; k++) c->tex_grass[k] = t->grass[k];
    const size_t es = c->fp16 ? 2 : 4;
    const size_t ch[4] = {3, 3, 4, 1};
    for (int k = 0; k < 4; k++)
        if (!c->gbt[k] && (st = dalloc(c, &c->gbt[k], c->npx * ch[k] * es)) != VPT_OK) return st;
    CK(c, cudaStreamSynchronize(c->stream));
    c->textured = true;
    return VPT_OK;
}

vpt_status vpt_generate_gbuffer(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!c->textured) return fail(c, VPT_ERR_STATE, "no block textures set (vpt_set_block_textures)");
    if (!c->have_cam) return fail(c, VPT_ERR_STATE, "no G-buffer yet (call vpt_trace_primary)");
    cudaSetDevice(c->dev);
    const BlockTexView tv = tex_view(c);
    pass_begin(c, VPT_PASS_GBUFFER);
    CK(c, gbuffer_textured(cam_view(c->cam), c->cfg.width, c->cfg.height, c->fp16, c->gbuf[c->cur][GB_T],
                           (const uint8_t*)c->gbuf[c->cur][GB_FACE], (const uint8_t*)c->gbuf[c->cur][GB_BLOCK], tv,
                           c->gbt[0], c->gbt[1], c->gbt[2], c->gbt[3], c->stream));
    pass_end(c, VPT_PASS_GBUFFER);
    c->launches += 1;
    c->gbt_valid = true;
    return VPT_OK;
}

vpt_status vpt_build_df(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!c->vox) return fail(c, VPT_ERR_STATE, "no world uploaded");
    cudaSetDevice(c->dev);
    int launches = 0;
    CK(c, df_build(c->vox, c->df, c->X, c->Y, c->Z, c->stream, &launches));
    c->launches += (uint64_t)launches;
    c->df_valid = true;
    return VPT_OK;
}

vpt_status vpt_edit_world(vpt_ctx* c, const uint8_t* voxels, int32_t x0, int32_t y0, int32_t z0, int32_t w,
                          int32_t h, int32_t d) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!c->vox) return fail(c, VPT_ERR_STATE, "no world uploaded");
    if (!voxels || w < 1 || h < 1 || d < 1 || x0 < 0 || y0 < 0 || z0 < 0 || x0 + (int64_t)w > c->X ||
        y0 + (int64_t)h > c->Y || z0 + (int64_t)d > c->Z)
        return fail(c, VPT_ERR_INVALID_ARG, "edit box [%d,%d)x[%d,%d)x[%d,%d) outside the %dx%dx%d world", x0, x0 + w, y0,
                    y0 + h, z0, z0 + d, c->X, c->Y, c->Z);
    cudaSetDevice(c->dev);
    for (int k = 0; k < d; k++) {
        uint8_t* dst = c->vox + (size_t)x0 + (size_t)c->X * ((size_t)y0 + (size_t)c->Y * (size_t)(z0 + k));
        CK(c, cudaMemcpy2DAsync(dst, (size_t)c->X, voxels + (size_t)k * w * h, (size_t)w, (size_t)w, (size_t)h,
                                cudaMemcpyHostToDevice, c->stream));
    }
    if (c->df_valid) {
        int launches = 0;
        CK(c, df_update(c->vox, c->df, c->X, c->Y, c->Z, x0, y0, z0, x0 + w, y0 + h, z0 + d, c->stream, &launches));
        c->launches += (uint64_t)launches;
    }
    CK(c, cudaStreamSynchronize(c->stream));   // the host voxels may be reused
    return VPT_OK;
}

vpt_status vpt_read_df(vpt_ctx* c, uint8_t* host, size_t bytes) {
    if (!c || !host) return VPT_ERR_INVALID_ARG;
    if (!c->df_valid) return fail(c, VPT_ERR_STATE, "distance field not built");
    size_t n = (size_t)c->X * c->Y * c->Z;
    if (bytes < n) return fail(c, VPT_ERR_INVALID_ARG, "buffer too small: %zu < %zu", bytes, n);
    cudaSetDevice(c->dev);
    CK(c, cudaMemcpyAsync(host, c->df, n, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return VPT_OK;
}

vpt_status vpt_df_build_device(const uint8_t* d_voxels, uint8_t* d_df, int32_t X, int32_t Y, int32_t Z, void* stream) {
    if (!d_voxels || !d_df || X <= 0 || Y <= 0 || Z <= 0 || (size_t)X * Y * Z > ((size_t)1 << 31))
        return VPT_ERR_INVALID_ARG;
    int launches = 0;
    cudaError_t e = df_build(d_voxels, d_df, X, Y, Z, (cudaStream_t)stream, &launches);
    return e == cudaSuccess ? VPT_OK : VPT_ERR_CUDA;
}

vpt_status vpt_trace_primary(vpt_ctx* c, const vpt_camera* cam) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!cam) return fail(c, VPT_ERR_INVALID_ARG, "camera is NULL");
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    cudaSetDevice(c->dev);
    c->cam = *cam;
    c->have_cam = true;
    c->gbt_valid = false;
    GBufferOut g;
    g.t = c->gbuf[c->cur][GB_T];
    g.face = (uint8_t*)c->gbuf[c->cur][GB_FACE];
    g.block = (uint8_t*)c->gbuf[c->cur][GB_BLOCK];
    g.hit = (int32_t*)c->gbuf[c->cur][GB_HIT];
    g.steps = (uint16_t*)c->gbuf[c->cur][GB_STEPS];
    // the alpha-tested traversal with block textures (u_ShouldAlphaTest);
    // K = 1 / (2 tan(fov / (2 W))), the vertical field of view from the projection
    AlphaStop stop;
    const bool alpha = c->cfg.alpha_test && c->textured;
    if (alpha) {
        stop.tv = tex_view(c);
        stop.cam = mk3(cam->inv_view[12], cam->inv_view[13], cam->inv_view[14]);
        stop.k = alpha_k(cam->proj[5], c->cfg.width);
    }
    pass_begin(c, VPT_PASS_PRIMARY);
    CK(c, trace_primary(world_view(c), cam_view(*cam), c->cfg.width, c->cfg.height, c->cfg.primary_max_steps, c->fp16,
                        g, c->stats ? c->counters : nullptr, c->stream, alpha ? &stop : nullptr));
    pass_end(c, VPT_PASS_PRIMARY);
    c->launches += 1;
    return VPT_OK;
}

vpt_status vpt_trace_shadow(vpt_ctx* c, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    vpt_status s = join_shadow(c);
    if (s != VPT_OK) return fail(c, s, "joining the previous shadow pass failed");
    return shadow_run(c, f, c->stream);
}

}  // extern "C"

namespace {

// The sun-shadow pass on stream `st` (the context stream, or the side stream
// when it overlaps the diffuse trace and SVGF).
vpt_status shadow_run(vpt_ctx* c, const vpt_frame* f, cudaStream_t st) {
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    if ((s = check_frame(c, f)) != VPT_OK) return s;
    cudaSetDevice(c->dev);
    pass_begin(c, VPT_PASS_SHADOW, st);
    // the alpha-tested shadow rays with block textures (ShouldAlphaTestShadows)
    AlphaStop stop;
    const bool alpha = c->cfg.alpha_test_shadows && c->textured;
    if (alpha) {
        stop.tv = tex_view(c);
        stop.cam = mk3(c->cam.inv_view[12], c->cam.inv_view[13], c->cam.inv_view[14]);
        stop.k = alpha_k(c->cam.proj[5], c->cfg.width);
        stop.flip_x = 0;
        stop.lod_bias = -2;
    }
    CK(c, trace_shadow(world_view(c), cam_view(c->cam), c->cfg.width, c->cfg.height, c->cfg.shadow_max_steps,
                       f->sun_dir, c->fp16, c->gbuf[c->cur][GB_T], (const uint8_t*)c->gbuf[c->cur][GB_FACE],
                       c->shadow, c->stats ? c->counters : nullptr, st, alpha ? &stop : nullptr));
    pass_end(c, VPT_PASS_SHADOW, st);
    c->launches += 1;
    return VPT_OK;
}

}  // namespace

extern "C" {

vpt_status vpt_trace_diffuse(vpt_ctx* c, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    if ((s = check_frame(c, f)) != VPT_OK) return s;
    cudaSetDevice(c->dev);
    DiffuseArgs a;
    a.diffuse_max_steps = c->cfg.diffuse_max_steps;
    a.bounce_shadow_max_steps = c->cfg.bounce_shadow_max_steps;
    a.bounces = c->cfg.bounces;
    a.spp = c->cfg.spp;
    a.frame_index = f->frame_index;
    a.seed = f->seed;
    a.lighting = gi_lighting(f);
    if (c->textured) {
        a.textured = 1;
        a.tex = tex_view(c);
    }
    GIOut o{c->gi[GI_SH], c->gi[GI_COCG], c->gi[GI_LUMA], c->gi[GI_AOSKY]};
    pass_begin(c, VPT_PASS_DIFFUSE);
    if ((s = refresh_view(c)) != VPT_OK) return s;
    CK(c, trace_diffuse(world_view(c), cam_view(c->cam), c->gw, c->gh, a, c->fp16, c->view[0],
                        (const uint8_t*)c->view[1], o, c->stats ? c->counters : nullptr, c->stream));
    pass_end(c, VPT_PASS_DIFFUSE);
    c->launches += 1;
    return VPT_OK;
}

vpt_status vpt_trace_frame(vpt_ctx* c, const vpt_camera* cam, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!cam || !f) return fail(c, VPT_ERR_INVALID_ARG, "camera and frame are required");
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    if (c->gd != 1) return fail(c, VPT_ERR_STATE, "the fused trace needs the GI on the G-buffer's grid");
    if (c->textured) return fail(c, VPT_ERR_STATE, "the fused trace samples no block textures");
    cudaSetDevice(c->dev);
    c->cam = *cam;
    c->have_cam = true;
    c->gbt_valid = false;
    const int W = c->cfg.width, H = c->cfg.height;
    FrameTraceArgs a;
    a.w = world_view(c);
    a.cam = cam_view(*cam);
    a.W = W;
    a.H = H;
    a.tiles_x = (W + 7) / 8;
    a.n_items = a.tiles_x * ((H + 3) / 4) * 32;
    a.primary_max_steps = c->cfg.primary_max_steps;
    a.shadow_max_steps = c->cfg.shadow_max_steps;
    for (int k = 0; k < 3; k++) a.sun[k] = f->sun_dir[k];
    a.refill_threshold = c->tuning.refill_threshold;
    a.d.diffuse_max_steps = c->cfg.diffuse_max_steps;
    a.d.bounce_shadow_max_steps = c->cfg.bounce_shadow_max_steps;
    a.d.bounces = c->cfg.bounces;
    a.d.spp = c->cfg.spp;
    a.d.frame_index = f->frame_index;
    a.d.seed = f->seed;
    a.d.lighting = gi_lighting(f);
    a.t = c->gbuf[c->cur][GB_T];
    a.face = (uint8_t*)c->gbuf[c->cur][GB_FACE];
    a.block = (uint8_t*)c->gbuf[c->cur][GB_BLOCK];
    a.hit = (int32_t*)c->gbuf[c->cur][GB_HIT];
    a.steps = (uint16_t*)c->gbuf[c->cur][GB_STEPS];
    a.shadow = c->shadow;
    a.sh = c->gi[GI_SH];
    a.cocg = c->gi[GI_COCG];
    a.luma = c->gi[GI_LUMA];
    a.aosky = c->gi[GI_AOSKY];
    a.queue = c->queue;
    a.stats = c->stats ? c->counters : nullptr;
    pass_begin(c, VPT_PASS_TRACE_FRAME);
    CK(c, cudaMemsetAsync(c->queue, 0, sizeof(int), c->stream));
    CK(c, trace_frame(a, c->fp16, c->tuning.trace_blocks, c->stream));
    pass_end(c, VPT_PASS_TRACE_FRAME);
    c->launches += 1;
    return VPT_OK;
}

vpt_status vpt_ground_truth(vpt_ctx* c, const vpt_frame* f, int32_t x0, int32_t y0, int32_t w, int32_t h,
                            int32_t spp, int32_t chunk, uint32_t seed, double* mean_out, double* m2_out) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!f || !mean_out || !m2_out) return fail(c, VPT_ERR_INVALID_ARG, "frame and output buffers are required");
    const int W = c->cfg.width, H = c->cfg.height;
    if (x0 < 0 || y0 < 0 || w <= 0 || h <= 0 || x0 + w > W || y0 + h > H || spp < 1 || chunk < 1)
        return fail(c, VPT_ERR_INVALID_ARG, "crop must lie inside the image, spp and chunk >= 1");
    if (c->fp16) return fail(c, VPT_ERR_STATE, "the ground truth needs an fp32-storage context");
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    if (!c->have_cam) return fail(c, VPT_ERR_STATE, "trace the primary rays of this frame first");
    cudaSetDevice(c->dev);
    const int nchunks = (spp + chunk - 1) / chunk;
    const size_t npx = (size_t)w * h;
    GroundTruthArgs a;
    a.w = world_view(c);
    a.cam = cam_view(c->cam);
    a.W = W;
    a.H = H;
    a.d.diffuse_max_steps = c->cfg.diffuse_max_steps;
    a.d.bounce_shadow_max_steps = c->cfg.bounce_shadow_max_steps;
    a.d.bounces = c->cfg.bounces;
    a.d.spp = 1;
    a.d.frame_index = f->frame_index;
    a.d.seed = f->seed;
    a.d.lighting = gi_lighting(f);
    if (c->textured) {   // the bounce hits read the block textures, as the diffuse trace's
        a.d.textured = 1;
        a.d.tex = tex_view(c);
    }
    a.t = (const float*)c->gbuf[c->cur][GB_T];
    a.face = (const uint8_t*)c->gbuf[c->cur][GB_FACE];
    a.x0 = x0;
    a.y0 = y0;
    a.cw = w;
    a.ch = h;
    a.spp = spp;
    a.chunk = chunk;
    a.nchunks = nchunks;
    a.seed = seed;
    void *part = nullptr, *mean = nullptr, *m2 = nullptr;
    cudaError_t e = cudaMalloc(&part, npx * nchunks * 15 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&mean, npx * 7 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&m2, npx * 7 * sizeof(double));
    if (e == cudaSuccess) {
        a.part = (double*)part;
        a.mean = (double*)mean;
        a.m2 = (double*)m2;
        e = ground_truth(a, c->stream);
        c->launches += 2;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(mean_out, mean, npx * 7 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m2_out, m2, npx * 7 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(part);
    cudaFree(mean);
    cudaFree(m2);
    if (e != cudaSuccess) {
        return fail(c, e == cudaErrorMemoryAllocation ? VPT_ERR_OOM : VPT_ERR_CUDA, "ground truth: %s",
                    cudaGetErrorString(e));
    }
    return VPT_OK;
}

vpt_status vpt_set_tuning(vpt_ctx* c, const vpt_tuning* t) {
    if (!c || !t) return VPT_ERR_INVALID_ARG;
    if (t->refill_threshold < 1 || t->refill_threshold > 32 || t->trace_blocks < 0 || t->trace_blocks > 65535 ||
        t->fused_trace < 0 || t->fused_trace > 1 || t->fused_prefilter < 0 || t->fused_prefilter > 1 ||
        t->overlap_shadow < 0 || t->overlap_shadow > 1 || t->split_temporal < 0 || t->split_temporal > 1)
        return fail(c, VPT_ERR_INVALID_ARG, "refill_threshold must be 1..32, trace_blocks 0..65535, fused_trace, "
                                            "fused_prefilter, overlap_shadow and split_temporal 0/1");
    c->tuning = *t;
    return VPT_OK;
}

vpt_status vpt_get_tuning(const vpt_ctx* c, vpt_tuning* t) {
    if (!c || !t) return VPT_ERR_INVALID_ARG;
    *t = c->tuning;
    return VPT_OK;
}

}  // extern "C"

namespace {

// The temporal pass's arguments for the previous camera pc
// (ProjectPositionPrevious's u_PrevProjection * u_PrevView, in the shader's
// operation order) and frame f.
TemporalArgs temporal_args(const vpt_camera& pc, const vpt_frame* f) {
    TemporalArgs ta;
    for (int col = 0; col < 4; col++)
        for (int r = 0; r < 4; r++)
            ta.prev_view_proj[col * 4 + r] = ((pc.proj[0 * 4 + r] * pc.view[col * 4 + 0] +
                                               pc.proj[1 * 4 + r] * pc.view[col * 4 + 1]) +
                                              pc.proj[2 * 4 + r] * pc.view[col * 4 + 2]) +
                                             pc.proj[3 * 4 + r] * pc.view[col * 4 + 3];
    ta.be_useful = f->temporal ? 1 : 0;
    return ta;
}

// The denoiser passes of one frame; `atrous` false stops after the SVGF
// variance pass (the learned path reads the temporal output instead).
vpt_status svgf_run(vpt_ctx* c, const vpt_camera* prev_cam, const vpt_frame* f, bool atrous) {
    vpt_status s = check_frame(c, f);
    if (s != VPT_OK) return s;
    cudaSetDevice(c->dev);
    // the passes run on the GI grid (W x H); the previous G-buffer and the
    // a-trous taps sample the G-buffer at its own Wf x Hf
    const int W = c->gw, H = c->gh, Wf = c->cfg.width, Hf = c->cfg.height, cur = c->cur, prv = 1 - c->cur;
    const CamView cv = cam_view(c->cam);
    const vpt_camera& pc = prev_cam ? *prev_cam : (c->have_prev ? c->prev_cam : c->cam);
    if ((s = refresh_view(c)) != VPT_OK) return s;
    const void* t = c->view[0];
    const uint8_t* face = (const uint8_t*)c->view[1];
    const uint8_t* block = (const uint8_t*)c->view[2];
    if (c->cfg.denoiser == VPT_DENOISER_ATROUS) {
        // the non-SVGF path (Core/Pipeline.cpp:2618-2786)
        TemporalArgs ta;
        for (int col = 0; col < 4; col++)
            for (int r = 0; r < 4; r++)
                ta.prev_view_proj[col * 4 + r] = ((pc.proj[0 * 4 + r] * pc.view[col * 4 + 0] +
                                                   pc.proj[1 * 4 + r] * pc.view[col * 4 + 1]) +
                                                  pc.proj[2 * 4 + r] * pc.view[col * 4 + 2]) +
                                                 pc.proj[3 * 4 + r] * pc.view[col * 4 + 3];
        ta.be_useful = f->temporal ? 1 : 0;
        PlainDenoiseIO io;
        io.t = t;
        io.prev_t = c->gbuf[prv][GB_T];
        io.Wf = Wf;
        io.Hf = Hf;
        io.face = face;
        io.block = block;
        io.cur = GIIn{c->gi[GI_SH], c->gi[GI_COCG], c->gi[GI_LUMA], c->gi[GI_AOSKY]};
        io.prev = HistIO{c->hist[prv][HI_SH], c->hist[prv][HI_COCG], c->hist[prv][HI_UTIL], c->hist[prv][HI_AOSKY]};
        io.temporal = HistIO{c->hist[cur][HI_SH], c->hist[cur][HI_COCG], c->hist[cur][HI_UTIL], c->hist[cur][HI_AOSKY]};
        io.variance = c->var[FI_VAR];
        for (int k = 0; k < 2; k++)
            io.out[k] = FiltIO{c->den[k][FI_SH], c->den[k][FI_COCG], c->den[k][FI_VAR], c->den[k][FI_AOSKY]};
        io.iterations = c->cfg.atrous_iterations;
        pass_begin(c, VPT_PASS_ATROUS);
        CK(c, plain_denoise(cv, W, H, c->fp16, ta, io, c->stream));
        pass_end(c, VPT_PASS_ATROUS);
        if (io.iterations > 0) c->den_last = (io.iterations - 1) & 1;
        c->launches += 2 + (uint64_t)io.iterations;
        return VPT_OK;
    }
    // Spatial3x3Initial (Core/Pipeline.cpp:2288-2330) and temporal (:2334-2436)
    const GIIn gin{c->gi[GI_SH], c->gi[GI_COCG], c->gi[GI_LUMA], c->gi[GI_AOSKY]};
    const GIOut pre{c->pre[GI_SH], c->pre[GI_COCG], c->pre[GI_LUMA], c->pre[GI_AOSKY]};
    if (!c->tuning.fused_prefilter) {
        pass_begin(c, VPT_PASS_SPATIAL_INITIAL);
        CK(c, svgf_spatial_initial(cv, W, H, c->fp16, t, face, gin, pre, c->stream));
        pass_end(c, VPT_PASS_SPATIAL_INITIAL);
        c->launches += 1;
    }
    const TemporalArgs ta = temporal_args(pc, f);
    HistIO hout{c->hist[cur][HI_SH], c->hist[cur][HI_COCG], c->hist[cur][HI_UTIL], c->hist[cur][HI_AOSKY]};
    HistIO hprev{c->hist[prv][HI_SH], c->hist[prv][HI_COCG], c->hist[prv][HI_UTIL], c->hist[prv][HI_AOSKY]};
    // the history gather queued by trace_all for this frame, if it used these arguments
    const bool gathered = c->tgather_pending && !c->tuning.fused_prefilter && W == Wf && H == Hf &&
                          std::memcmp(&ta, &c->tgather_args, sizeof ta) == 0;
    c->tgather_pending = false;
    pass_begin(c, VPT_PASS_TEMPORAL);
    if (gathered) {
        CK(c, cudaStreamWaitEvent(c->stream, c->ev_tgather, 0));
        CK(c, svgf_temporal_blend(W, H, c->fp16, ta, c->tsum,
                                  GIIn{c->pre[GI_SH], c->pre[GI_COCG], c->pre[GI_LUMA], c->pre[GI_AOSKY]}, hout,
                                  c->stream));
    } else if (!c->tuning.fused_prefilter)
        CK(c, svgf_temporal(cv, W, H, Wf, Hf, c->fp16, ta, t, face, block, c->gbuf[prv][GB_T],
                            (const uint8_t*)c->gbuf[prv][GB_FACE], (const uint8_t*)c->gbuf[prv][GB_BLOCK],
                            GIIn{c->pre[GI_SH], c->pre[GI_COCG], c->pre[GI_LUMA], c->pre[GI_AOSKY]}, hprev, hout,
                            c->stream));
    else   // the pre-filter fused into the temporal kernel
        CK(c, svgf_pre_temporal(cv, W, H, Wf, Hf, c->fp16, ta, t, face, block, c->gbuf[prv][GB_T],
                                (const uint8_t*)c->gbuf[prv][GB_FACE], (const uint8_t*)c->gbuf[prv][GB_BLOCK], gin,
                                pre, hprev, hout, c->stream));
    pass_end(c, VPT_PASS_TEMPORAL);
    // variance (:2438-2475)
    pass_begin(c, VPT_PASS_VARIANCE);
    CK(c, svgf_variance(cv, W, H, c->fp16, t, face, hout, FiltIO{c->var[FI_SH], c->var[FI_COCG], c->var[FI_VAR], nullptr},
                        c->stream));
    pass_end(c, VPT_PASS_VARIANCE);
    c->launches += 2;
    if (!atrous) return VPT_OK;
    // a-trous iterations with steps 16, 8, 4, 2, 1 (:2481-2610)
    const float tmod = f->time * 100.493850275f;
    pass_begin(c, VPT_PASS_ATROUS);
    for (int it = 0; it < c->cfg.atrous_iterations; it++) {
        AtrousArgs aa;
        aa.step = 16 >> it;
        if (aa.step < 1) aa.step = 1;
        aa.add_scale = mixf(1.0f, 2.4f, c->cfg.resolution_scale);
        aa.phi_bias = fmaxf(c->cfg.color_phi_bias, 0.1f);
        aa.tmod500 = tmod - 500.0f * floorf(tmod / 500.0f);
        FiltIO in;
        const void* in_ao;
        if (it == 0) {
            in = FiltIO{c->var[FI_SH], c->var[FI_COCG], c->var[FI_VAR], nullptr};
            in_ao = c->hist[cur][HI_AOSKY];
        } else {
            int k = (it - 1) & 1;
            in = FiltIO{c->den[k][FI_SH], c->den[k][FI_COCG], c->den[k][FI_VAR], c->den[k][FI_AOSKY]};
            in_ao = c->den[k][FI_AOSKY];
        }
        int k = it & 1;
        FiltIO out{c->den[k][FI_SH], c->den[k][FI_COCG], c->den[k][FI_VAR], c->den[k][FI_AOSKY]};
        CK(c, svgf_atrous(cv, W, H, Wf, Hf, c->fp16, aa, t, face, c->gbuf[cur][GB_T],
                          (const uint8_t*)c->gbuf[cur][GB_FACE], c->hist[cur][HI_UTIL], in, in_ao, out, c->stream));
        c->den_last = k;
        c->launches += 1;
    }
    pass_end(c, VPT_PASS_ATROUS);
    return VPT_OK;
}

// The denoised diffuse GI (DiffuseDenoiseFBO): the last a-trous output, or
// the variance / temporal output without a-trous iterations.
void denoised_gi(vpt_ctx* c, const void** sh, const void** cocg, const void** ao) {
    const bool plain = c->cfg.denoiser == VPT_DENOISER_ATROUS;
    const bool den = c->cfg.atrous_iterations > 0;
    *sh = den ? c->den[c->den_last][FI_SH] : (plain ? c->hist[c->cur][HI_SH] : c->var[FI_SH]);
    *cocg = den ? c->den[c->den_last][FI_COCG] : (plain ? c->hist[c->cur][HI_COCG] : c->var[FI_COCG]);
    *ao = den ? c->den[c->den_last][FI_AOSKY] : c->hist[c->cur][HI_AOSKY];
}

// The reflection pass of this frame (ReflectionTraceFrag.glsl, then the
// firefly rejection of SpecularTemporalFilter.glsl); runs after the diffuse
// denoiser, whose output it reads (Core/Pipeline.cpp:2998-3130).
vpt_status reflection_run(vpt_ctx* c, const vpt_frame* f) {
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    if ((s = join_shadow(c)) != VPT_OK) return fail(c, s, "joining the shadow pass failed");
    if ((s = check_frame(c, f)) != VPT_OK) return s;
    if (c->cfg.reflection_spp <= 0) return fail(c, VPT_ERR_STATE, "reflections are off (reflection_spp = 0)");
    cudaSetDevice(c->dev);
    if ((s = refresh_view(c)) != VPT_OK) return s;
    ReflectionArgs a;
    a.spp = c->cfg.reflection_spp;
    a.max_steps = c->cfg.reflection_max_steps;
    a.shadow_max_steps = c->cfg.reflection_shadow_max_steps;
    a.frame_index = f->frame_index;
    a.seed = f->seed;
    const vpt_camera& cm = c->cam;
    for (int col = 0; col < 4; col++)
        for (int r = 0; r < 4; r++)
            a.view_proj[col * 4 + r] = ((cm.proj[0 * 4 + r] * cm.view[col * 4 + 0] + cm.proj[1 * 4 + r] * cm.view[col * 4 + 1]) +
                                        cm.proj[2 * 4 + r] * cm.view[col * 4 + 2]) +
                                       cm.proj[3 * 4 + r] * cm.view[col * 4 + 3];
    const GILighting L = gi_lighting(f);
    const v3 mixed = vmix(mk3(f->sun_radiance[0], f->sun_radiance[1], f->sun_radiance[2]),
                          mk3(f->moon_radiance[0], f->moon_radiance[1], f->moon_radiance[2]), 1.0f - L.sun_visibility);
    for (int k = 0; k < 3; k++) {
        a.light_dir[k] = L.light_dir[k];
        a.viewer[k] = cm.position[k];
    }
    a.mixed[0] = mixed.x;
    a.mixed[1] = mixed.y;
    a.mixed[2] = mixed.z;
    // with block textures the passes read the textured G-buffer of this frame
    const bool tex = c->textured;
    if (tex) {
        if (!c->gbt_valid)
            return fail(c, VPT_ERR_STATE, "block textures are set: run vpt_generate_gbuffer after the primary trace");
        a.gb_normal = c->gbt[1];
        a.gb_pbr = c->gbt[2];
        a.textured = 1;
        a.tex = tex_view(c);
    }
    const void *sh, *cocg, *ao;
    denoised_gi(c, &sh, &cocg, &ao);
    const int cur = c->cur, prv = 1 - c->cur;
    const vpt_camera& pc = c->have_prev ? c->prev_cam : c->cam;
    SpecTemporalArgs ta;
    for (int col = 0; col < 4; col++)
        for (int r = 0; r < 4; r++)
            ta.prev_view_proj[col * 4 + r] = ((pc.proj[0 * 4 + r] * pc.view[col * 4 + 0] +
                                               pc.proj[1 * 4 + r] * pc.view[col * 4 + 1]) +
                                              pc.proj[2 * 4 + r] * pc.view[col * 4 + 2]) +
                                             pc.proj[3 * 4 + r] * pc.view[col * 4 + 3];
    for (int k = 0; k < 3; k++) {
        ta.cur_pos[k] = cm.position[k];
        ta.prev_pos[k] = pc.position[k];
    }
    ta.temporal = c->cfg.reflection_temporal ? 1 : 0;
    if (tex) ta.gb_pbr = c->gbt[2];
    pass_begin(c, VPT_PASS_REFLECTION);
    CK(c, trace_reflection(world_view(c), cam_view(cm), c->cfg.width, c->cfg.height, c->gw, c->gh, c->fp16, a,
                           c->gbuf[cur][GB_T], (const uint8_t*)c->gbuf[cur][GB_FACE], c->shadow, c->view[0],
                           (const uint8_t*)c->view[1], (const uint8_t*)c->view[2], sh, cocg, ao, c->rspec, c->rhit[cur],
                           c->rmask, c->stats ? c->counters : nullptr, c->stream));
    // the two bilateral passes over the hit distance (Core/Pipeline.cpp:3141-3215)
    CK(c, spec_hit_blur(c->gw, c->gh, c->fp16, 1, c->view[0], (const uint8_t*)c->view[1], c->rhit[cur], c->rhit_tmp,
                        c->stream));
    CK(c, spec_hit_blur(c->gw, c->gh, c->fp16, 2, c->view[0], (const uint8_t*)c->view[1], c->rhit_tmp, c->rhit[cur],
                        c->stream));
    // SpecularTemporalFilter (:3217-3262)
    CK(c, spec_temporal(world_view(c), cam_view(cm), ta, c->cfg.width, c->cfg.height, c->gw, c->gh, c->fp16,
                        c->view[0], (const uint8_t*)c->view[1], (const uint8_t*)c->view[2], c->gbuf[prv][GB_T],
                        (const uint8_t*)c->gbuf[prv][GB_FACE], c->rspec, c->rhit[cur], c->rmask, c->rout[prv],
                        c->rhit[prv], c->rstable[prv], c->rout[cur], c->racc, c->rstable[cur], c->stream));
    c->launches += 4;
    if (c->cfg.reflection_denoise) {
        // ReflectionDenoiserNew, x then y (:3312-3440); the hit distance is the
        // stabilised one with the temporal filter on, else the blurred trace's
        SpecDenoiseArgs da;
        if (tex) {
            da.gb_normal = c->gbt[1];
            da.gb_pbr = c->gbt[2];
        }
        memcpy(da.view, cm.view, sizeof da.view);
        da.res_scale = 1.0f / (float)c->gd;
        da.temporal_weight = ta.temporal;
        const void* hd = ta.temporal ? c->rstable[cur] : c->rhit[cur];
        const uint8_t* gface = (const uint8_t*)c->gbuf[cur][GB_FACE];
        const uint8_t* gblock = (const uint8_t*)c->gbuf[cur][GB_BLOCK];
        for (int pass = 0; pass < 2; pass++) {
            da.dir = pass == 0 ? 1 : 0;
            CK(c, spec_denoise(world_view(c), cam_view(cm), da, c->cfg.width, c->cfg.height, c->gw, c->gh, c->fp16,
                               c->gbuf[cur][GB_T], gface, gblock, c->view[0], (const uint8_t*)c->view[1],
                               (const uint8_t*)c->view[2], pass == 0 ? c->rout[cur] : c->rden1, hd, c->racc,
                               pass == 0 ? c->rden1 : c->rden, c->stream));
        }
        c->launches += 2;
    }
    pass_end(c, VPT_PASS_REFLECTION);
    return VPT_OK;
}

// The colour pass. source 0: the denoised GI (last a-trous output, or the
// variance / temporal output without a-trous iterations); 1: the temporally
// accumulated GI before any spatial filter; 2: the raw GI of this frame.
// Writes `out` (the COLOR plane when NULL).
vpt_status shade_run(vpt_ctx* c, const vpt_frame* f, int source, void* out = nullptr) {
    vpt_status s = check_world(c);
    if (s != VPT_OK) return s;
    if ((s = join_shadow(c)) != VPT_OK) return fail(c, s, "joining the shadow pass failed");
    if ((s = check_frame(c, f)) != VPT_OK) return s;
    cudaSetDevice(c->dev);
    ShadeArgs a;
    v3 sun = mk3(f->sun_dir[0], f->sun_dir[1], f->sun_dir[2]);
    v3 moon = normalize(mk3(-sun.x, -sun.y, sun.z));
    a.sun[0] = sun.x; a.sun[1] = sun.y; a.sun[2] = sun.z;
    a.moon[0] = moon.x; a.moon[1] = moon.y; a.moon[2] = moon.z;
    for (int k = 0; k < 3; k++) {
        a.sun_color[k] = f->sun_radiance[k];
        a.moon_color[k] = f->moon_radiance[k];
    }
    float sv = clampf(dot(sun, mk3(0.0f, 1.0f, 0.0f)) + 0.05f, 0.0f, 0.1f) * 12.0f;
    a.sun_vis = 1.0f - sv;
    const bool plain = c->cfg.denoiser == VPT_DENOISER_ATROUS;
    a.vxao = plain ? 0 : 1;
    a.gi_div = c->gd;
    const void *sh, *cocg, *ao;
    denoised_gi(c, &sh, &cocg, &ao);
    // the specular indirect of this frame's reflection pass (the learned
    // path's inputs, sources 1 and 2, are shaded without it)
    const void* spec = (c->cfg.reflection_spp > 0 && source == 0)
                           ? (c->cfg.reflection_denoise ? c->rden : c->rout[c->cur])
                           : nullptr;
    if (source == 1) {
        sh = c->hist[c->cur][HI_SH];
        cocg = c->hist[c->cur][HI_COCG];
        ao = c->hist[c->cur][HI_AOSKY];
    } else if (source == 2) {
        sh = c->gi[GI_SH];
        cocg = c->gi[GI_COCG];
        ao = c->gi[GI_AOSKY];
    }
    // the plain frame with block textures reads the textured G-buffer; the
    // learned path's inputs (sources 1 and 2) keep the block table's flat
    // materials its network was trained on
    if (c->textured && source == 0) {
        if (!c->gbt_valid)
            return fail(c, VPT_ERR_STATE, "block textures are set: run vpt_generate_gbuffer after the primary trace");
        a.gb_albedo = c->gbt[0];
        a.gb_normal = c->gbt[1];
        a.gb_pbr = c->gbt[2];
        a.gb_ao = c->gbt[3];
    }
    // an asynchronous readback of the colour plane must finish before it is rewritten
    if (!out && c->copy_pending) CK(c, cudaStreamWaitEvent(c->stream, c->ev_copy, 0));
    pass_begin(c, VPT_PASS_SHADE);
    CK(c, shade(world_view(c), cam_view(c->cam), c->cfg.width, c->cfg.height, c->fp16, a, c->gbuf[c->cur][GB_T],
                (const uint8_t*)c->gbuf[c->cur][GB_FACE], (const uint8_t*)c->gbuf[c->cur][GB_BLOCK], c->shadow, sh, cocg,
                ao, spec, out ? out : c->color, c->stream));
    pass_end(c, VPT_PASS_SHADE);
    c->launches += 1;
    return VPT_OK;
}

vpt_status trace_all(vpt_ctx* c, const vpt_camera* cam, const vpt_frame* f) {
    vpt_status s;
    if (c->tuning.fused_trace && c->gd == 1 && !c->textured) return vpt_trace_frame(c, cam, f);
    if ((s = vpt_trace_primary(c, cam)) != VPT_OK) return s;
    if (c->tuning.overlap_shadow) {
        // the shadow pass reads only this frame's G-buffer and writes only the
        // shadow plane, which nothing reads before the reflection and colour
        // passes: it runs on the side stream beside the diffuse trace and SVGF
        // each handle created once (a call after a failed creation retries the missing ones)
        if (!c->side_stream) CK(c, cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking));
        if (!c->ev_fork) CK(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
        if (!c->ev_join) CK(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
        if ((s = join_shadow(c)) != VPT_OK) return fail(c, s, "joining the previous shadow pass failed");
        CK(c, cudaEventRecord(c->ev_fork, c->stream));
        CK(c, cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0));
        c->tgather_pending = false;
        if (c->tuning.split_temporal && c->cfg.denoiser == VPT_DENOISER_SVGF && !c->tuning.fused_prefilter &&
            c->gd == 1 && !c->textured) {
            // the temporal pass's history gather reads only this frame's
            // G-buffer and the previous frame's planes: it runs here, ahead
            // of the shadow pass, and svgf_run blends its sums (the previous
            // camera as the frame calls pass it to svgf_run)
            if (!c->tsum && (s = dalloc(c, &c->tsum, c->npx * 64)) != VPT_OK) return s;
            if (!c->ev_tgather) CK(c, cudaEventCreateWithFlags(&c->ev_tgather, cudaEventDisableTiming));
            const vpt_camera prev = c->have_prev ? c->prev_cam : *cam;
            const TemporalArgs ta = temporal_args(prev, f);
            const int cur = c->cur, prv = 1 - c->cur;
            CK(c, svgf_temporal_gather(cam_view(c->cam), c->cfg.width, c->cfg.height, c->fp16, ta,
                                       c->gbuf[cur][GB_T], (const uint8_t*)c->gbuf[cur][GB_FACE],
                                       (const uint8_t*)c->gbuf[cur][GB_BLOCK], c->gbuf[prv][GB_T],
                                       (const uint8_t*)c->gbuf[prv][GB_FACE], (const uint8_t*)c->gbuf[prv][GB_BLOCK],
                                       HistIO{c->hist[prv][HI_SH], c->hist[prv][HI_COCG], c->hist[prv][HI_UTIL],
                                              c->hist[prv][HI_AOSKY]},
                                       c->tsum, c->side_stream));
            CK(c, cudaEventRecord(c->ev_tgather, c->side_stream));
            c->launches += 1;
            c->tgather_args = ta;
            c->tgather_pending = true;
        }
        if ((s = shadow_run(c, f, c->side_stream)) != VPT_OK) return s;
        CK(c, cudaEventRecord(c->ev_join, c->side_stream));   // after both: joining it joins the gather too
        c->shadow_forked = true;
    } else if ((s = vpt_trace_shadow(c, f)) != VPT_OK) {
        return s;
    }
    return vpt_trace_diffuse(c, f);
}

vpt_status read_color(vpt_ctx* c, float* rgb_out) {
    const size_t n = c->npx * 3;
    if (c->fp16) {
        std::vector<__half> tmp(n);
        CK(c, cudaMemcpyAsync(tmp.data(), c->color, n * 2, cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        for (size_t k = 0; k < n; k++) rgb_out[k] = __half2float(tmp[k]);
    } else {
        CK(c, cudaMemcpyAsync(rgb_out, c->color, n * 4, cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
    }
    return VPT_OK;
}

}  // namespace

extern "C" {

vpt_status vpt_svgf(vpt_ctx* c, const vpt_camera* prev_cam, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    return svgf_run(c, prev_cam, f, true);
}

vpt_status vpt_trace_reflections(vpt_ctx* c, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    return reflection_run(c, f);
}

vpt_status vpt_shade(vpt_ctx* c, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    return shade_run(c, f, 0);
}

vpt_status vpt_shade_from(vpt_ctx* c, const vpt_frame* f, int32_t source) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (source < 0 || source > 2) return fail(c, VPT_ERR_INVALID_ARG, "shade source must be 0, 1 or 2");
    return shade_run(c, f, source);
}

vpt_status vpt_learned_input(vpt_ctx* c, const vpt_camera* cam, const vpt_frame* f) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!cam || !f) return fail(c, VPT_ERR_INVALID_ARG, "camera and frame are required");
    if (c->cfg.denoiser != VPT_DENOISER_SVGF) return fail(c, VPT_ERR_STATE, "the learned path needs the SVGF denoiser");
    if (c->gd != 1) return fail(c, VPT_ERR_STATE, "the learned path needs the GI on the G-buffer's grid");
    const vpt_camera prev = c->have_prev ? c->prev_cam : *cam;
    vpt_status s;
    if ((s = trace_all(c, cam, f)) != VPT_OK) return s;
    if ((s = svgf_run(c, &prev, f, false)) != VPT_OK) return s;
    if (!c->color_raw && (s = dalloc(c, &c->color_raw, c->npx * 3 * (c->fp16 ? 2 : 4))) != VPT_OK) return s;
    if ((s = shade_run(c, f, 2, c->color_raw)) != VPT_OK) return s;
    return shade_run(c, f, 1);
}

vpt_status vpt_learned_features(vpt_ctx* c, int32_t x0, int32_t y0, int32_t w, int32_t h, void* dst) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!dst || w < 1 || h < 1 || w > 16384 || h > 16384) return fail(c, VPT_ERR_INVALID_ARG, "bad crop or NULL dst");
    if (!c->blocks) return fail(c, VPT_ERR_STATE, "no block table set");
    cudaSetDevice(c->dev);
    if (!c->color_raw) return fail(c, VPT_ERR_STATE, "call vpt_learned_input first");
    CK(c, learned_features(c->cfg.width, c->cfg.height, x0, y0, w, h, c->fp16, c->color, c->color_raw,
                           c->gbuf[c->cur][GB_T],
                           (const uint8_t*)c->gbuf[c->cur][GB_FACE], (const uint8_t*)c->gbuf[c->cur][GB_BLOCK],
                           c->blocks, c->n_blocks, c->var[FI_VAR], dst, c->stream));
    c->launches += 1;
    return VPT_OK;
}

vpt_status vpt_render_frame_learned(vpt_ctx* c, vpt_unet* net, const vpt_camera* cam, const vpt_frame* f,
                                    float* rgb_out, int32_t* used_net) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!cam || !f) return fail(c, VPT_ERR_INVALID_ARG, "camera and frame are required");
    if (used_net) *used_net = 0;
    const int W = c->cfg.width, H = c->cfg.height;
    const bool fits = net && c->cfg.denoiser == VPT_DENOISER_SVGF && c->gd == 1 && (W % 4) == 0 && (H % 4) == 0;
    vpt_status s;
    if (!fits) {
        // SVGF fallback: the plain frame
        const vpt_camera prev = c->have_prev ? c->prev_cam : *cam;
        if ((s = trace_all(c, cam, f)) != VPT_OK) return s;
        if ((s = svgf_run(c, &prev, f, true)) != VPT_OK) return s;
        if (c->cfg.reflection_spp > 0 && (s = reflection_run(c, f)) != VPT_OK) return s;
        if ((s = shade_run(c, f, 0)) != VPT_OK) return s;
    } else {
        if ((s = vpt_learned_input(c, cam, f)) != VPT_OK) return s;
        cudaSetDevice(c->dev);
        if (!c->feat) {
            if ((s = dalloc(c, &c->feat, c->npx * 16 * 2)) != VPT_OK) return s;
            for (int k = 0; k < 2; k++)
                if (!c->ev_net[k]) CK(c, cudaEventCreateWithFlags(&c->ev_net[k], cudaEventDisableTiming));
        }
        void* ns = nullptr;
        if ((s = vpt_unet_get_stream(net, &ns)) != VPT_OK) return fail(c, s, "learned denoiser: bad network");
        pass_begin(c, VPT_PASS_LEARNED);
        CK(c, learned_features(W, H, 0, 0, W, H, c->fp16, c->color, c->color_raw, c->gbuf[c->cur][GB_T],
                               (const uint8_t*)c->gbuf[c->cur][GB_FACE], (const uint8_t*)c->gbuf[c->cur][GB_BLOCK],
                               c->blocks, c->n_blocks, c->var[FI_VAR], c->feat, c->stream));
        CK(c, cudaEventRecord(c->ev_net[0], c->stream));
        CK(c, cudaStreamWaitEvent((cudaStream_t)ns, c->ev_net[0], 0));
        s = vpt_unet_forward(net, c->feat, 1, H, W, nullptr);
        if (s != VPT_OK) return fail(c, s, "learned denoiser: %s", vpt_unet_last_error(net));
        const float* out = nullptr;
        vpt_unet_output(net, &out);
        CK(c, cudaEventRecord(c->ev_net[1], (cudaStream_t)ns));
        CK(c, cudaStreamWaitEvent(c->stream, c->ev_net[1], 0));
        if (c->copy_pending) CK(c, cudaStreamWaitEvent(c->stream, c->ev_copy, 0));
        CK(c, learned_unpack(W, H, c->fp16, out, c->color, c->stream));
        pass_end(c, VPT_PASS_LEARNED);
        c->launches += 2;
        if (used_net) *used_net = 1;
    }
    if (rgb_out && (s = read_color(c, rgb_out)) != VPT_OK) return s;
    return vpt_end_frame(c);
}

vpt_status vpt_end_frame(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (join_shadow(c) != VPT_OK) return fail(c, VPT_ERR_CUDA, "joining the shadow pass failed");
    if (c->have_cam) {
        c->prev_cam = c->cam;
        c->have_prev = true;
    }
    c->cur = 1 - c->cur;
    c->have_cam = false;
    return VPT_OK;
}

vpt_status vpt_reset_history(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    return clear_history(c);
}

vpt_status vpt_render_frame(vpt_ctx* c, const vpt_camera* cam, const vpt_frame* f, float* rgb_out) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!cam || !f) return fail(c, VPT_ERR_INVALID_ARG, "camera and frame are required");
    vpt_status s;
    const vpt_camera prev = c->have_prev ? c->prev_cam : *cam;
    if ((s = trace_all(c, cam, f)) != VPT_OK) return s;
    if (c->textured && (s = vpt_generate_gbuffer(c)) != VPT_OK) return s;
    if ((s = vpt_svgf(c, &prev, f)) != VPT_OK) return s;
    if (c->cfg.reflection_spp > 0 && (s = reflection_run(c, f)) != VPT_OK) return s;
    if ((s = vpt_shade(c, f)) != VPT_OK) return s;
    if (rgb_out && (s = read_color(c, rgb_out)) != VPT_OK) return s;
    return vpt_end_frame(c);
}

namespace {
__global__ void k_half_to_float(const __half* in, float* out, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        out[k] = __half2float(in[k]);
}
}  // namespace

vpt_status vpt_render_frame_async(vpt_ctx* c, const vpt_camera* cam, const vpt_frame* f, float* rgb_out) {
    if (!c) return VPT_ERR_INVALID_ARG;
    if (!cam || !f || !rgb_out) return fail(c, VPT_ERR_INVALID_ARG, "camera, frame and rgb_out are required");
    cudaSetDevice(c->dev);
    if (!c->copy_stream) CK(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    if (!c->ev_color) CK(c, cudaEventCreateWithFlags(&c->ev_color, cudaEventDisableTiming));
    if (!c->ev_copy) CK(c, cudaEventCreateWithFlags(&c->ev_copy, cudaEventDisableTiming));
    vpt_status s;
    const vpt_camera prev = c->have_prev ? c->prev_cam : *cam;
    if ((s = trace_all(c, cam, f)) != VPT_OK) return s;
    if (c->textured && (s = vpt_generate_gbuffer(c)) != VPT_OK) return s;
    if ((s = vpt_svgf(c, &prev, f)) != VPT_OK) return s;
    if (c->cfg.reflection_spp > 0 && (s = reflection_run(c, f)) != VPT_OK) return s;
    if ((s = vpt_shade(c, f)) != VPT_OK) return s;   // waits for the previous readback on the device
    // this frame is queued: the previous image is complete once its copy is
    if (c->copy_pending) CK(c, cudaEventSynchronize(c->ev_copy));
    const size_t n = c->npx * 3;
    const void* src = c->color;
    if (c->fp16) {
        if (!c->color_stage && (s = dalloc(c, &c->color_stage, n * 4)) != VPT_OK) return s;
        const long long blocks = ((long long)n + 255) / 256;
        k_half_to_float<<<(unsigned)(blocks < 65535 ? blocks : 65535), 256, 0, c->stream>>>((const __half*)c->color,
                                                                                       (float*)c->color_stage,
                                                                                       (long long)n);
        CK(c, cudaGetLastError());
        c->launches += 1;
        src = c->color_stage;
    }
    CK(c, cudaEventRecord(c->ev_color, c->stream));
    CK(c, cudaStreamWaitEvent(c->copy_stream, c->ev_color, 0));
    CK(c, cudaMemcpyAsync(rgb_out, src, n * 4, cudaMemcpyDeviceToHost, c->copy_stream));
    CK(c, cudaEventRecord(c->ev_copy, c->copy_stream));
    c->copy_pending = true;
    return vpt_end_frame(c);
}

vpt_status vpt_readback_wait(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    if (c->copy_pending) CK(c, cudaEventSynchronize(c->ev_copy));
    c->copy_pending = false;
    return VPT_OK;
}

vpt_status vpt_plane_info(const vpt_ctx* c, int32_t plane, size_t* bytes, int32_t* channels, int32_t* dtype) {
    if (!c || plane < 0 || plane >= VPT_PLANE_COUNT) return VPT_ERR_INVALID_ARG;
    int ch = 0, dt = 0;
    size_t b = plane_bytes(c, plane, &ch, &dt);
    if (bytes) *bytes = b;
    if (channels) *channels = ch;
    if (dtype) *dtype = dt;
    return VPT_OK;
}

vpt_status vpt_plane_dims(const vpt_ctx* c, int32_t plane, int32_t* width, int32_t* height) {
    if (!c || plane < 0 || plane >= VPT_PLANE_COUNT) return VPT_ERR_INVALID_ARG;
    const bool gi = plane_meta(plane).gi != 0;
    if (width) *width = gi ? c->gw : c->cfg.width;
    if (height) *height = gi ? c->gh : c->cfg.height;
    return VPT_OK;
}

vpt_status vpt_read_plane(vpt_ctx* c, int32_t plane, void* host, size_t bytes) {
    if (!c || !host || plane < 0 || plane >= VPT_PLANE_COUNT) return VPT_ERR_INVALID_ARG;
    size_t need = plane_bytes(c, plane, nullptr, nullptr);
    if (bytes < need) return fail(c, VPT_ERR_INVALID_ARG, "buffer too small: %zu < %zu", bytes, need);
    if (!plane_ptr(c, plane)) return fail(c, VPT_ERR_STATE, "plane %d is not allocated (reflections or block textures off)", plane);
    cudaSetDevice(c->dev);
    CK(c, cudaMemcpyAsync(host, plane_ptr(c, plane), need, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return VPT_OK;
}

vpt_status vpt_write_plane(vpt_ctx* c, int32_t plane, const void* host, size_t bytes) {
    if (!c || !host || plane < 0 || plane >= VPT_PLANE_COUNT) return VPT_ERR_INVALID_ARG;
    size_t need = plane_bytes(c, plane, nullptr, nullptr);
    if (bytes != need) return fail(c, VPT_ERR_INVALID_ARG, "size mismatch: %zu != %zu", bytes, need);
    if (!plane_ptr(c, plane)) return fail(c, VPT_ERR_STATE, "plane %d is not allocated (reflections or block textures off)", plane);
    cudaSetDevice(c->dev);
    CK(c, cudaMemcpyAsync(plane_ptr(c, plane), host, need, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return VPT_OK;
}

vpt_status vpt_plane_device_ptr(vpt_ctx* c, int32_t plane, void** dptr) {
    if (!c || !dptr || plane < 0 || plane >= VPT_PLANE_COUNT) return VPT_ERR_INVALID_ARG;
    *dptr = plane_ptr(c, plane);
    return VPT_OK;
}

vpt_status vpt_synchronize(vpt_ctx* c) {
    if (!c) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    CK(c, cudaStreamSynchronize(c->stream));
    return VPT_OK;
}

vpt_status vpt_set_stats(vpt_ctx* c, int32_t enabled) {
    if (!c) return VPT_ERR_INVALID_ARG;
    c->stats = enabled != 0;
    return VPT_OK;
}

vpt_status vpt_read_stats(vpt_ctx* c, vpt_stats* out) {
    if (!c || !out) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    Counters h;
    CK(c, cudaMemcpyAsync(&h, c->counters, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaMemsetAsync(c->counters, 0, sizeof(Counters), c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 6; k++) {
        out->rays[k] = h.rays[k];
        out->steps[k] = h.steps[k];
    }
    return VPT_OK;
}

vpt_status vpt_set_profiling(vpt_ctx* c, int32_t enabled) {
    if (!c) return VPT_ERR_INVALID_ARG;
    c->profiling = enabled != 0;
    for (int p = 0; p < VPT_PASS_COUNT; p++) c->ev_used[p] = false;
    return VPT_OK;
}

vpt_status vpt_read_pass_times(vpt_ctx* c, float* ms, int32_t n) {
    if (!c || !ms || n <= 0) return VPT_ERR_INVALID_ARG;
    cudaSetDevice(c->dev);
    CK(c, cudaStreamSynchronize(c->stream));
    for (int p = 0; p < n && p < VPT_PASS_COUNT; p++) {
        ms[p] = 0.0f;
        if (c->ev_used[p]) {
            float v = 0.0f;
            if (cudaEventElapsedTime(&v, c->ev[p][0], c->ev[p][1]) == cudaSuccess) ms[p] = v;
            else cudaGetLastError();
        }
    }
    return VPT_OK;
}

vpt_status vpt_launch_count(const vpt_ctx* c, uint64_t* out) {
    if (!c || !out) return VPT_ERR_INVALID_ARG;
    *out = c->launches;
    return VPT_OK;
}

vpt_status vpt_get_stream(const vpt_ctx* c, void** stream) {
    if (!c || !stream) return VPT_ERR_INVALID_ARG;
    *stream = (void*)c->stream;
    return VPT_OK;
}

// Exposed for the parity tests of the deterministic math (not in vpt.h's
// frame API): evaluates op over n host inputs on the device, or on the host
// when on_device is 0.
vpt_status vpt_detmath(int32_t op, const float* x, const float* y, float* out, int32_t n, int32_t on_device) {
    if (!x || !out || n < 0 || op < 0 || op > 17 || ((op == 3 || op >= 6) && !y)) return VPT_ERR_INVALID_ARG;
    if (!on_device) {
        for (int k = 0; k < n; k++) {
            float a = x[k], r;
            switch (op) {
                case 0: r = dexp(a); break;
                case 1: r = dexp2(a); break;
                case 2: r = dlog2(a); break;
                case 3: r = dpow(a, y[k]); break;
                case 4: r = dsin(a); break;
                case 5: r = dcos(a); break;
                case 6: case 7: r = a * y[k]; break;
                case 8: case 9: r = a + y[k]; break;
                case 10: case 11: case 16: case 17: r = dexp(a); break;
                case 12: r = a + y[k] * a; break;
                case 15: r = a / 5.0f; break;
                default: {
                    const float ax = y[k] - floorf(y[k]), ay = 2.0f * y[k] - floorf(2.0f * y[k]);
                    const float bx = 1.0f - ax, by = 1.0f - ay;
                    const float lo = a * bx + (2.0f * a) * ax, hi = (-a) * bx + y[k] * ax;
                    r = lo * by + hi * ay;
                    break;
                }
            }
            out[k] = r;
        }
        return VPT_OK;
    }
    float *dx = nullptr, *dy = nullptr, *dout = nullptr;
    size_t b = (size_t)(n > 0 ? n : 1) * 4;
    if (cudaMalloc(&dx, b) != cudaSuccess || cudaMalloc(&dy, b) != cudaSuccess || cudaMalloc(&dout, b) != cudaSuccess) {
        cudaFree(dx); cudaFree(dy); cudaFree(dout);
        return VPT_ERR_OOM;
    }
    vpt_status st = VPT_OK;
    if (cudaMemcpy(dx, x, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess) st = VPT_ERR_CUDA;
    if (st == VPT_OK && y && cudaMemcpy(dy, y, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess) st = VPT_ERR_CUDA;
    if (st == VPT_OK && detmath_eval(op, dx, dy, dout, n, 0) != cudaSuccess) st = VPT_ERR_CUDA;
    if (st == VPT_OK && cudaMemcpy(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) st = VPT_ERR_CUDA;
    cudaFree(dx); cudaFree(dy); cudaFree(dout);
    return st;
}

}  // extern "C"
