// Fused, persistent trace of a whole frame: for every pixel the primary ray
// (InitialRayTraceFrag.glsl), the sun-shadow ray (ShadowRayTraceFrag.glsl)
// and the diffuse GI bounces with their shadow rays (DiffuseRayTraceFrag.glsl
// CalculateDiffuse), writing the G-buffer, shadow and GI planes. The results
// are bit-identical to the three separate passes in trace.cu.
//
// Why one kernel: the rays of a pixel have very different lengths (0 to 350
// DDA steps), so a thread-per-pixel kernel idles most lanes of a warp. Here
// each lane runs a small state machine (primary -> sun shadow -> bounce ->
// bounce shadow -> ... -> outputs) and the warp is persistent:
//   * all lanes that are tracing take one DDA step per loop iteration;
//   * a lane whose ray ended waits; once `refill_threshold` lanes wait (or no
//     lane is tracing) the warp services them together: each advances its
//     state machine (shading, next ray) and lanes whose pixel is complete take
//     new pixels from a global queue with one warp-aggregated atomicAdd;
//   * pixels are handed out in 8x4 tiles so the rays a warp starts together
//     are coherent.
// The grid is sized to fill every SM once (persistent blocks).
#include <mutex>

#include "dda.cuh"
#include "kernels.cuh"

namespace vpt {

namespace {

constexpr unsigned kFull = 0xffffffffu;
enum Phase : int { PH_DONE = 0, PH_IDLE = 1, PH_PRIMARY = 2, PH_SUN = 3, PH_GI = 4, PH_BSH = 5 };

struct Lane {
    int px;          // pixel index
    int phase;
    int face;        // primary face id
    int block_at;    // voxel at the sun-shadow ray origin
    uint32_t rng;
    v3 pos;          // primary hit position from the stored hit distance
    // current diffuse sample
    int s, b;        // sample and bounce index
    v3 thr, contrib, odir;
    float ao;
    int skyhit;
    // last bounce hit, kept while its shadow ray runs
    v3 ip, rd_in;
    int hnorm;       // (axis << 2) | (sign + 1) of the hit normal
    int hblock;
    float T;
    // sums over samples
    float tsh[4], tcc[2];
    v3 rad;
    float acc_ao, skyhits;
};

template <bool STATS>
struct Tally {
    unsigned rays[4], steps[4];
    __device__ void add(int k, int n) {
        if (STATS) {
            rays[k] += 1u;
            steps[k] += (unsigned)n;
        }
    }
};

__device__ __forceinline__ int encode_normal(v3 n) {
    // the traversal's normal has one non-zero axis (or none): -sign on min_idx
    if (n.x != 0.0f) return (0 << 2) | (n.x < 0.0f ? 0 : 2);
    if (n.y != 0.0f) return (1 << 2) | (n.y < 0.0f ? 0 : 2);
    if (n.z != 0.0f) return (2 << 2) | (n.z < 0.0f ? 0 : 2);
    return (2 << 2) | 1;   // zero vector
}
__device__ __forceinline__ v3 decode_normal(int e) {
    const float v = (float)((e & 3) - 1);
    const int m = e >> 2;
    return mk3(m == 0 ? v : 0.0f, m == 1 ? v : 0.0f, m == 2 ? v : 0.0f);
}

template <typename S>
__device__ __forceinline__ float stored(float v) {
    return v;
}
template <>
__device__ __forceinline__ float stored<__half>(float v) {
    return __half2float(__float2half_rn(v));
}

template <typename S, bool STATS>
struct Engine {
    const FrameTraceArgs& a;
    Lane& ln;
    RayState& ray;
    Tally<STATS>& cnt;

    __device__ v3 light_dir() const {
        return mk3(a.d.lighting.light_dir[0], a.d.lighting.light_dir[1], a.d.lighting.light_dir[2]);
    }
    __device__ int spp() const {
        int n = min(max(a.d.spp, 1), 32);
        return a.d.lighting.moon_stronger ? n * 2 : n;
    }

    // primary ray of queue item q (8x4 tiles, row-major over the image)
    __device__ __forceinline__ void start_pixel(int q) {
        const int tile = q >> 5, within = q & 31;
        const int i = (tile % a.tiles_x) * 8 + (within & 7);
        const int j = (tile / a.tiles_x) * 4 + (within >> 3);
        if (i >= a.W || j >= a.H) return;   // stays idle
        ln.px = j * a.W + i;
        const v3 dir = normalize(ray_dir_at(a.cam, texcoord(i, j, a.W, a.H)));
        ray_start(ray, ray_origin(a.cam), dir, a.primary_max_steps);
        ln.phase = PH_PRIMARY;
    }

    __device__ __forceinline__ void write_sky_gi(v3 dir) {
        float sh[4], cocg[2];
        irradiance_to_sh(muls(sky_radiance(dir), 2.66f), normal_from_id(ln.face, 0.5f), sh, cocg);
        const size_t px = (size_t)ln.px;
        st4((S*)a.sh + 4 * px, sh[0], sh[1], sh[2], sh[3]);
        st2((S*)a.cocg + 2 * px, cocg[0], cocg[1]);
        st((S*)a.luma + px, luminance(mk3(0.0f, 0.0f, 0.0f)));
        st2((S*)a.aosky + 2 * px, 1.0f, 0.0f);
    }

    // DiffuseRayTraceFrag.glsl main (:874-893): start the per-pixel sums
    __device__ __forceinline__ void begin_diffuse() {
        ln.rng = pcg_hash((uint32_t)ln.px + pcg_hash(a.d.frame_index + pcg_hash(a.d.seed)));
        ln.s = 0;
        ln.tsh[0] = ln.tsh[1] = ln.tsh[2] = ln.tsh[3] = 0.0f;
        ln.tcc[0] = ln.tcc[1] = 0.0f;
        ln.rad = mk3(0.0f, 0.0f, 0.0f);
        ln.acc_ao = 0.0f;
        ln.skyhits = 0.0f;
        begin_sample();
    }

    // CalculateDiffuse (:535-556): first ray of a sample. Returns false when
    // there is no bounce to trace (the sample is complete already).
    __device__ __forceinline__ bool sample_ray() {
        const v3 n = normal_from_id(ln.face, 0.5f);
        const v3 ro = add(ln.pos, muls(n, 0.06f));
        const v3 rd = cos_hemisphere(n, &ln.rng);
        ln.ao = 1.0f;
        ln.contrib = mk3(0.0f, 0.0f, 0.0f);
        ln.thr = mk3(1.0f, 1.0f, 1.0f);
        ln.skyhit = 0;
        ln.b = 0;
        ln.odir = mk3(0.0f, 0.0f, 0.0f);
        if (a.d.bounces <= 0) return false;
        ln.odir = rd;
        ray_start(ray, ro, rd, a.d.diffuse_max_steps);
        ln.phase = PH_GI;
        return true;
    }

    __device__ __forceinline__ void begin_sample() {
        if (!sample_ray()) end_sample();
    }

    // the rest of a bounce after its hit (:602-623, :637-659)
    __device__ __forceinline__ void continue_hit(float shadow_at) {
        const GILighting& L = a.d.lighting;
        const v3 ldir = light_dir();
        const v3 lcol = mk3(L.light_color[0], L.light_color[1], L.light_color[2]);
        const Material m = material(a.w, ln.hblock);
        const v3 hn = decode_normal(ln.hnorm);
        const v3 rd = ln.rd_in;
        float emissivity = 0.0f;
        if (m.emissive) emissivity = 1.0f * L.emissivity_multiplier * L.diffuse_light_intensity;
        const v3 emissive_color = muls(m.albedo, emissivity * mixf(1.0f, 1.0f, L.sun_visibility));
        const float hs = diffuse_hammon(hn, neg(rd), ldir, m.rough);
        const v3 sun_brdf = muls(muls(mul(muls(m.albedo, hs), muls(lcol, 3.5f)), 1.0f - shadow_at), kPI);
        const v3 new_dir = cos_hemisphere(hn, &ln.rng);
        const float cos_theta = clampf(dot(hn, new_dir), 0.0f, 1.0f);
        const float pdf = fmaxf(cos_theta / kPI, 0.00001f);
        const float att = diffuse_hammon(hn, neg(rd), new_dir, m.rough);
        ln.contrib = add(ln.contrib, mul(ln.thr, sun_brdf));
        ln.contrib = add(ln.contrib, mul(emissive_color, ln.thr));
        ln.thr = mul(ln.thr, divs(muls(m.albedo, att), pdf));
        if (ln.b == 0) {
            const float dao = 2.0f;
            if (ln.T < dao && ln.T > 0.0f) ln.ao = fmaxf(ln.T / dao, 0.0f);
        }
        ln.b++;
        if (ln.b < a.d.bounces) {
            ray_start(ray, add(ln.ip, muls(hn, 0.06f)), new_dir, a.d.diffuse_max_steps);
            ln.phase = PH_GI;
        } else {
            end_sample();
        }
    }

    // main (:901-935): accumulate a sample, then the next one or the outputs
    __device__ __forceinline__ void end_sample() {
        const int n = spp();
        for (;;) {
            const v3 xc = vclamp(ln.contrib, 0.0f, 8.0f);
            ln.rad = add(ln.rad, xc);
            ln.acc_ao += ln.ao;
            float sh[4], cocg[2];
            irradiance_to_sh(xc, ln.odir, sh, cocg);
            for (int c = 0; c < 4; c++) ln.tsh[c] += sh[c];
            ln.tcc[0] += cocg[0];
            ln.tcc[1] += cocg[1];
            ln.skyhits += ln.skyhit ? 1.0f : 0.0f;
            ln.s++;
            if (ln.s >= n) break;
            if (sample_ray()) return;   // next sample's first ray is tracing
        }
        const float fs = (float)n;
        const float acc_ao = ln.acc_ao / fs;
        float tsh[4];
        for (int c = 0; c < 4; c++) tsh[c] = ln.tsh[c] / fs;
        const float c0 = ln.tcc[0] / fs, c1 = ln.tcc[1] / fs;
        const v3 rad = divs(ln.rad, fs);
        const float sky = ln.skyhits / fs;
        const size_t px = (size_t)ln.px;
        st4((S*)a.sh + 4 * px, clampf(tsh[0], -100.0f, 100.0f), clampf(tsh[1], -100.0f, 100.0f),
            clampf(tsh[2], -100.0f, 100.0f), clampf(tsh[3], -100.0f, 100.0f));
        st2((S*)a.cocg + 2 * px, clampf(c0, -100.0f, 100.0f), clampf(c1, -100.0f, 100.0f));
        st((S*)a.luma + px, clampf(fmaxf(luminance(rad), 0.01f), 0.001f, 64.0f));
        st2((S*)a.aosky + 2 * px, clampf(acc_ao, 0.0f, 1.0f), clampf(sky, 0.0f, 1.0f));
        ln.phase = PH_IDLE;
    }

    // the ray of the current phase has ended
    __device__ __forceinline__ void advance() {
        const TraceResult tr = ray_finish(a.w, ray);
        const size_t px = (size_t)ln.px;
        if (ln.phase == PH_PRIMARY) {
            // InitialRayTraceFrag.glsl main (:445-467)
            cnt.add(kRayPrimary, tr.steps);
            const bool intersect = tr.t > 0.0f && tr.block > 0;
            ln.face = intersect ? normal_id(tr.normal) : kFaceMiss;
            st((S*)a.t + px, tr.t);
            a.face[px] = (uint8_t)ln.face;
            a.block[px] = (uint8_t)(intersect ? tr.block : 0);
            a.hit[px * 3 + 0] = tr.cell[0];
            a.hit[px * 3 + 1] = tr.cell[1];
            a.hit[px * 3 + 2] = tr.cell[2];
            a.steps[px] = (uint16_t)tr.steps;
            const float d = stored<S>(tr.t);   // what the later passes read back
            const v3 dir = ray.d;
            if (d < 0.0f) {
                a.shadow[px] = 0;
                write_sky_gi(dir);
                ln.phase = PH_IDLE;
                return;
            }
            ln.pos = add(ray_origin(a.cam), muls(dir, d));
            // ShadowRayTraceFrag.glsl main (:480-512)
            const v3 L = mk3(a.sun[0], a.sun[1], a.sun[2]);
            const v3 n = normal_from_id(ln.face, 1.0f);
            if (dot(n, L) <= 0.01f) {
                a.shadow[px] = 1;
                begin_diffuse();
                return;
            }
            const v3 o = add(ln.pos, mul(n, mk3(0.06f, 0.06f, 0.06f)));
            ln.block_at = get_voxel(a.w, f2i_floor(o.x), f2i_floor(o.y), f2i_floor(o.z));
            if (d > 0.0f) {
                ray_start(ray, o, L, a.shadow_max_steps);
                ln.phase = PH_SUN;
                return;
            }
            a.shadow[px] = ln.block_at > 0 ? 1 : 0;
            begin_diffuse();
        } else if (ln.phase == PH_SUN) {
            cnt.add(kRayShadow, tr.steps);
            a.shadow[px] = (tr.t > 0.0f || ln.block_at > 0) ? 1 : 0;
            begin_diffuse();
        } else if (ln.phase == PH_GI) {
            cnt.add(kRayDiffuse, tr.steps);
            const float T = tr.t;
            const v3 rd = ray.d;
            const v3 ip = add(ray.init, muls(rd, T));
            if (T > 0.0f && tr.block > 0) {
                const GILighting& L = a.d.lighting;
                const v3 ldir = light_dir();
                ln.T = T;
                ln.ip = ip;
                ln.rd_in = rd;
                ln.hnorm = encode_normal(tr.normal);
                ln.hblock = min(max(tr.block, 0), 127);
                const float ndl = fmaxf(dot(tr.normal, ldir), 0.0f);
                if (L.moon_stronger) {
                    continue_hit(1.0f);
                } else if (ndl < 0.001f) {
                    continue_hit(0.0f);
                } else {
                    // GetShadowAt (:1202-1222)
                    ray_start(ray, add(ip, muls(tr.normal, 0.045f)), ldir, a.d.bounce_shadow_max_steps);
                    ln.phase = PH_BSH;
                }
            } else {
                const GILighting& L = a.d.lighting;
                float x = mixf(1.0f, 1.05f, L.sun_visibility);
                x = clampf(x * 1.0f * L.gi_sky_strength, 0.0f, 5.0f);
                ln.contrib = add(ln.contrib, mul(muls(sky_color_at(rd), x), ln.thr));
                ln.skyhit = 1;
                end_sample();
            }
        } else {   // PH_BSH
            cnt.add(kRayBounceShadow, tr.steps);
            continue_hit(tr.t > 0.0f ? 1.0f : 0.0f);
        }
    }
};

template <typename S, bool STATS>
__global__ void __launch_bounds__(128) k_trace_frame(FrameTraceArgs a) {
    const int lane = threadIdx.x & 31;
    const unsigned lanes_below = (1u << lane) - 1u;
    Lane ln;
    ln.phase = PH_IDLE;
    ln.px = 0;
    RayState ray;
    Tally<STATS> cnt;
    for (int k = 0; k < 4; k++) cnt.rays[k] = cnt.steps[k] = 0u;
    Engine<S, STATS> eng{a, ln, ray, cnt};
    bool fin = true;   // not tracing: idle, done, or a ray that has ended
    for (;;) {
        const unsigned tracing = __ballot_sync(kFull, !fin);
        const unsigned waiting = __ballot_sync(kFull, fin && ln.phase != PH_DONE);
        if (tracing == 0u && waiting == 0u) break;
        if (waiting != 0u && (tracing == 0u || __popc(waiting) >= a.refill_threshold)) {
            if (fin && ln.phase >= PH_PRIMARY) eng.advance();
            const unsigned idle = __ballot_sync(kFull, ln.phase == PH_IDLE);
            if (idle != 0u) {
                const int leader = __ffs(idle) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(a.queue, __popc(idle));
                base = __shfl_sync(kFull, base, leader);
                if (ln.phase == PH_IDLE) {
                    const int q = base + __popc(idle & lanes_below);
                    if (q >= a.n_items) ln.phase = PH_DONE;
                    else eng.start_pixel(q);
                }
            }
            fin = ln.phase < PH_PRIMARY;
        }
        if (!fin) fin = dda_step(a.w, ray);
    }
    if (STATS) {
        for (int k = 0; k < 4; k++) {
            const unsigned r = __reduce_add_sync(kFull, cnt.rays[k]);
            const unsigned s = __reduce_add_sync(kFull, cnt.steps[k]);
            if (lane == 0 && (r | s)) {
                atomicAdd(&a.stats->rays[k], (unsigned long long)r);
                atomicAdd(&a.stats->steps[k], (unsigned long long)s);
            }
        }
    }
}

// Resident-grid size (SMs x resident blocks of 128 threads) of one kernel
// instantiation, looked up once per device: devices of different models get
// their own grid, and concurrent first calls are serialised by the mutex.
constexpr int kMaxGridDevices = 64;

template <typename S, bool STATS>
cudaError_t launch_frame(const FrameTraceArgs& a, int blocks_hint, cudaStream_t s) {
    static int grid[kMaxGridDevices];
    static std::mutex mu;
    int blocks = blocks_hint;
    if (blocks <= 0) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kMaxGridDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(mu);
        if (grid[dev] == 0) {
            int sms = 0, per_sm = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_frame<S, STATS>, 128, 0);
            if (e != cudaSuccess) return e;
            grid[dev] = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        }
        blocks = grid[dev];
    }
    k_trace_frame<S, STATS><<<blocks, 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t trace_frame(const FrameTraceArgs& a, int fp16, int blocks_hint, cudaStream_t s) {
    if (fp16) return a.stats ? launch_frame<__half, true>(a, blocks_hint, s) : launch_frame<__half, false>(a, blocks_hint, s);
    return a.stats ? launch_frame<float, true>(a, blocks_hint, s) : launch_frame<float, false>(a, blocks_hint, s);
}

}  // namespace vpt

// ------------------------------------------------- allocation-free variant --
// For callers that cannot allocate device memory on the frame path: engines
// that hand every byte of GPU memory out from a budget fixed at start-up, or
// frame loops that cannot afford cudaMalloc's implicit device-wide
// synchronisation. They pass all inputs and outputs; the only scratch the
// kernel needs, its work-queue counter, lives in this fixed array instead of a
// cudaMalloc'd buffer. Every process that loads libvpt holds these 256 bytes
// on each GPU it uses until it exits.
static constexpr int kNoAllocScratchInts = 64;   // 256 bytes; [0] is the work-queue counter
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocScratchInts];

namespace {

constexpr int kMaxDevices = 64;
int* g_noalloc_ptr[kMaxDevices];   // device address of g_noalloc_scratch, per device
std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device. Host code may
// not use &g_noalloc_scratch (that is a host-side stand-in), so the address is
// looked up once per device, with that device current, and kept for the life
// of the process: after a cudaDeviceReset of that device the module and its
// array are reloaded elsewhere, so the library must not be called on a
// device that was reset.
vpt_status noalloc_scratch(int** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return VPT_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return VPT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return VPT_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<int*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return VPT_OK;
}

}  // namespace

extern "C" vpt_status vpt_trace_frame_noalloc(const vpt_trace_buffers* b, const vpt_config* cfg, const vpt_camera* cam,
                                              const vpt_frame* f, void* stream) {
    using namespace vpt;
    if (!b || !cfg || !cam || !f) return VPT_ERR_INVALID_ARG;
    if (!b->voxels || !b->df || !b->blocks || !b->t || !b->face || !b->block || !b->hit || !b->steps || !b->shadow ||
        !b->gi_sh || !b->gi_cocg || !b->gi_luma || !b->gi_aosky)
        return VPT_ERR_INVALID_ARG;
    if (b->X <= 0 || b->Y <= 0 || b->Z <= 0 || (size_t)b->X * b->Y * b->Z > ((size_t)1 << 31) || b->n_blocks <= 0 ||
        b->n_blocks > 256)
        return VPT_ERR_INVALID_ARG;
    // the work-queue counter indexes 8x4-pixel tiles * 32 entries in an int
    if (cfg->width <= 0 || cfg->height <= 0 || cfg->width > 16384 || cfg->height > 16384) return VPT_ERR_INVALID_ARG;
    // every plane, the GI ones included, is width x height: the coarser GI
    // grid of gi_divisor > 1 is not traced by the fused kernel
    if (cfg->gi_divisor > 1) return VPT_ERR_INVALID_ARG;
    if ((cfg->storage != VPT_STORAGE_F32 && cfg->storage != VPT_STORAGE_F16) || cfg->spp < 1 || cfg->spp > 32 ||
        cfg->bounces < 0 || cfg->bounces > 8 || cfg->primary_max_steps < 0 || cfg->shadow_max_steps < 0 ||
        cfg->diffuse_max_steps < 0 || cfg->bounce_shadow_max_steps < 0)
        return VPT_ERR_INVALID_ARG;
    int* scratch = nullptr;
    vpt_status st = noalloc_scratch(&scratch);
    if (st != VPT_OK) return st;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    FrameTraceArgs a;
    a.w.vox = b->voxels;
    a.w.df = b->df;
    a.w.X = b->X;
    a.w.Y = b->Y;
    a.w.Z = b->Z;
    a.w.blocks = b->blocks;
    a.w.n_blocks = b->n_blocks;
    for (int k = 0; k < 16; k++) {
        a.cam.inv_view[k] = cam->inv_view[k];
        a.cam.inv_proj[k] = cam->inv_proj[k];
    }
    for (int k = 0; k < 3; k++) a.cam.pos[k] = cam->position[k];
    a.W = cfg->width;
    a.H = cfg->height;
    a.tiles_x = (cfg->width + 7) / 8;
    a.n_items = a.tiles_x * ((cfg->height + 3) / 4) * 32;
    a.primary_max_steps = cfg->primary_max_steps;
    a.shadow_max_steps = cfg->shadow_max_steps;
    for (int k = 0; k < 3; k++) a.sun[k] = f->sun_dir[k];
    a.refill_threshold = 16;
    a.d.diffuse_max_steps = cfg->diffuse_max_steps;
    a.d.bounce_shadow_max_steps = cfg->bounce_shadow_max_steps;
    a.d.bounces = cfg->bounces;
    a.d.spp = cfg->spp;
    a.d.frame_index = f->frame_index;
    a.d.seed = f->seed;
    a.d.lighting = gi_lighting(f);
    a.t = b->t;
    a.face = b->face;
    a.block = b->block;
    a.hit = b->hit;
    a.steps = b->steps;
    a.shadow = b->shadow;
    a.sh = b->gi_sh;
    a.cocg = b->gi_cocg;
    a.luma = b->gi_luma;
    a.aosky = b->gi_aosky;
    a.queue = scratch;
    a.stats = nullptr;
    // the array keeps the previous call's count: the counter must start at zero
    if (cudaMemsetAsync(scratch, 0, sizeof(int), s) != cudaSuccess) {
        cudaGetLastError();
        return VPT_ERR_CUDA;
    }
    return trace_frame(a, cfg->storage == VPT_STORAGE_F16, 0, s) == cudaSuccess ? VPT_OK : VPT_ERR_CUDA;
}
