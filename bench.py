#!/usr/bin/env python3
"""Benchmark of the VoxelPathTracer hot path on one GB300 (or N replicas).

Workload (the full-frame configuration): a 256^3 uint8 world from the seeded
value-noise generator, a 100-block table (5% emissive), 1920x1080 at 1 spp:
primary ray, sun-shadow ray, one cosine-weighted diffuse bounce with its
shadow ray, then SVGF (pre-temporal 3x3, temporal, variance, 5 a-trous
iterations) and the colour pass. One step = one frame; the camera drifts a
little every frame so the temporal pass reprojects real motion.

`value` is DF-DDA rays per second over the whole denoised frame (trace +
SVGF + shade inside the timed region, inputs resident in HBM); `frame_ms` is
the denoised frame time. `e2e` is the same metric through the public C ABI
call vpt_render_frame_async, every frame's image copied to pinned host memory
(double-buffered readback). The L2 is flushed (a 512 MiB write) between timed
steps.

--impl reference times the reference's algorithm on the host cores: the CPU
restatement of the shaders (oracle/; the reference itself is GLSL and cannot
run without an OpenGL context), OpenMP over all host threads, rendering the
same whole frames (traces, SVGF and colour pass) from inputs generated by
oracle.inputs, so that arm never loads libvpt.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "rays/s DF-DDA + denoised 1080p frame ms, batched/learned vs plain at same error"
WORLD = (256, 256, 256)
RES = (1920, 1080)
CAM_POS = (128.0, 90.0, 128.0)
PEAKS_FILE = REPO / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
TRACE_KINDS = {"primary": ["primary"], "shadow": ["shadow"], "diffuse": ["diffuse", "bounce_shadow"],
               "trace_frame": ["primary", "shadow", "diffuse", "bounce_shadow"],
               # the reflection pass's bytes are its rays' (its filters are small beside them)
               "reflection": ["reflection", "reflection_shadow"]}
# Algorithmic bytes per pixel of the filter and colour kernels (planes read +
# planes written once), fp32 / fp16 storage.
FILTER_BYTES_PER_PX = {
    "spatial_initial": (77, 39),   # t, face, SH, CoCg, luma, AO in; SH, CoCg, luma, AO out
    "temporal": (144, 74),         # current G-buffer + pre-filtered planes, previous G-buffer + history;
                                   # history out
    "temporal_fused": (180, 92),   # k_pre_temporal (vpt_tuning.fused_prefilter): the pre-filter's inputs and
                                   # outputs (77 / 39) + the temporal pass's, less the pre-filtered planes and
                                   # the t / face it does not read twice
    "variance": (65, 33),          # t, face, SH, CoCg, util.xy in; SH, CoCg, variance out
    "atrous": (81, 41),            # t, face, util.x, SH, CoCg, variance, AO in; SH, CoCg, variance, AO out
    "shade": (47, 25),             # t, face, block, shadow, SH, CoCg, AO.x in; RGB out
}
KERNEL_NAMES = {"primary": "k_trace_primary", "shadow": "k_trace_shadow", "diffuse": "k_trace_diffuse_staged",
                "trace_frame": "k_trace_frame",
                "spatial_initial": "k_spatial_initial", "temporal": "k_temporal", "variance": "k_variance",
                "atrous": "k_atrous", "shade": "k_shade",
                "reflection": "k_trace_reflection (+ hit blur, temporal and denoiser kernels)"}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    """RANK / WORLD_SIZE / LOCAL_RANK (read here too, so the reference arm needs no import of the package)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, 200 ms period"}


class NvmlClockSampler:
    """SM clock and clock-event reasons read through NVML (read-only queries)
    every millisecond on a background thread, so a timed region of a few tens
    of milliseconds still gets many samples. The GPU is found by its PCI
    address when torch reports it. start() returns False where NVML cannot be
    loaded or the device not found; the caller then takes ClockSampler."""

    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, torch, index: int):
        import ctypes
        self.C = ctypes
        self.index = index
        self.torch = torch
        self.lib = None
        self.handle = None
        self.samples = []
        self.stop_flag = threading.Event()
        self.thread = None

    def start(self) -> bool:
        C = self.C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return False
        except (OSError, AttributeError):
            return False
        try:
            h = C.c_void_p()
            props = self.torch.cuda.get_device_properties(self.index)
            bus = getattr(props, "pci_bus_id", None)
            ok = False
            if bus is not None:
                addr = (f"{getattr(props, 'pci_domain_id', 0):08x}:{bus:02x}:"
                        f"{getattr(props, 'pci_device_id', 0):02x}.0").encode()
                ok = lib.nvmlDeviceGetHandleByPciBusId_v2(C.c_char_p(addr), C.byref(h)) == 0
            if not ok:
                n = C.c_uint()
                if lib.nvmlDeviceGetCount_v2(C.byref(n)) != 0 or n.value != 1:
                    lib.nvmlShutdown()
                    return False   # several GPUs and no PCI address to tell them apart
                ok = lib.nvmlDeviceGetHandleByIndex_v2(0, C.byref(h)) == 0
            if not ok:
                lib.nvmlShutdown()
                return False
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        except (OSError, AttributeError, RuntimeError):
            lib.nvmlShutdown()
            return False
        self.lib, self.handle = lib, h
        mx = C.c_uint()
        self.max_mhz = float(mx.value) if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 else None
        self.thread = threading.Thread(target=self._poll, daemon=True)
        self.thread.start()
        return True

    def _poll(self):
        C = self.C
        mhz, reasons = C.c_uint(), C.c_ulonglong()
        while not self.stop_flag.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.handle, 1, C.byref(mhz)) == 0 and \
                    self.reasons_fn(self.handle, C.byref(reasons)) == 0:
                self.samples.append((float(mhz.value), int(reasons.value)))
            time.sleep(0.001)

    def stop(self):
        self.stop_flag.set()
        if self.thread is not None:
            self.thread.join(timeout=5)
        if self.lib is not None:
            self.lib.nvmlShutdown()
        sm = [m for m, _ in self.samples]
        bits = 0
        for _, r in self.samples:
            bits |= r
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(n for b, n in self.REASONS.items() if bits & b), "samples": len(sm),
                "source": "NVML, 1 ms period, during the timed frames"}


def start_clock_sampler(torch, local):
    """NVML sampler where NVML answers, else the nvidia-smi one."""
    s = NvmlClockSampler(torch, local)
    if s.start():
        return s
    s = ClockSampler(local)
    s.start()
    return s


def peak_hbm():
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def workload_inputs(vpt, seed=0):
    X, Y, Z = WORLD
    vox = vpt.generate_world(X, Y, Z, seed=seed)
    blocks = vpt.generate_block_table(100, seed=seed)
    yaw, pitch = vpt.seeded_pose(seed)
    return vox, blocks, yaw, pitch


def camera_at(gen, yaw, pitch, step):
    """Camera of frame `step`: a slow pan, 0.25 degree of yaw and 0.05 voxel of
    travel per frame. gen is libvpt's package or oracle.inputs (same matrices)."""
    W, H = RES
    pos = (CAM_POS[0] + 0.05 * step, CAM_POS[1], CAM_POS[2])
    return gen.camera_from_pose(pos, yaw + 0.25 * step, pitch, 90.0, W / H)


def frame_at(gen, step):
    return gen.default_frame(frame_index=step, seed=0, time=1.0 + step / 60.0)


def workload_config(args, world):
    """The `config` object of both arms' lines."""
    nb = f"{args.bounces} bounce" + ("s" if args.bounces > 1 else "")
    return {"workload": f"full frame 1920x1080, 256^3 world (seed 0), 1 spp + sun shadow + {nb} "
                        "(+ bounce shadow), SVGF temporal + variance + 5 a-trous, colour pass",
            "world": list(WORLD), "resolution": list(RES), "spp": 1, "bounces": args.bounces,
            "storage": "fp32" if args.storage == 0 else "fp16",
            "gi_divisor": args.gi_divisor, "reflection_spp": args.reflection_spp,
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "flushed (512 MiB write) between timed steps"}


# ------------------------------------------------------------- our arm --
def run_ours(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    import voxelpathtracer_gb300 as vpt

    from voxelpathtracer_gb300.replicas import Replicas
    dist = Replicas(world)
    W, H = RES
    if args.bounces > 1:   # two bounces take the per-texel diffuse kernel
        KERNEL_NAMES["diffuse"] = "k_trace_diffuse"
    vox, blocks, yaw, pitch = workload_inputs(vpt, seed=rank)
    ctx = vpt.Context(width=W, height=H, device=local, storage=args.storage, gi_divisor=args.gi_divisor,
                      reflection_spp=args.reflection_spp, bounces=args.bounces)
    if args.inline_shadow:
        ctx.set_tuning(overlap_shadow=False)
    if args.split_temporal:
        ctx.set_tuning(split_temporal=True)
    ctx.upload_world(vox)
    ctx.set_block_table(blocks)
    ctx.build_df()
    ctx.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    total = args.warmup + args.steps

    # 1) counting pass (untimed): rays and DDA steps per frame of the same sequence
    ctx.set_stats(True)
    rays, steps = [], []
    for s in range(total):
        ctx.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
        st = ctx.read_stats()
        rays.append(st["rays"])
        steps.append(st["steps"])
    ctx.set_stats(False)
    ctx.reset_history()

    # 2) device-resident timed run: frame events only, nothing recorded
    # between the passes inside the timed frames
    times = []
    with torch.cuda.stream(stream):
        for s in range(args.warmup):
            ctx.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
        torch.cuda.synchronize()
        dist.barrier()
        clocks = start_clock_sampler(torch, local)
        launches0 = ctx.launch_count()
        for s in range(args.warmup, total):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        launches = ctx.launch_count() - launches0
        torch.cuda.synchronize()
        dist.barrier()
        clk = clocks.stop()

    # 2b) the same frames again (history restarted) with an event pair
    # around every pass, for the per-pass times and the kernel rooflines;
    # the passes run one after another here (the sun-shadow trace in line),
    # so each pass time is its kernels' own
    ctx.reset_history()
    overlap = ctx.tuning().overlap_shadow
    ctx.set_tuning(overlap_shadow=False)
    ctx.set_profiling(True)
    pass_ms = {p: [] for p in vpt.PASSES}
    with torch.cuda.stream(stream):
        for s in range(args.warmup):
            ctx.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
        for s in range(args.warmup, total):
            flush.zero_()
            ctx.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
            for k, v in ctx.pass_times().items():
                pass_ms[k].append(v)
        torch.cuda.synchronize()
    ctx.set_profiling(False)
    ctx.set_tuning(overlap_shadow=bool(overlap))

    timed = slice(args.warmup, total)
    frame_rays = [sum(r.values()) for r in rays[timed]]
    t_total = dist.max(sum(times) / 1e3)
    rays_total = dist.sum(float(sum(frame_rays)))
    ms_per_step = t_total * 1e3 / args.steps
    value = rays_total / t_total
    trace_ms = sum(sum(pass_ms[p]) for p in ("primary", "shadow", "diffuse", "trace_frame"))
    trace_rays_per_s = sum(frame_rays) / (trace_ms / 1e3)

    # roofline of every kernel; the dominant one has the largest share of the frame
    mean_pass = {k: (sum(v) / len(v) if v else 0.0) for k, v in pass_ms.items()}
    peak, peak_kind = peak_hbm()
    iters = ctx.config.atrous_iterations
    kernels = {}
    mean_pass = {p: ms for p, ms in mean_pass.items() if ms > 0}   # passes this frame path ran
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    l2_gbs = l2_read_roof(vpt, local)
    for p, ms in mean_pass.items():
        launches_per_frame = iters if p == "atrous" else 1
        per_launch_ms = ms / launches_per_frame
        if p in TRACE_KINDS:
            # the DDA is bound by instruction issue on L2-resident gathers, not
            # by HBM: its roof comes from the kernel's ncu summary
            st_ = float(np.mean([sum(st[k] for k in TRACE_KINDS[p]) for st in steps[timed]]))
            ry = float(np.mean([sum(r[k] for k in TRACE_KINDS[p]) for r in rays[timed]]))
            kernels[p] = dict(trace_roofline(KERNEL_NAMES[p], per_launch_ms, st_, ry, sm_count, clk.get("sm_mhz"),
                                             l2_gbs), launches_per_frame=launches_per_frame,
                              ms_per_launch=per_launch_ms)
            continue
        fused_pre = p == "temporal" and "spatial_initial" not in mean_pass
        key = "temporal_fused" if fused_pre else p
        b = float(FILTER_BYTES_PER_PX[key][args.storage] * W * H)
        if p != "shade":   # the GI-side filters run on the GI grid
            b /= float(args.gi_divisor * args.gi_divisor)
        gbs = b / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
        kernels[p] = {"bound": "hbm", "launches_per_frame": launches_per_frame, "ms_per_launch": per_launch_ms,
                      "algorithmic_bytes_per_launch": b, "achieved_gbs": gbs, "frac": gbs / peak}
        ev, prof = issue_roof(KERNEL_NAMES[p], per_launch_ms, sm_count, clk.get("sm_mhz"))
        kernels[p]["issue_frac_captured_launch"] = prof
        if p == "variance":   # the captured launch is a young-history frame, the event time a mean over frames
            kernels[p]["issue_note"] = "captured launch: every texel on the 81-tap branch (young history)"
        else:
            kernels[p]["issue_frac"] = ev
        if fused_pre:
            kernels[p]["kernel"] = "k_pre_temporal"
    dom = max((p for p in mean_pass if p not in TRACE_KINDS), key=mean_pass.get)
    per_launch_bytes = kernels[dom]["algorithmic_bytes_per_launch"]
    achieved = kernels[dom]["achieved_gbs"]
    traffic, traffic_source = args.traffic, "--traffic" if args.traffic is not None else None
    if traffic is None and args.storage == 0 and args.gi_divisor == 1 and args.reflection_spp == 0:
        traffic, traffic_source = profile_traffic(KERNEL_NAMES[dom])

    # 3) end-to-end through the C ABI with host buffers (pinned): every frame's
    # image is copied to host memory by vpt_render_frame_async, double
    # buffered (the copy of frame k runs while frame k + 1 computes); the
    # timed region ends when the last image is in host memory
    ctx.reset_history()
    outs = [torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    for s in range(args.warmup):
        ctx.render_frame_async(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), outs[s % 2])
    ctx.readback_wait()
    dist.barrier()
    t0 = time.perf_counter()
    for s in range(args.warmup, total):
        cam = camera_at(vpt, yaw, pitch, s)
        fr = frame_at(vpt, s)
        ctx.render_frame_async(cam, fr, outs[s % 2])
    ctx.readback_wait()
    e2e_t = dist.max(time.perf_counter() - t0)
    e2e_value = rays_total / e2e_t
    h2d = len(bytes(memoryview(vpt.Camera()))) + len(bytes(memoryview(vpt.Frame())))
    last_rgb = {"fp32": outs[(total - 1) % 2].copy()}

    # 4) variants on the same frames (device-resident timing): FP16 storage, and
    # the reference's default GI grid (DiffuseTraceResolution 1/4: diffuse rays
    # and SVGF on 480x270, joint-bilateral upscale in the colour pass)
    def run_variant(textures=None, **cfg):
        vc = vpt.Context(width=W, height=H, device=local, bounces=args.bounces, **cfg)
        vc.upload_world(vox)
        vc.set_block_table(blocks)
        vc.build_df()
        if textures is not None:
            vc.set_block_textures(textures)
        vc.set_stats(True)
        vrays = 0
        for s in range(total):
            vc.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
            # read (and reset) every frame, so the warm-up frames' rays are not counted
            st = vc.read_stats()
            if s >= args.warmup:
                vrays += sum(st["rays"].values())
        vc.set_stats(False)
        vc.reset_history()
        vs = torch.cuda.ExternalStream(vc.stream(), device=local)
        tv = []
        with torch.cuda.stream(vs):
            for s in range(total):
                if s >= args.warmup:
                    flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(vs)
                vc.render_frame(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), readback=False)
                b.record(vs)
                b.synchronize()
                if s >= args.warmup:
                    tv.append(a.elapsed_time(b))
        # the last frame's image, read after the timed region (the colour
        # plane is not part of the swapped history, so it still holds it)
        rgb = vc.read_plane("COLOR").astype(np.float32)
        vc.close()
        vms = dist.max(sum(tv) / 1e3) * 1e3 / args.steps
        vrays = dist.sum(float(vrays))
        return {"frame_ms": vms, "value": vrays / (vms * args.steps / 1e3), "unit": "rays/s"}, rgb

    variant = None
    if not args.no_variants:
        v16, last_rgb["fp16"] = run_variant(storage=1)
        vq, _ = run_variant(gi_divisor=4)
        vq["gi_grid"] = [W // 4, H // 4]
        # with the reflection pass (ReflectionSPP 2, temporal filter and
        # denoiser on, as the reference runs it), on the full and the 1/4 grid
        vr, _ = run_variant(reflection_spp=2)
        vrq, _ = run_variant(gi_divisor=4, reflection_spp=2)
        vrq["gi_grid"] = [W // 4, H // 4]
        # with block textures (GenerateGBuffer + the colour pass over it):
        # 24 seeded 512 x 512 layers per array, as the reference's block PNGs
        tex = vpt.generate_block_textures(512, 24, seed=0, grass_block=1)
        vt, last_rgb["textured"] = run_variant(textures=tex)
        vt["textures"] = {"size": 512, "layers": 24}
        variant = {"fp16_storage": v16, "gi_quarter": vq, "reflections": vr, "gi_quarter_reflections": vrq,
                   "block_textures": vt}

    # 5) error against the FP64 ground truth of the last frame on the centre crop
    quality_out = None
    if not args.no_quality and rank == 0:
        from voxelpathtracer_gb300 import quality
        crop = quality.DEFAULT_CROP_1080P
        t0 = time.perf_counter()
        gt, se = quality.ground_truth_color(ctx, camera_at(vpt, yaw, pitch, total - 1), frame_at(vpt, total - 1),
                                            crop, spp=args.gt_spp, chunk=256)
        gt_s = time.perf_counter() - t0
        x0, y0, cw, ch = crop
        quality_out = {"crop": list(crop), "gt_spp": args.gt_spp, "gt_accumulation": "fp64 Welford",
                       "gt_seconds": gt_s, "gt_luma_sh_stderr_mean": float(np.mean(se)),
                       "frame": total - 1, "rmse": {}}
        for k, img in last_rgb.items():
            if k == "textured":   # against the ground truth of the textured frame
                with quality.make_gt_context(W, H, vox, blocks, textures=tex) as g:
                    gt_t, _ = quality.ground_truth_color(g, camera_at(vpt, yaw, pitch, total - 1),
                                                         frame_at(vpt, total - 1), crop, spp=args.gt_spp, chunk=256)
                quality_out["rmse"]["textured_svgf"] = quality.rmse(img[y0:y0 + ch, x0:x0 + cw], gt_t)
                continue
            quality_out["rmse"][f"{k}_svgf"] = quality.rmse(img[y0:y0 + ch, x0:x0 + cw], gt)

    if args.error_curve and rank == 0:
        # RMSE against the FP64 ground truth as the history grows, for a static
        # and for the benchmark's panning camera: the SVGF output, its temporal
        # input before any spatial filter and this frame's raw 1-spp GI
        from voxelpathtracer_gb300 import quality
        sample_at = (0, 1, 2, 4, 8, 16, 32)
        frames = [frame_at(vpt, s) for s in range(max(sample_at) + 1)]
        curves = {}
        with quality.make_gt_context(W, H, vox, blocks) as g:
            for name, cams in (("static", [camera_at(vpt, yaw, pitch, 0)] * len(frames)),
                               ("pan", [camera_at(vpt, yaw, pitch, s) for s in range(len(frames))])):
                with vpt.Context(width=W, height=H, device=local) as c2:
                    c2.upload_world(vox)
                    c2.set_block_table(blocks)
                    c2.build_df()
                    curves[name] = quality.error_by_history(c2, g, cams, frames, quality.DEFAULT_CROP_1080P,
                                                            sample_at, spp=args.gt_spp)
        if quality_out is None:
            quality_out = {}
        quality_out["error_by_history"] = {"crop": list(quality.DEFAULT_CROP_1080P), "gt_spp": args.gt_spp,
                                           "rmse_by_frame": curves}

    df_out = df_section(vpt, torch, local, flush, peak) if not args.no_df else None

    batched = None
    if not args.no_batch:
        batched = batched_section(vpt, torch, args, local, flush)
    learned_out = None
    if not args.no_learned:
        try:
            peaks = json.loads(PEAKS_FILE.read_text())
        except Exception:
            peaks = {}
        learned_out = learned_section(vpt, torch, args, local, flush, vox, blocks, yaw, pitch, peaks)
    large = None
    if not args.no_large:
        large = large_section(vpt, torch, args, local)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, vox, blocks, yaw, pitch)
    ctx.close()
    dist.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "rays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "frame_ms": ms_per_step,
        "trace_rays_per_s": trace_rays_per_s,
        "rays_per_frame": float(np.mean(frame_rays)),
        "rays_per_frame_by_kind": {k: float(np.mean([r[k] for r in rays[timed]])) for k in rays[0]},
        "dda_steps_per_frame_by_kind": {k: float(np.mean([s_[k] for s_ in steps[timed]])) for k in steps[0]},
        "pass_ms": {k: round(v, 4) for k, v in mean_pass.items()},
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if args.storage == 0 else "f16-storage/f32",
        "data": "synthetic",
        "config": workload_config(args, world),
        "e2e": {"value": e2e_value, "unit": "rays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": W * H * 3 * 4, "ms_per_step": e2e_t * 1e3 / args.steps,
                "api": "vpt_render_frame_async -> pinned host RGB, double-buffered readback"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dom],
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback", "traffic": traffic, "traffic_source": traffic_source,
                     "algorithmic_bytes_per_launch": per_launch_bytes,
                     "l2_read_roof_gbs": l2_gbs,
                     "kernels": {KERNEL_NAMES[k]: v for k, v in kernels.items()}},
        "clocks": clk,
        "distance_field": df_out,
        "variants": variant,
        "quality": quality_out,
        "batched": batched,
        "learned": learned_out,
        "large": large,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- distance field --
def df_section(vpt, torch, local, flush, peak):
    """The distance-field build (x, y and z sweeps) of the 256^3 and 512^3
    worlds through vpt_df_build_device: median of 10 builds, L2 flushed
    between them. Algorithmic bytes: 1 read + 1 write per voxel per sweep."""
    import ctypes as C
    out = {}
    stream = torch.cuda.Stream(device=local)
    for edge in (256, 512):
        vox = vpt.generate_world(edge, edge, edge, seed=0)
        d_vox = torch.from_numpy(vox.reshape(-1)).to(f"cuda:{local}")
        d_df = torch.empty_like(d_vox)
        ms = []
        with torch.cuda.stream(stream):
            for k in range(13):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                st = vpt.lib.vpt_df_build_device(C.c_void_p(d_vox.data_ptr()), C.c_void_p(d_df.data_ptr()), edge,
                                                 edge, edge, C.c_void_p(stream.cuda_stream))
                e1.record(stream)
                e1.synchronize()
                if st != vpt.OK:
                    raise RuntimeError(f"vpt_df_build_device failed: {st}")
                if k >= 3:
                    ms.append(e0.elapsed_time(e1))
        med = float(statistics.median(ms))
        alg = 3 * 2 * edge ** 3
        gbs = alg / (med * 1e-3) / 1e9
        out[f"{edge}^3"] = {"ms": med, "launches": 3, "algorithmic_bytes": alg, "achieved_gbs": gbs,
                            "frac": gbs / peak}
        del d_vox, d_df
    return out


# ------------------------------------------------------- batched worlds --
BATCH_EDGES = (64, 96, 128, 192, 256)


def batch_worlds(n=64, seed=0):
    """n worlds, each edge uniform in BATCH_EDGES, each ray tile uniform between
    256x256 and 1024x576, cameras above the terrain with seeded yaw/pitch."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        X, Y, Z = (int(e) for e in rng.choice(BATCH_EDGES, 3))
        W, H = int(rng.integers(256, 1025)), int(rng.integers(256, 577))
        out.append({"dims": (X, Y, Z), "tile": (W, H), "seed": 1000 + k})
    return out


def batched_section(vpt, torch, args, local, flush):
    """One persistent launch over 64 uneven worlds (graph replay and direct)
    against the plain path's three pass kernels per world, same rays."""
    specs = batch_worlds(64, seed=0)
    b = vpt.Batch(max_worlds=len(specs), device=local)
    for k, sp in enumerate(specs):
        X, Y, Z = sp["dims"]
        W, H = sp["tile"]
        vox = vpt.generate_world(X, Y, Z, seed=sp["seed"])
        blocks = vpt.generate_block_table(100, seed=sp["seed"])
        yaw, pitch = vpt.seeded_pose(sp["seed"])
        b.add_world(vox, blocks, W, H)
        b.set_camera(k, vpt.camera_from_pose((X / 2, min(Y - 3.0, 90.0), Z / 2), yaw, pitch, 90.0, W / H))
    b.build_df()
    frame = vpt.default_frame(frame_index=1, seed=0)
    b.set_stats(True)
    b.trace(frame, vpt.BATCH_PER_WORLD)
    st = b.read_stats()
    b.set_stats(False)
    rays = sum(st["rays"].values())
    t0 = time.perf_counter()
    recs = b.autotune(frame, reps=3)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.stream(), device=local)
    steps = max(3, min(args.steps, 10))
    out = {}
    with torch.cuda.stream(stream):
        for name, mode in (("graph", vpt.BATCH_GRAPH), ("persistent", vpt.BATCH_PERSISTENT),
                           ("per_world", vpt.BATCH_PER_WORLD)):
            for _ in range(3):
                b.trace(frame, mode)
            torch.cuda.synchronize()
            l0 = b.launch_count()
            ms = []
            for _ in range(steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                b.trace(frame, mode)
                e1.record(stream)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            kernels = (b.launch_count() - l0) / steps
            med = float(statistics.median(ms))
            out[name] = {"ms": med, "rays_per_s": rays / (med * 1e-3), "kernels_per_step": kernels,
                         "host_calls_per_step": 1 if mode == vpt.BATCH_GRAPH else kernels}
    tiles = [sp["tile"] for sp in specs]
    res = {
        "worlds": len(specs),
        "world_edges": BATCH_EDGES,
        "rays_per_step": rays,
        "rays_by_kind": st["rays"],
        "pixels": int(sum(w * h for w, h in tiles)),
        "modes": out,
        "speedup_graph_vs_per_world": out["per_world"]["ms"] / out["graph"]["ms"],
        "autotuned": b.tuning().as_dict(),
        "autotune_candidates": len(recs),
        "autotune_seconds": tune_s,
        "autotune_worst_ms": max(r["ms"] for r in recs),
        "per_world_kernels_per_step": 3 * len(specs),
        "timing": f"median of {steps} steps, L2 flushed between steps",
    }
    b.close()
    return res


# ------------------------------------------------------ learned denoiser --
def unet_flops(vpt, H, W, real=True):
    """Multiply-add FLOPs of one U-Net inference on an H x W image (2 per MAC)."""
    levels = [1, 1, 2, 2, 4, 4, 2, 2, 1, 1, 1]   # resolution divisor of each layer, in layer order
    f = 0
    for (cin, cout, cin_r, cout_r, _off), d in zip(vpt.unet_layers(), levels):
        f += 2 * 9 * (cin_r * cout_r if real else cin * cout) * (H // d) * (W // d)
    return f


def learned_section(vpt, torch, args, local, flush, vox, blocks, yaw, pitch, peaks):
    """The learned denoiser on the full-frame workload: frame ms of the learned
    path, U-Net inference time and tensor throughput, and the error of the
    noisy input, SVGF and the network against the FP64 ground truth."""
    from voxelpathtracer_gb300 import learned
    if not learned.WEIGHTS.exists():
        return {"unavailable": "no trained weights in the package; frames fall back to SVGF"}
    params, meta = learned.load()
    W, H = RES
    out = {"weights": {k: meta[k] for k in ("pairs", "crop", "spp", "steps", "holdout_rmse_noisy",
                                             "holdout_rmse_net") if k in meta}}
    out["weights"]["deviation"] = ("trained on random crops of 1920x1080 frames (the crop size above), not on "
                                   "whole 1080p pairs: the same per-pixel statistics at a fraction of the "
                                   "1024-spp ground-truth cost")
    with vpt.UNet(1, H, W, device=local) as net, vpt.Context(width=W, height=H, device=local) as ctx:
        net.set_params(params)
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
        ms = []
        with torch.cuda.stream(stream):
            for s in range(args.warmup + args.steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                _, used = ctx.render_frame_learned(camera_at(vpt, yaw, pitch, s), frame_at(vpt, s), net,
                                                   readback=False)
                e1.record(stream)
                e1.synchronize()
                if s >= args.warmup:
                    ms.append(e0.elapsed_time(e1))
        out["frame_ms"] = float(statistics.median(ms))
        out["used_net"] = bool(used)
        # inference alone, on the features of the last frame
        feat = torch.empty((1, H, W, 16), dtype=torch.bfloat16, device=f"cuda:{local}")
        ctx.learned_input(camera_at(vpt, yaw, pitch, 0), frame_at(vpt, 0))
        ctx.learned_features((0, 0, W, H), feat[0])
        ctx.synchronize()
        ctx.end_frame()
        ns = torch.cuda.ExternalStream(net.stream(), device=local)
        inf = []
        with torch.cuda.stream(ns):
            for k in range(8):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ns)
                net.forward(feat)
                e1.record(ns)
                e1.synchronize()
                if k >= 3:
                    inf.append(e0.elapsed_time(e1))
        net.synchronize()
        inf_ms = float(statistics.median(inf))
        flops = unet_flops(vpt, H, W)
        peak = float(peaks.get("bf16_tflops", 1900.0))
        out["unet_ms"] = inf_ms
        out["unet_tflop_per_inference"] = flops / 1e12
        out["unet_tflops"] = flops / (inf_ms * 1e-3) / 1e12
        out["tensor_roofline"] = {"bound": "tensor", "achieved": out["unet_tflops"], "peak": peak,
                                  "unit": "TFLOP/s", "frac": out["unet_tflops"] / peak,
                                  "peak_source": "measured (MEASURED_PEAKS.json bf16_tflops)"}
        if not args.no_quality:
            frames = args.warmup + args.steps
            r = learned.evaluate_frame(net, vox, blocks, CAM_POS, yaw, pitch, frames, gt_spp=args.gt_spp,
                                       device=local)
            out["quality"] = dict(r, frames=frames, crop=list(quality_crop()), gt_spp=args.gt_spp)
    return out


def quality_crop():
    from voxelpathtracer_gb300 import quality
    return quality.DEFAULT_CROP_1080P


def profile_metrics(kernel):
    """Rows of the committed ncu summary profiles/<kernel>_1080p.md, as
    {metric: value in base units}; {} when there is none."""
    import re
    path = Path(__file__).resolve().parent / "profiles" / f"{kernel}_1080p.md"
    if not path.exists():
        return {}
    units = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "inst": 1.0, "us": 1e-6, "ms": 1e-3,
             "ns": 1e-9, "": 1.0, "%": 1.0}
    out = {}
    for m in re.finditer(r"^\| ([^|]+?) \| ([0-9.eE+-]+) \| ([^|]*?) \|$", path.read_text(), re.M):
        name, val, unit = m.group(1).strip(), m.group(2), m.group(3).strip()
        if unit in units:
            out.setdefault(name, []).append(float(val) * units[unit])   # one value per captured launch
    return {k: float(np.mean(v)) for k, v in out.items()} | {"_source": f"profiles/{path.name}",
                                                             "_launches": max(map(len, out.values()), default=0)}


def issue_roof(kernel, ms_per_launch, sm_count, sm_mhz):
    """Fraction of the instruction-issue roof (SMs x 4 schedulers x the sampled
    SM clock, one warp instruction per scheduler and cycle) a kernel reaches:
    its warp instructions per launch (committed ncu summary, mean over the
    captured launches) over its event-timed duration, and over the captured
    launches' own duration (which differ when the captured frame is not a
    typical one, as for the variance estimate's young-history frames)."""
    m = profile_metrics(kernel)
    if "instructions (warp)" not in m or not sm_mhz or ms_per_launch <= 0:
        return None, None
    peak = sm_count * 4 * sm_mhz * 1e6
    ev = m["instructions (warp)"] / (ms_per_launch * 1e-3) / peak
    prof = m["instructions (warp)"] / m["duration"] / peak if m.get("duration") else None
    return ev, prof


def l2_read_roof(vpt, local):
    """Achievable L2 read bandwidth: 128-bit reads of a 32 MiB buffer that
    stays in L2 (vpt_measure_l2_read), median of 20 reads (GB/s)."""
    import ctypes as C
    g = C.c_float()
    if vpt.lib.vpt_measure_l2_read(local, 32 * 1024 * 1024, 20, C.byref(g)) != vpt.OK:
        return None
    return float(g.value)


def trace_roofline(kernel, ms_per_launch, steps, rays, sm_count, sm_mhz, l2_gbs):
    """The DDA kernels' roofs from their committed ncu summary: instruction
    issue (warp instructions / event time against SMs x 4 schedulers x the
    sampled SM clock), L2 -> L1 bytes per DDA step and their rate against the
    measured L2 read roof, and SIMD efficiency (threads per instruction / 32)."""
    m = profile_metrics(kernel)
    if "instructions (warp)" not in m or not sm_mhz:
        return {"bound": "issue", "frac": None, "note": "no ncu summary for this kernel"}
    t = ms_per_launch * 1e-3
    issue = m["instructions (warp)"] / t
    issue_peak = sm_count * 4 * sm_mhz * 1e6
    l2l1 = m.get("L2 -> L1 read bytes")
    out = {"bound": "issue", "unit": "warp instructions/s", "achieved": issue, "peak": issue_peak,
           "frac": issue / issue_peak, "warp_instructions_per_launch": m["instructions (warp)"],
           "simd_efficiency": m.get("threads per instruction (of 32)", 0.0) / 32.0,
           "dda_steps_per_launch": steps, "rays_per_launch": rays, "source": m["_source"]}
    if l2l1 is not None:
        out["l2_to_l1_bytes_per_launch"] = l2l1
        out["l2_to_l1_bytes_per_step"] = l2l1 / max(steps, 1.0)
        out["l2_to_l1_gbs"] = l2l1 / t / 1e9
        if l2_gbs:
            out["l2_roof_gbs"] = l2_gbs
            out["l2_frac"] = l2l1 / t / 1e9 / l2_gbs
    return out


def profile_traffic(kernel):
    """DRAM bytes (read + write) of one launch of `kernel` on this workload,
    from its committed ncu summary (profiles/<kernel>_1080p.md); (None, None)
    when there is none."""
    import re
    path = Path(__file__).resolve().parent / "profiles" / f"{kernel}_1080p.md"
    if not path.exists():
        return None, None
    units = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    total = 0.0
    for what in ("DRAM read", "DRAM write"):
        m = re.search(rf"^\| {what} \| ([0-9.]+) \| (\w+) \|$", path.read_text(), re.M)
        if not m or m.group(2) not in units:
            return None, None
        total += float(m.group(1)) * units[m.group(2)]
    return total, f"profiles/{path.name} (ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch)"


# ------------------------------------------------------ large combined --
LARGE_WORLD = (512, 512, 512)
LARGE_RES = (3840, 2160)


def orbit_camera(vpt, k, theta0, W, H, step_deg=1.0):
    """Frame k of the orbit (radius 200, height 150) around the world's centre column."""
    from voxelpathtracer_gb300 import learned
    return learned.orbit_camera(LARGE_WORLD, theta0 + step_deg * k, W / H)


def large_section(vpt, torch, args, local):
    """512^3 world, 3840x2160, 1 spp with 2 diffuse bounces, a seeded 64-frame
    orbit with temporal reprojection, FP16 planes, the learned denoiser with
    SVGF fallback: per-frame device ms (p50, p99) and the error against the
    FP64 ground truth on 4 sampled frames."""
    from voxelpathtracer_gb300 import learned, quality
    X, Y, Z = LARGE_WORLD
    W, H = LARGE_RES
    rng = np.random.default_rng(0)
    theta0 = float(rng.uniform(0.0, 360.0))
    t0 = time.perf_counter()
    vox = vpt.generate_world(X, Y, Z, seed=0)
    blocks = vpt.generate_block_table(100, seed=0)
    gen_s = time.perf_counter() - t0
    net = None
    weights = learned.WEIGHTS_LARGE if learned.WEIGHTS_LARGE.exists() else learned.WEIGHTS
    if weights.exists():
        net = vpt.UNet(1, H, W, device=local)
        net.set_params(learned.load(weights)[0])
    sampled = (15, 31, 47, 63)
    crop = (W // 2 - 320, H // 2 - 180, 640, 360)
    x0, y0, cw, ch = crop
    ms, crops, used_all = [], {}, []
    with vpt.Context(width=W, height=H, device=local, storage=1, bounces=2) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.synchronize()
        stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
        with torch.cuda.stream(stream):
            for k in range(3):   # warm-up on the first camera, then a fresh history
                ctx.render_frame_learned(orbit_camera(vpt, 0, theta0, W, H), frame_at(vpt, 0), net, readback=False)
            torch.cuda.synchronize()
            ctx.reset_history()
            for k in range(64):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                _, used = ctx.render_frame_learned(orbit_camera(vpt, k, theta0, W, H), frame_at(vpt, k), net,
                                                   readback=False)
                e1.record(stream)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
                used_all.append(used)
                if k in sampled:
                    # the colour plane is not part of the swapped history: it still holds this frame
                    crops[k] = ctx.read_plane("COLOR")[y0:y0 + ch, x0:x0 + cw].astype(np.float64)
    if net is not None:
        net.close()
    errs, errs_svgf = {}, {}
    if not args.no_quality:
        # the SVGF path on the same orbit: the fallback, and the yardstick of the error
        svgf_crops = {}
        with vpt.Context(width=W, height=H, device=local, storage=1, bounces=2) as ctx:
            ctx.upload_world(vox)
            ctx.set_block_table(blocks)
            ctx.build_df()
            for k in range(64):
                ctx.render_frame(orbit_camera(vpt, k, theta0, W, H), frame_at(vpt, k), readback=False)
                if k in sampled:
                    svgf_crops[k] = ctx.read_plane("COLOR")[y0:y0 + ch, x0:x0 + cw].astype(np.float64)
        with quality.make_gt_context(W, H, vox, blocks, device=local, bounces=2) as g:
            for k in sampled:
                gt, _ = quality.ground_truth_color(g, orbit_camera(vpt, k, theta0, W, H), frame_at(vpt, k), crop,
                                                   spp=1024)
                errs[str(k)] = quality.rmse(crops[k], gt)
                errs_svgf[str(k)] = quality.rmse(svgf_crops[k], gt)
    return {"world": list(LARGE_WORLD), "resolution": list(LARGE_RES), "spp": 1, "bounces": 2, "storage": "fp16",
            "frames": 64, "orbit": {"radius": 200.0, "height": 150.0, "deg_per_frame": 1.0, "theta0_deg": theta0},
            "denoiser": "learned" if all(used_all) else ("svgf fallback" if not any(used_all) else "mixed"),
            "weights": weights.name if net is not None else None,
            "frame_ms_p50": float(np.percentile(ms, 50)), "frame_ms_p99": float(np.percentile(ms, 99)),
            "frame_ms_max": float(max(ms)), "world_generate_s": gen_s,
            "error_vs_fp64_gt": {"crop": list(crop), "gt_spp": 1024, "rmse_by_frame": errs,
                                 "svgf_rmse_by_frame": errs_svgf}}


# ------------------------------------------------------- CPU (oracle) arm --
class OracleFrames:
    """Whole frames of the workload rendered by the CPU restatement (oracle/):
    primary, sun-shadow and diffuse traces, SVGF (pre-temporal 3x3, temporal,
    variance, 5 a-trous iterations) and the colour pass, the history carried
    from frame to frame as libvpt carries it. gen makes the cameras and frame
    constants (oracle.inputs for the reference arm)."""

    def __init__(self, oracle, gen, vox, blocks, yaw, pitch, storage=0, gi_divisor=1, reflection_spp=0, bounces=1):
        W, H = RES
        self.oracle, self.gen, self.yaw, self.pitch = oracle, gen, yaw, pitch
        from oracle import inputs
        self.cfg = inputs.default_config(width=W, height=H, storage=storage, gi_divisor=gi_divisor,
                                         reflection_spp=reflection_spp, bounces=bounces)
        self.world = oracle.World(vox, oracle.build_df(vox), blocks)
        self.prev_g, self.hist = oracle.empty_history(H, W, gi_divisor)
        self.prev_refl = None
        self.prev_cam = None

    def render(self, step):
        """Frame `step`; returns (seconds, DF-DDA rays traced)."""
        o = self.oracle
        cam = camera_at(self.gen, self.yaw, self.pitch, step)
        fr = frame_at(self.gen, step)
        prev_cam = self.prev_cam if self.prev_cam is not None else cam
        with o.Counting() as cnt:
            t0 = time.perf_counter()
            r = o.render_frame(self.world, cam, prev_cam, self.cfg, fr, self.prev_g, self.hist, self.prev_refl)
            dt = time.perf_counter() - t0
        self.prev_g = {k: r["g"][k] for k in ("t", "face", "block")}
        self.hist = r["svgf"]["temporal"]
        if r["refl"] is not None:
            self.prev_refl = {"out": r["refl"]["out"], "hit": r["refl"]["hit"], "stable": r["refl"]["stable"]}
        self.prev_cam = cam
        return dt, sum(cnt.rays.values())


def cpu_baseline(args, vox, blocks, yaw, pitch):
    """Whole frames of the workload rendered by the CPU restatement on all host
    threads, repeated until args.cpu_seconds of CPU work have accumulated."""
    import oracle
    from oracle import inputs
    of = OracleFrames(oracle, inputs, vox, blocks, yaw, pitch, args.storage, args.gi_divisor, args.reflection_spp,
                      args.bounces)
    t_sum, rays_sum, frames = 0.0, 0, 0
    while t_sum < args.cpu_seconds:
        dt, rays = of.render(frames)
        t_sum += dt
        rays_sum += rays
        frames += 1
    return {"value": rays_sum / t_sum, "unit": "rays/s", "cores": oracle.omp_threads(), "kind": "port",
            "ms_per_frame": 1e3 * t_sum / frames,
            "sample": f"whole frames 0..{frames - 1} of the workload (traces, SVGF and colour pass of the CPU "
                      f"restatement): {rays_sum} rays in {t_sum:.1f} s"}


def run_reference(args):
    """The reference's algorithm on the host cores: the CPU restatement renders
    the same whole frames as the GPU arm. Nothing of libvpt is loaded."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle
    from oracle import inputs
    X, Y, Z = WORLD
    vox = inputs.generate_world(X, Y, Z, seed=0)
    blocks = inputs.generate_block_table(100, seed=0)
    yaw, pitch = inputs.seeded_pose(0)
    of = OracleFrames(oracle, inputs, vox, blocks, yaw, pitch, args.storage, args.gi_divisor, args.reflection_spp,
                      args.bounces)
    times, rays = [], []
    for s in range(args.warmup + args.steps):
        dt, n = of.render(s)
        if s >= args.warmup:
            times.append(dt)
            rays.append(n)
    value = sum(rays) / sum(times)
    sample = (f"whole frames {args.warmup}..{args.warmup + args.steps - 1} of the workload after {args.warmup} "
              f"warm-up frames: traces, SVGF and colour pass of the CPU restatement, {sum(rays)} rays in "
              f"{sum(times):.1f} s")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "rays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times),
        "frame_ms": 1e3 * sum(times) / len(times),
        "rays_per_frame": float(np.mean(rays)),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if args.storage == 0 else "f16-storage/f32",
        "data": "synthetic",
        "config": workload_config(args, world),
        "cpu_baseline": {"value": value, "unit": "rays/s", "cores": oracle.omp_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference implements this path in GLSL behind OpenGL, which cannot run here; its CPU "
                "restatement (oracle/, OpenMP) renders the same frames on the host cores instead",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--storage", type=int, default=0, help="0 = fp32 planes, 1 = fp16 planes")
    ap.add_argument("--gi-divisor", type=int, default=1,
                    help="GI grid = frame / this (the reference's DiffuseTraceResolution is 1/4)")
    ap.add_argument("--bounces", type=int, default=1, choices=[1, 2],
                    help="diffuse bounces in the timed frame (2 takes the per-texel diffuse kernel)")
    ap.add_argument("--reflection-spp", type=int, default=0,
                    help="reflection rays per GI texel in the timed frame (0: no reflection pass)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="CPU work accumulated by the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the FP16-storage variant")
    ap.add_argument("--no-quality", action="store_true", help="skip the ground-truth error measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-world batched comparison")
    ap.add_argument("--no-df", action="store_true", help="skip the distance-field build timing")
    ap.add_argument("--split-temporal", action="store_true",
                    help="run the temporal pass's history gather on the second stream beside the diffuse trace and "
                         "only its blend after the pre-filter (vpt_tuning.split_temporal = 1)")
    ap.add_argument("--inline-shadow", action="store_true",
                    help="run the main frame's sun-shadow pass in line on the context stream instead of on a second "
                         "stream beside the diffuse trace and SVGF (vpt_tuning.overlap_shadow = 0)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-denoiser measurements")
    ap.add_argument("--no-large", action="store_true", help="skip the 512^3 / 3840x2160 combined run")
    ap.add_argument("--gt-spp", type=int, default=4096, help="samples per pixel of the FP64 ground truth")
    ap.add_argument("--error-curve", action="store_true",
                    help="also measure the RMSE against the ground truth over 33 frames, static and panning camera")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the dominant kernel from an ncu capture")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
