"""The benchmark's seeded inputs, generated on the CPU without libvpt.

TEST INFRASTRUCTURE ONLY (like the rest of oracle/): the CPU reference arm of
bench.py renders its frames from these, so it never loads the product library,
and tests/test_oracle_inputs.py checks them against libvpt's own generators
value for value, so a defect in either generator shows.

What is restated:

* the terrain of the benchmark text (configs 1-2: h(x, z) = 40 + 16 fbm(x, z),
  4 octaves of smoothstep value noise, base frequency 1/64, gain 0.5; the top
  voxel grass or, in 1 column of 16, a seeded surface block; three layers of
  dirt; stone below) over lattice values hashed with splitmix64 -- vectorised
  over all columns with numpy, in float64 with the same operation order as
  the scalar C++ generator so the heights agree bit for bit;
* the 100-entry block table (albedo RGB8, roughness, metalness uniform from the
  seed, round(5%) of the ids >= 4 emissive, picked by a seeded Fisher-Yates);
* glm::lookAt / glm::perspective cameras (Core/FpsCamera.cpp:24 builds its
  matrices with glm) and their inverses by Gauss-Jordan elimination with
  partial pivoting, in float64 through Python's math module, rounded to fp32;
* the per-frame and per-context defaults (sun direction, radiances, step caps).
"""
from __future__ import annotations

import math

import numpy as np

from . import OCamera, OFrame, OParams

_M64 = (1 << 64) - 1
BLOCK_DTYPE = np.dtype([("albedo", np.uint8, 3), ("roughness", np.uint8), ("metalness", np.uint8),
                        ("emissive", np.uint8)])


# ------------------------------------------------------------------ world --
def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on a uint64 array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def _lattice(ix: np.ndarray, iz: np.ndarray, octave: int, seed: int) -> np.ndarray:
    """Lattice value in [-1, 1] at integer (ix, iz) of one octave."""
    with np.errstate(over="ignore"):
        key = (ix.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)) ^ \
              (iz.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)) ^ \
              np.uint64(((octave + 1) * 0x165667B19E3779F9) & _M64)
        h = _splitmix64(np.uint64(seed) ^ _splitmix64(key))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) * 2.0 - 1.0


def _value_noise(x: np.ndarray, z: np.ndarray, octave: int, seed: int) -> np.ndarray:
    fx0, fz0 = np.floor(x), np.floor(z)
    ix, iz = fx0.astype(np.int64), fz0.astype(np.int64)
    fx, fz = x - fx0, z - fz0
    ux = fx * fx * (3.0 - 2.0 * fx)
    uz = fz * fz * (3.0 - 2.0 * fz)
    a, b = _lattice(ix, iz, octave, seed), _lattice(ix + 1, iz, octave, seed)
    c, d = _lattice(ix, iz + 1, octave, seed), _lattice(ix + 1, iz + 1, octave, seed)
    ab = a + (b - a) * ux
    cd = c + (d - c) * ux
    return ab + (cd - ab) * uz


def _fbm(x: np.ndarray, z: np.ndarray, seed: int) -> np.ndarray:
    total = np.zeros_like(x)
    amp, norm, freq = 1.0, 0.0, 1.0 / 64.0
    for octave in range(4):
        total = total + amp * _value_noise(x * freq, z * freq, octave, seed)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def generate_world(X: int, Y: int, Z: int, seed: int = 0, n_blocks: int = 100) -> np.ndarray:
    """Seeded value-noise terrain, shape (Z, Y, X) uint8, x fastest in memory."""
    if min(X, Y, Z) <= 0 or not 4 <= n_blocks <= 256:
        raise ValueError("bad world dimensions or block count")
    z, x = np.meshgrid(np.arange(Z, dtype=np.float64), np.arange(X, dtype=np.float64), indexing="ij")
    top = np.floor(40.0 + 16.0 * _fbm(x, z, seed)).astype(np.int64)
    top = np.clip(top, 0, Y - 1)
    with np.errstate(over="ignore"):
        col = _splitmix64(np.uint64((seed * 0x2545F4914F6CDD1D) & _M64) +
                          x.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15) +
                          z.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03))
    top_block = np.ones((Z, X), np.uint8)
    if n_blocks > 4:
        scattered = (col & np.uint64(15)) == 0
        pick = (np.uint64(4) + (col >> np.uint64(8)) % np.uint64(n_blocks - 4)).astype(np.uint8)
        top_block = np.where(scattered, pick, top_block)
    y = np.arange(Y, dtype=np.int64)[None, :, None]
    t = top[:, None, :]
    vox = np.where(y > t, 0, np.where(y == t, top_block[:, None, :], np.where(y >= t - 3, 2, 3)))
    return np.ascontiguousarray(vox, dtype=np.uint8)


# ------------------------------------------------------------ block table --
def _splitmix64_int(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def generate_block_table(n: int = 100, seed: int = 0) -> np.ndarray:
    """n entries of {albedo RGB8, roughness, metalness, emissive}; entry 0 is air."""
    if not 1 <= n <= 256:
        raise ValueError("block count out of range")
    state = [(seed ^ 0xA0761D6478BD642F) & _M64]

    def nxt() -> int:
        state[0] = _splitmix64_int(state[0])
        return state[0]

    t = np.zeros(n, BLOCK_DTYPE)
    for i in range(1, n):
        r = nxt()
        t[i]["albedo"] = [r & 0xFF, (r >> 8) & 0xFF, (r >> 16) & 0xFF]
        t[i]["roughness"] = (r >> 24) & 0xFF
        t[i]["metalness"] = (r >> 32) & 0xFF
    candidates = n - 4
    if candidates > 0:
        k = min(max(int(math.floor(0.05 * (n - 1) + 0.5)), 1), candidates)
        ids = list(range(4, n))
        for i in range(candidates - 1, 0, -1):
            j = nxt() % (i + 1)
            ids[i], ids[j] = ids[j], ids[i]
        for i in ids[:k]:
            t[i]["emissive"] = 1
    return t


# ----------------------------------------------------------------- camera --
def _inverse(m: list) -> list:
    """Inverse of a column-major 4x4 (list of 16 floats), Gauss-Jordan with partial pivoting."""
    a = [[m[c * 4 + r] for c in range(4)] + [1.0 if r == c else 0.0 for c in range(4)] for r in range(4)]
    for col in range(4):
        piv = col
        for r in range(col + 1, 4):
            if abs(a[r][col]) > abs(a[piv][col]):
                piv = r
        if a[piv][col] == 0.0:
            raise ValueError("singular matrix")
        a[piv], a[col] = a[col], a[piv]
        inv = 1.0 / a[col][col]
        a[col] = [v * inv for v in a[col]]
        for r in range(4):
            if r == col or a[r][col] == 0.0:
                continue
            f = a[r][col]
            a[r] = [a[r][c] - f * a[col][c] for c in range(8)]
    return [a[r][c + 4] for c in range(4) for r in range(4)]


def camera_from_pose(position, yaw_deg: float, pitch_deg: float, fov_deg: float = 90.0, aspect: float = 16 / 9,
                     znear: float = 0.1, zfar: float = 1000.0) -> OCamera:
    """View / projection matrices (glm::lookAt, glm::perspective) and their inverses."""
    f32 = lambda v: float(np.float32(v))  # noqa: E731  (the ABI passes fp32 arguments)
    yaw_deg, pitch_deg, fov_deg, aspect, znear, zfar = map(f32, (yaw_deg, pitch_deg, fov_deg, aspect, znear, zfar))
    pos = [f32(p) for p in position]
    yaw, pitch = yaw_deg * math.pi / 180.0, pitch_deg * math.pi / 180.0
    f = [math.cos(yaw) * math.cos(pitch), math.sin(pitch), math.sin(yaw) * math.cos(pitch)]
    fl = math.sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
    f = [v / fl for v in f]
    up = (0.0, 1.0, 0.0)
    s = [f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]]
    sl = math.sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2])
    if sl < 1e-9:
        raise ValueError("looking straight up or down")
    s = [v / sl for v in s]
    u = [s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]]
    view = [1.0 if k % 5 == 0 else 0.0 for k in range(16)]
    view[0], view[4], view[8] = s
    view[1], view[5], view[9] = u
    view[2], view[6], view[10] = -f[0], -f[1], -f[2]
    view[12] = -(s[0] * pos[0] + s[1] * pos[1] + s[2] * pos[2])
    view[13] = -(u[0] * pos[0] + u[1] * pos[1] + u[2] * pos[2])
    view[14] = f[0] * pos[0] + f[1] * pos[1] + f[2] * pos[2]
    th = math.tan(fov_deg * math.pi / 180.0 / 2.0)
    proj = [0.0] * 16
    proj[0] = 1.0 / (aspect * th)
    proj[5] = 1.0 / th
    proj[10] = -(zfar + znear) / (zfar - znear)
    proj[11] = -1.0
    proj[14] = -(2.0 * zfar * znear) / (zfar - znear)
    cam = OCamera()
    cam.view[:] = [f32(v) for v in view]
    cam.proj[:] = [f32(v) for v in proj]
    cam.inv_view[:] = [f32(v) for v in _inverse(view)]
    cam.inv_proj[:] = [f32(v) for v in _inverse(proj)]
    cam.position[:] = pos
    cam.pad = 0.0
    return cam


def seeded_pose(seed: int, yaw_range=(0.0, 360.0), pitch_range=(-40.0, -10.0)):
    """Yaw and pitch drawn uniformly from the seed."""
    rng = np.random.default_rng(seed)
    return float(rng.uniform(*yaw_range)), float(rng.uniform(*pitch_range))


# --------------------------------------------------------------- defaults --
def default_config(**kw) -> OParams:
    """The per-context defaults: 1920x1080, the reference's step caps (350 primary
    and shadow, 48 diffuse, 128 bounce shadow), 1 spp, 1 bounce, fp32 planes, SVGF
    with 5 a-trous iterations and ColorPhiBias 3.325 (Core/Pipeline.cpp:85)."""
    p = OParams()
    vals = dict(width=1920, height=1080, primary_max_steps=350, shadow_max_steps=350, diffuse_max_steps=48,
                bounce_shadow_max_steps=128, bounces=1, spp=1, storage=0, atrous_iterations=5,
                resolution_scale=1.0, gi_divisor=1, reflection_spp=0, reflection_max_steps=64,
                reflection_shadow_max_steps=150, reflection_temporal=1, reflection_denoise=1,
                color_phi_bias=3.325, device=0, denoiser=0, alpha_test=0, alpha_test_shadows=0)
    vals.update(kw)
    for k, v in vals.items():
        setattr(p, k, v)
    return p


def default_frame(**kw) -> OFrame:
    """A morning sun along normalize(0.3, 0.8, 0.5), evaluated in fp32."""
    f = OFrame()
    sx, sy, sz = np.float32(0.3), np.float32(0.8), np.float32(0.5)
    ln = np.sqrt((sx * sx + sy * sy) + sz * sz, dtype=np.float32)
    f.sun_dir[:] = [float(sx / ln), float(sy / ln), float(sz / ln)]
    f.time = 1.0
    f.sun_radiance[:] = [5.2, 4.9, 4.4]
    f.moon_radiance[:] = [0.05, 0.06, 0.09]
    f.frame_index = 0
    f.seed = 0
    f.gi_sun_strength = 1.0
    f.gi_sky_strength = 1.125
    f.diffuse_light_intensity = 1.25
    f.temporal = 1
    for k, v in kw.items():
        if k in ("sun_dir", "sun_radiance", "moon_radiance"):
            getattr(f, k)[:] = [float(x) for x in v]
        else:
            setattr(f, k, v)
    return f
