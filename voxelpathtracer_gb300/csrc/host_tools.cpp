// Host-side helpers of libvpt: the seeded synthetic world and block table the
// benchmarks use, and the glm-style camera matrices. Everything here runs in
// double precision on the host and is deterministic across x86-64 and aarch64
// (built with -ffp-contract=off).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include "vpt.h"

namespace {

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Lattice value in [-1, 1] for (ix, iz) of octave `o`.
double lattice(int64_t ix, int64_t iz, int o, uint64_t seed) {
    uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)ix * 0x9E3779B97F4A7C15ull ^
                                              (uint64_t)iz * 0xC2B2AE3D27D4EB4Full ^
                                              (uint64_t)(o + 1) * 0x165667B19E3779F9ull));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

// Value noise: smoothstep-interpolated lattice values.
double value_noise(double x, double z, int o, uint64_t seed) {
    double fx0 = std::floor(x), fz0 = std::floor(z);
    int64_t ix = (int64_t)fx0, iz = (int64_t)fz0;
    double fx = x - fx0, fz = z - fz0;
    double ux = fx * fx * (3.0 - 2.0 * fx);
    double uz = fz * fz * (3.0 - 2.0 * fz);
    double a = lattice(ix, iz, o, seed), b = lattice(ix + 1, iz, o, seed);
    double c = lattice(ix, iz + 1, o, seed), d = lattice(ix + 1, iz + 1, o, seed);
    double ab = a + (b - a) * ux;
    double cd = c + (d - c) * ux;
    return ab + (cd - ab) * uz;
}

// fbm: 4 octaves, base frequency 1/64, gain 0.5, normalised to [-1, 1].
double fbm(double x, double z, uint64_t seed) {
    double sum = 0.0, amp = 1.0, norm = 0.0, freq = 1.0 / 64.0;
    for (int o = 0; o < 4; o++) {
        sum += amp * value_noise(x * freq, z * freq, o, seed);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return sum / norm;
}

void mat_identity(double* m) {
    for (int k = 0; k < 16; k++) m[k] = (k % 5 == 0) ? 1.0 : 0.0;
}

// Gauss-Jordan inverse of a column-major 4x4 with partial pivoting.
bool mat_inverse(const double* m, double* out) {
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = (r == c) ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (a[piv][col] == 0.0) return false;
        if (piv != col)
            for (int c = 0; c < 8; c++) std::swap(a[piv][c], a[col][c]);
        double inv = 1.0 / a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            double f = a[r][col];
            if (f == 0.0) continue;
            for (int c = 0; c < 8; c++) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[c * 4 + r] = a[r][c + 4];
    return true;
}

}  // namespace

extern "C" {

vpt_status vpt_generate_world(uint8_t* out, int32_t X, int32_t Y, int32_t Z, uint64_t seed, int32_t n_blocks) {
    if (!out || X <= 0 || Y <= 0 || Z <= 0 || n_blocks < 4 || n_blocks > 256) return VPT_ERR_INVALID_ARG;
    const size_t plane = (size_t)X * Y;
    std::memset(out, 0, plane * (size_t)Z);
    for (int z = 0; z < Z; z++) {
        for (int x = 0; x < X; x++) {
            double h = 40.0 + 16.0 * fbm((double)x, (double)z, seed);
            int top = (int)std::floor(h);
            if (top > Y - 1) top = Y - 1;
            if (top < 0) top = 0;
            uint64_t col = splitmix64(seed * 0x2545F4914F6CDD1Dull + (uint64_t)x * 0x9E3779B97F4A7C15ull +
                                      (uint64_t)z * 0xD1B54A32D192ED03ull);
            uint8_t top_block = 1;
            if ((col & 15u) == 0 && n_blocks > 4) top_block = (uint8_t)(4 + (col >> 8) % (uint64_t)(n_blocks - 4));
            for (int y = 0; y <= top; y++) {
                uint8_t b;
                if (y == top) b = top_block;        // grass (or a scattered surface block)
                else if (y >= top - 3) b = 2;       // three layers of dirt
                else b = 3;                         // stone
                out[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * (size_t)z)] = b;
            }
        }
    }
    return VPT_OK;
}

vpt_status vpt_generate_block_table(vpt_block* out, int32_t n, uint64_t seed) {
    if (!out || n < 1 || n > 256) return VPT_ERR_INVALID_ARG;
    uint64_t s = seed ^ 0xA0761D6478BD642Full;
    auto next = [&]() { s = splitmix64(s); return s; };
    std::memset(out, 0, sizeof(vpt_block) * (size_t)n);
    for (int i = 1; i < n; i++) {
        uint64_t r = next();
        out[i].albedo[0] = (uint8_t)(r & 0xff);
        out[i].albedo[1] = (uint8_t)((r >> 8) & 0xff);
        out[i].albedo[2] = (uint8_t)((r >> 16) & 0xff);
        out[i].roughness = (uint8_t)((r >> 24) & 0xff);
        out[i].metalness = (uint8_t)((r >> 32) & 0xff);
        out[i].emissive = 0;
    }
    // exactly round(5% of the blocks) emissive, chosen among the scattered
    // surface blocks (ids >= 4) so the terrain layers stay non-emissive
    int candidates = n - 4;
    if (candidates > 0) {
        int k = (int)std::floor(0.05 * (double)(n - 1) + 0.5);
        if (k < 1) k = 1;
        if (k > candidates) k = candidates;
        std::vector<int> ids((size_t)candidates);
        for (int i = 0; i < candidates; i++) ids[(size_t)i] = 4 + i;
        for (int i = candidates - 1; i > 0; i--) {
            int j = (int)(next() % (uint64_t)(i + 1));
            std::swap(ids[(size_t)i], ids[(size_t)j]);
        }
        for (int i = 0; i < k; i++) out[ids[(size_t)i]].emissive = 1;
    }
    return VPT_OK;
}

vpt_status vpt_camera_from_pose(vpt_camera* out, const float position[3], float yaw_deg, float pitch_deg,
                                float fov_deg, float aspect, float znear, float zfar) {
    if (!out || !position || !(aspect > 0.0f) || !(fov_deg > 0.0f && fov_deg < 180.0f) || !(znear > 0.0f) ||
        !(zfar > znear))
        return VPT_ERR_INVALID_ARG;
    const double pi = 3.14159265358979323846;
    double yaw = (double)yaw_deg * pi / 180.0, pitch = (double)pitch_deg * pi / 180.0;
    double f[3] = {std::cos(yaw) * std::cos(pitch), std::sin(pitch), std::sin(yaw) * std::cos(pitch)};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& v : f) v /= fl;
    double eye[3] = {position[0], position[1], position[2]};
    double up[3] = {0.0, 1.0, 0.0};
    // glm::lookAt (right-handed)
    double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (sl < 1e-9) return VPT_ERR_INVALID_ARG;   // looking straight up or down
    for (double& v : s) v /= sl;
    double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    double view[16];
    mat_identity(view);
    view[0] = s[0]; view[4] = s[1]; view[8] = s[2];
    view[1] = u[0]; view[5] = u[1]; view[9] = u[2];
    view[2] = -f[0]; view[6] = -f[1]; view[10] = -f[2];
    view[12] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    view[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    view[14] = (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2]);
    // glm::perspective (right-handed, depth -1..1)
    double th = std::tan((double)fov_deg * pi / 180.0 / 2.0);
    double proj[16];
    for (double& v : proj) v = 0.0;
    proj[0] = 1.0 / ((double)aspect * th);
    proj[5] = 1.0 / th;
    proj[10] = -((double)zfar + (double)znear) / ((double)zfar - (double)znear);
    proj[11] = -1.0;
    proj[14] = -(2.0 * (double)zfar * (double)znear) / ((double)zfar - (double)znear);
    double iv[16], ip[16];
    if (!mat_inverse(view, iv) || !mat_inverse(proj, ip)) return VPT_ERR_INVALID_ARG;
    for (int k = 0; k < 16; k++) {
        out->view[k] = (float)view[k];
        out->proj[k] = (float)proj[k];
        out->inv_view[k] = (float)iv[k];
        out->inv_proj[k] = (float)ip[k];
    }
    out->position[0] = position[0];
    out->position[1] = position[1];
    out->position[2] = position[2];
    out->pad = 0.0f;
    return VPT_OK;
}

// ------------------------------------------------------------ world files --
// The reference's .sav (Core/WorldFileHandler.cpp:10-83) is the raw x-fastest
// volume of uint8 block ids, X*Y*Z bytes, no header (its dimensions are the
// compile-time WORLD_SIZE_*). With `header` the same bytes follow a 32-byte
// header: "VPTWORLD", uint32 version 1, uint32 X, Y, Z, uint64 seed (little
// endian).
static const char kMagic[8] = {'V', 'P', 'T', 'W', 'O', 'R', 'L', 'D'};

static void put32(unsigned char* p, uint32_t v) {
    for (int k = 0; k < 4; k++) p[k] = (unsigned char)(v >> (8 * k));
}
static uint32_t get32(const unsigned char* p) {
    uint32_t v = 0;
    for (int k = 0; k < 4; k++) v |= (uint32_t)p[k] << (8 * k);
    return v;
}

vpt_status vpt_save_world(const char* path, const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z, uint64_t seed,
                          int32_t header) {
    if (!path || !voxels || X <= 0 || Y <= 0 || Z <= 0 || X > 4096 || Y > 4096 || Z > 4096) return VPT_ERR_INVALID_ARG;
    FILE* f = fopen(path, "wb");
    if (!f) return VPT_ERR_INVALID_ARG;
    bool ok = true;
    if (header) {
        unsigned char h[32] = {0};
        memcpy(h, kMagic, 8);
        put32(h + 8, 1u);
        put32(h + 12, (uint32_t)X);
        put32(h + 16, (uint32_t)Y);
        put32(h + 20, (uint32_t)Z);
        put32(h + 24, (uint32_t)(seed & 0xffffffffu));
        put32(h + 28, (uint32_t)(seed >> 32));
        ok = fwrite(h, 1, 32, f) == 32;
    }
    const size_t n = (size_t)X * Y * Z;
    ok = ok && fwrite(voxels, 1, n, f) == n;
    ok = (fclose(f) == 0) && ok;
    return ok ? VPT_OK : VPT_ERR_INVALID_ARG;
}

vpt_status vpt_load_world(const char* path, uint8_t* out, size_t out_bytes, int32_t dims[3], uint64_t* seed) {
    if (!path || !dims) return VPT_ERR_INVALID_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) return VPT_ERR_INVALID_ARG;
    vpt_status st = VPT_OK;
    long size = -1;
    if (fseek(f, 0, SEEK_END) == 0) size = ftell(f);
    if (size < 0 || fseek(f, 0, SEEK_SET) != 0) st = VPT_ERR_INVALID_ARG;
    unsigned char h[32] = {0};
    size_t off = 0;
    if (st == VPT_OK && size >= 32 && fread(h, 1, 32, f) == 32 && memcmp(h, kMagic, 8) == 0) {
        const uint32_t X = get32(h + 12), Y = get32(h + 16), Z = get32(h + 20);
        if (get32(h + 8) != 1u || X == 0 || Y == 0 || Z == 0 || X > 4096 || Y > 4096 || Z > 4096) {
            st = VPT_ERR_INVALID_ARG;
        } else {
            dims[0] = (int32_t)X;
            dims[1] = (int32_t)Y;
            dims[2] = (int32_t)Z;
            if (seed) *seed = (uint64_t)get32(h + 24) | ((uint64_t)get32(h + 28) << 32);
            off = 32;
        }
    } else if (st == VPT_OK) {
        // raw: the caller names the dimensions
        if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) st = VPT_ERR_INVALID_ARG;
        if (seed) *seed = 0;
    }
    const size_t n = st == VPT_OK ? (size_t)dims[0] * dims[1] * dims[2] : 0;
    if (st == VPT_OK && (size_t)size != off + n) st = VPT_ERR_INVALID_ARG;   // truncated or oversized
    if (st == VPT_OK && out) {
        if (out_bytes < n || fseek(f, (long)off, SEEK_SET) != 0 || fread(out, 1, n, f) != n) st = VPT_ERR_INVALID_ARG;
    }
    fclose(f);
    return st;
}

// Positions of voxels whose block is emissive (the light list LoadWorld
// collects, Core/WorldFileHandler.cpp:50-66), in x-fastest order.
vpt_status vpt_emissive_voxels(const uint8_t* voxels, int32_t X, int32_t Y, int32_t Z, const vpt_block* table,
                               int32_t n_blocks, int32_t* xyz_out, int64_t max_out, int64_t* count) {
    if (!voxels || !table || !count || X <= 0 || Y <= 0 || Z <= 0 || n_blocks < 1 || n_blocks > 256 ||
        (max_out > 0 && !xyz_out))
        return VPT_ERR_INVALID_ARG;
    int64_t c = 0;
    for (int32_t z = 0; z < Z; z++)
        for (int32_t y = 0; y < Y; y++)
            for (int32_t x = 0; x < X; x++) {
                const uint8_t b = voxels[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)];
                if (b && b < n_blocks && table[b].emissive) {
                    if (c < max_out) {
                        xyz_out[3 * c] = x;
                        xyz_out[3 * c + 1] = y;
                        xyz_out[3 * c + 2] = z;
                    }
                    c++;
                }
            }
    *count = c;
    return VPT_OK;
}

}  // extern "C"
