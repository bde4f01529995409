// Minecraft Anvil region import (Core/NBT/Importer.cpp, whose decoding the
// reference delegates to enkiMI): region files (.mca) of zlib-compressed NBT
// chunks in the pre-flattening layout (Level / xPos, zPos / Sections[] with
// Y, Blocks[4096] and the Data nibble array), written into the reference's
// 384 x 128 x 384 world around an import origin. Host code; the DEFLATE
// decoder (RFC 1951, zlib wrapper RFC 1950) and the NBT reader are written
// here from the published formats.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <dirent.h>

#include "../../include/vpt.h"

namespace {

// ------------------------------------------------------------- inflate --
struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool err = false;
    int bits(int need) {
        while (cnt < need) {
            if (pos >= n) {
                err = true;
                return 0;
            }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const int v = (int)(buf & ((1u << need) - 1u));
        buf >>= need;
        cnt -= need;
        return v;
    }
};

// Canonical Huffman code: counts per length and symbols in code order.
struct Huffman {
    uint16_t count[16] = {};
    uint16_t symbol[320] = {};
    bool build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof count);
        for (int s = 0; s < n; s++) count[lengths[s]]++;
        if (count[0] == n) return true;   // no codes: a valid, empty table
        int left = 1;
        for (int len = 1; len < 16; len++) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;   // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++) offs[len + 1] = offs[len] + count[len];
        for (int s = 0; s < n; s++)
            if (lengths[s]) symbol[offs[lengths[s]]++] = (uint16_t)s;
        return true;
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= br.bits(1);
            if (br.err) return -1;
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t cap) {
    for (;;) {
        int sym = lit.decode(br);
        if (sym < 0) return false;
        if (sym < 256) {
            if (out.size() >= cap) return false;
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29) return false;
            const int len = kLenBase[sym] + br.bits(kLenExtra[sym]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30) return false;
            const size_t d = (size_t)kDistBase[ds] + (size_t)br.bits(kDistExtra[ds]);
            if (br.err || d > out.size() || out.size() + (size_t)len > cap) return false;
            const size_t from = out.size() - d;
            for (int k = 0; k < len; k++) out.push_back(out[from + (size_t)k]);
        }
    }
}

// zlib stream (RFC 1950) -> bytes; false on any malformed input, a failed
// Adler-32 check or more than `cap` output bytes.
bool zlib_inflate(const uint8_t* src, size_t n, std::vector<uint8_t>& out, size_t cap) {
    out.clear();
    if (n < 6) return false;
    const int cmf = src[0], flg = src[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;
    BitReader br{src + 2, n - 6};
    int last = 0;
    while (!last) {
        last = br.bits(1);
        const int type = br.bits(2);
        if (br.err) return false;
        if (type == 0) {   // stored
            br.buf = 0;
            br.cnt = 0;
            if (br.pos + 4 > br.n) return false;
            const unsigned len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            const unsigned nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
            br.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || br.pos + len > br.n || out.size() + len > cap) return false;
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {   // fixed codes (RFC 1951 3.2.6)
            Huffman lit, dist;
            uint8_t l[288], dl[30];
            for (int s = 0; s < 144; s++) l[s] = 8;
            for (int s = 144; s < 256; s++) l[s] = 9;
            for (int s = 256; s < 280; s++) l[s] = 7;
            for (int s = 280; s < 288; s++) l[s] = 8;
            for (int s = 0; s < 30; s++) dl[s] = 5;
            lit.build(l, 288);
            dist.build(dl, 30);
            if (!inflate_codes(br, lit, dist, out, cap)) return false;
        } else if (type == 2) {   // dynamic codes
            const int nlen = br.bits(5) + 257, ndist = br.bits(5) + 1, ncode = br.bits(4) + 4;
            if (br.err || nlen > 286 || ndist > 30) return false;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int k = 0; k < ncode; k++) cl[order[k]] = (uint8_t)br.bits(3);
            Huffman lencode;
            if (br.err || !lencode.build(cl, 19)) return false;
            uint8_t lengths[320] = {};
            int idx = 0;
            while (idx < nlen + ndist) {
                const int sym = lencode.decode(br);
                if (sym < 0) return false;
                if (sym < 16) {
                    lengths[idx++] = (uint8_t)sym;
                } else {
                    int rep, val = 0;
                    if (sym == 16) {
                        if (idx == 0) return false;
                        val = lengths[idx - 1];
                        rep = 3 + br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + br.bits(3);
                    } else {
                        rep = 11 + br.bits(7);
                    }
                    if (br.err || idx + rep > nlen + ndist) return false;
                    while (rep--) lengths[idx++] = (uint8_t)val;
                }
            }
            if (lengths[256] == 0) return false;
            Huffman lit, dist;
            if (!lit.build(lengths, nlen) || !dist.build(lengths + nlen, ndist)) return false;
            if (!inflate_codes(br, lit, dist, out, cap)) return false;
        } else {
            return false;
        }
    }
    // Adler-32 of the output, big-endian after the stream (byte aligned)
    size_t tail = 2 + br.pos;
    if (tail + 4 > n) return false;
    uint32_t a = 1, b = 0;
    for (uint8_t v : out) {
        a = (a + v) % 65521u;
        b = (b + a) % 65521u;
    }
    const uint32_t want = ((uint32_t)src[tail] << 24) | ((uint32_t)src[tail + 1] << 16) |
                          ((uint32_t)src[tail + 2] << 8) | src[tail + 3];
    return ((b << 16) | a) == want;
}

// ------------------------------------------------------------------ NBT --
// A pre-flattening chunk: its position and, per section Y (-128..127), the
// 4096 block ids (YZX order) and the 2048-byte data nibble array (or none).
struct Section {
    int y = 0;
    const uint8_t* blocks = nullptr;
    const uint8_t* data = nullptr;
};
struct Chunk {
    bool has_x = false, has_z = false;
    int32_t x = 0, z = 0;
    std::vector<Section> sections;
};

struct NbtReader {
    const uint8_t* p;
    size_t n, pos = 0;
    bool err = false;
    int depth = 0;
    bool need(size_t k) {
        if (pos + k > n) err = true;
        return !err;
    }
    uint8_t u8() { return need(1) ? p[pos++] : 0; }
    int32_t i32() {
        if (!need(4)) return 0;
        const uint32_t v = ((uint32_t)p[pos] << 24) | ((uint32_t)p[pos + 1] << 16) | ((uint32_t)p[pos + 2] << 8) | p[pos + 3];
        pos += 4;
        return (int32_t)v;
    }
    uint16_t u16() {
        if (!need(2)) return 0;
        const uint16_t v = (uint16_t)((p[pos] << 8) | p[pos + 1]);
        pos += 2;
        return v;
    }
    std::string name() {
        const uint16_t len = u16();
        if (!need(len)) return std::string();
        std::string s((const char*)p + pos, len);
        pos += len;
        return s;
    }
    // Reads the payload of a tag of `type`; `field` is its name (empty inside
    // lists). Records what the importer needs, like enkiMI's scan: the first
    // xPos / zPos ints and, inside a section compound, Y, Blocks and Data.
    void payload(int type, const std::string& field, Chunk& c, Section* sec) {
        if (err) return;
        if (++depth > 64) {
            err = true;
            return;
        }
        switch (type) {
            case 1: {
                const int8_t v = (int8_t)u8();
                if (sec && field == "Y") sec->y = v;
                break;
            }
            case 2: u16(); break;
            case 3: {
                const int32_t v = i32();
                if (sec && field == "Y") sec->y = v;
                if (field == "xPos" && !c.has_x) { c.x = v; c.has_x = true; }
                if (field == "zPos" && !c.has_z) { c.z = v; c.has_z = true; }
                break;
            }
            case 4: case 6: need(8); pos += err ? 0 : 8; break;
            case 5: need(4); pos += err ? 0 : 4; break;
            case 7: {
                const int32_t len = i32();
                if (len < 0 || !need((size_t)len)) { err = true; break; }
                if (sec && field == "Blocks" && !sec->blocks && len >= 4096) sec->blocks = p + pos;
                if (sec && field == "Data" && !sec->data && len >= 2048) sec->data = p + pos;
                pos += (size_t)len;
                break;
            }
            case 8: name(); break;
            case 9: {
                const int et = u8();
                const int32_t len = i32();
                if (len < 0) { err = true; break; }
                const bool sections = field == "Sections" && et == 10;
                for (int32_t k = 0; k < len && !err; k++) {
                    if (sections) {
                        Section s;
                        payload(et, std::string(), c, &s);
                        if (!err) c.sections.push_back(s);
                    } else {
                        payload(et, std::string(), c, nullptr);
                    }
                }
                break;
            }
            case 10: {
                for (;;) {
                    const int t = u8();
                    if (err || t == 0) break;
                    const std::string nm = name();
                    payload(t, nm, c, sec);
                    if (err) break;
                }
                break;
            }
            case 11: {
                const int32_t len = i32();
                if (len < 0 || !need((size_t)len * 4)) { err = true; break; }
                pos += (size_t)len * 4;
                break;
            }
            case 12: {
                const int32_t len = i32();
                if (len < 0 || !need((size_t)len * 8)) { err = true; break; }
                pos += (size_t)len * 8;
                break;
            }
            default: err = true;
        }
        --depth;
    }
};

// ------------------------------------------------------------ importer --
constexpr int kWX = 384, kWY = 128, kWZ = 384;   // WORLD_SIZE_* (Core/Macros.h:3-5)

// WriteVoxel (Core/NBT/Importer.cpp:91-108): shift by the import origin
// (truncated to integers) and half the world in x and z, drop air and
// anything outside, store x + y X + z X Y.
inline void write_voxel(uint8_t* out, uint8_t voxel, int x, int y, int z, const int origin[3]) {
    x -= origin[0];
    y -= origin[1];
    z -= origin[2];
    x += kWX / 2;
    z += kWZ / 2;
    if (y >= 128 || x >= 384 || z >= 384 || y < 0 || x < 0 || z < 0 || voxel == 0) return;
    out[(size_t)x + (size_t)y * kWX + (size_t)z * kWX * kWY] = voxel;
}

// ImportRegionFile (Core/NBT/Importer.cpp:111-166): every present chunk,
// every section, y-z-x order; a voxel goes in only when its data value is 0,
// through the Minecraft-id table. Returns false on an unreadable file.
bool import_region(const std::string& path, const uint8_t lut[256], const int origin[3], uint8_t* out,
                   int* chunks_read) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::vector<uint8_t> file;
    uint8_t tmp[1 << 16];
    size_t got;
    while ((got = std::fread(tmp, 1, sizeof tmp, f)) > 0) file.insert(file.end(), tmp, tmp + got);
    std::fclose(f);
    if (file.size() < 8192) return false;
    std::vector<uint8_t> nbt;
    for (int i = 0; i < 1024; i++) {
        const uint8_t* loc = file.data() + 4 * i;
        const size_t offset = (((size_t)loc[0] << 16) | ((size_t)loc[1] << 8) | loc[2]) * 4096u;
        const size_t sectors = loc[3];
        if (offset == 0 || sectors == 0 || offset + 5 > file.size()) continue;
        const uint8_t* h = file.data() + offset;
        const size_t len = ((size_t)h[0] << 24) | ((size_t)h[1] << 16) | ((size_t)h[2] << 8) | h[3];
        if (len < 1 || offset + 4 + len > file.size()) continue;
        if (h[4] != 2) continue;   // zlib only
        if (!zlib_inflate(h + 5, len - 1, nbt, (size_t)64 << 20)) continue;
        NbtReader rd{nbt.data(), nbt.size()};
        Chunk c;
        const int root = rd.u8();
        if (root != 10) continue;
        rd.name();
        rd.payload(10, std::string(), c, nullptr);
        if (rd.err || !c.has_x || !c.has_z) continue;
        *chunks_read += 1;
        // sections in index order (Y + 128), as enkiMI stores them
        for (int idx = 0; idx < 256; idx++) {
            const Section* s = nullptr;
            for (const Section& t : c.sections)
                if (t.blocks && t.y + 128 == idx) s = &t;   // the last section with this Y wins, as in enkiMI
            if (!s) continue;
            const int ox = c.x * 16, oy = s->y * 16, oz = c.z * 16;
            for (int y = 0; y < 16; y++)
                for (int z = 0; z < 16; z++)
                    for (int x = 0; x < 16; x++) {
                        const int pos = y * 256 + z * 16 + x;
                        uint8_t voxel = s->blocks[pos];
                        uint8_t dataval = 0;
                        if (s->data) dataval = (uint8_t)(0xF & (s->data[pos / 2] >> (4 * (pos & 1))));
                        if (dataval == 0) {
                            voxel = lut[voxel];
                            write_voxel(out, voxel, ox + x, oy + y, oz + z, origin);
                        }
                    }
        }
    }
    return true;
}

}  // namespace

extern "C" {

vpt_status vpt_import_mca_world(const char* directory, const uint8_t mcid_to_block[256], const float origin[3],
                                uint8_t* out, size_t out_bytes, int32_t* chunks_read) {
    const size_t need = (size_t)kWX * kWY * kWZ;
    if (!directory || !mcid_to_block || !origin || !out || out_bytes < need) return VPT_ERR_INVALID_ARG;
    DIR* d = opendir(directory);
    if (!d) return VPT_ERR_INVALID_ARG;
    std::vector<std::string> files;
    while (const dirent* e = readdir(d)) {
        const std::string nm = e->d_name;
        const size_t dot = nm.find_last_of('.');
        if (dot != std::string::npos && nm.substr(dot + 1) == "mca") files.push_back(std::string(directory) + "/" + nm);
    }
    closedir(d);
    // glm::ivec3(ImportOrigin): truncation toward zero
    const int org[3] = {(int)origin[0], (int)origin[1], (int)origin[2]};
    std::memset(out, 0, need);
    int read = 0;
    for (const std::string& f : files)
        if (!import_region(f, mcid_to_block, org, out, &read)) return VPT_ERR_INVALID_ARG;
    if (chunks_read) *chunks_read = read;
    return VPT_OK;
}

}  // extern "C"
