"""CPU restatement of the reference's Minecraft region import, in Python.

TEST INFRASTRUCTURE ONLY (the tests use it as the checker of
vpt_import_mca_world). It follows Core/NBT/Importer.cpp: ImportRegionFile
(:111-166) walks the 1024 chunk slots of a region file, decodes each chunk's
NBT (the reference does this through enkiMI, Dependencies/enkiMI/enkimi.c:
region header of 3-byte sector offsets and sector counts, a 4-byte length
and a compression byte per chunk, zlib data; Level / xPos, zPos / Sections
with Y, Blocks[4096] in y-z-x order and the Data nibble array), and writes
every voxel whose data value is 0 through the Minecraft-id table with
WriteVoxel (:91-108): minus the origin (truncated), plus half the world in x
and z, air and out-of-range voxels dropped, into the 384 x 128 x 384 world.
Decompression uses Python's zlib; the NBT walk is written here.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

WORLD = (384, 128, 384)   # X, Y, Z (Core/Macros.h:3-5)


class _Nbt:
    def __init__(self, data: bytes):
        self.d, self.p = data, 0
        self.x = self.z = None
        self.sections = []

    def take(self, n):
        if self.p + n > len(self.d):
            raise ValueError("truncated NBT")
        b = self.d[self.p:self.p + n]
        self.p += n
        return b

    def name(self):
        (n,) = struct.unpack(">H", self.take(2))
        return self.take(n).decode("utf-8", "replace")

    def payload(self, t, field, sec):
        if t == 1:
            (v,) = struct.unpack(">b", self.take(1))
            if sec is not None and field == "Y":
                sec["y"] = v
        elif t == 2:
            self.take(2)
        elif t == 3:
            (v,) = struct.unpack(">i", self.take(4))
            if sec is not None and field == "Y":
                sec["y"] = v
            if field == "xPos" and self.x is None:
                self.x = v
            if field == "zPos" and self.z is None:
                self.z = v
        elif t in (4, 6):
            self.take(8)
        elif t == 5:
            self.take(4)
        elif t == 7:
            (n,) = struct.unpack(">i", self.take(4))
            b = self.take(n)
            if sec is not None and field == "Blocks" and "blocks" not in sec and n >= 4096:
                sec["blocks"] = np.frombuffer(b[:4096], np.uint8)
            if sec is not None and field == "Data" and "data" not in sec and n >= 2048:
                sec["data"] = np.frombuffer(b[:2048], np.uint8)
        elif t == 8:
            self.name()
        elif t == 9:
            et = self.take(1)[0]
            (n,) = struct.unpack(">i", self.take(4))
            for _ in range(n):
                if field == "Sections" and et == 10:
                    s = {}
                    self.payload(et, "", s)
                    self.sections.append(s)
                else:
                    self.payload(et, "", None)
        elif t == 10:
            while True:
                tt = self.take(1)[0]
                if tt == 0:
                    break
                self.payload(tt, self.name(), sec)
        elif t == 11:
            (n,) = struct.unpack(">i", self.take(4))
            self.take(4 * n)
        elif t == 12:
            (n,) = struct.unpack(">i", self.take(4))
            self.take(8 * n)
        else:
            raise ValueError(f"bad NBT tag {t}")


def import_region(path, lut, origin, out) -> int:
    """Adds one region file's voxels to `out` (Z, Y, X); returns the chunks read."""
    data = Path(path).read_bytes()
    X, Y, Z = WORLD
    ox, oy, oz = (int(v) for v in origin)
    read = 0
    for i in range(1024):
        loc = data[4 * i:4 * i + 4]
        off = ((loc[0] << 16) | (loc[1] << 8) | loc[2]) * 4096
        if off == 0 or loc[3] == 0 or off + 5 > len(data):
            continue
        (n,) = struct.unpack(">I", data[off:off + 4])
        if n < 1 or off + 4 + n > len(data) or data[off + 4] != 2:
            continue
        try:
            nbt = _Nbt(zlib.decompress(data[off + 5:off + 4 + n]))
            if nbt.take(1)[0] != 10:
                continue
            nbt.name()
            nbt.payload(10, "", None)
        except (zlib.error, ValueError, struct.error, IndexError):
            continue
        if nbt.x is None or nbt.z is None:
            continue
        read += 1
        by_index = {}
        for s in nbt.sections:
            if "blocks" in s:
                s.setdefault("y", 0)
                by_index[s["y"] + 128] = s          # the last section of a Y wins
        for idx in sorted(by_index):
            s = by_index[idx]
            pos = np.arange(4096)
            sy, sz, sx = pos // 256, (pos // 16) % 16, pos % 16
            voxel = s["blocks"].astype(np.int64)
            if "data" in s:
                dv = (s["data"][pos // 2] >> (4 * (pos & 1))) & 0xF
            else:
                dv = np.zeros(4096, np.int64)
            keep = dv == 0
            wx = nbt.x * 16 + sx - ox + X // 2
            wy = s["y"] * 16 + sy - oy
            wz = nbt.z * 16 + sz - oz + Z // 2
            v = lut[voxel]
            ok = keep & (v != 0) & (wx >= 0) & (wx < 384) & (wy >= 0) & (wy < 128) & (wz >= 0) & (wz < 384)
            # y-z-x order: later writes win, as in the reference's loop
            out[wz[ok], wy[ok], wx[ok]] = v[ok]
    return read


def import_world(directory, lut, origin):
    """ImportWorld (:168-186): every .mca file of the directory."""
    X, Y, Z = WORLD
    out = np.zeros((Z, Y, X), np.uint8)
    lut = np.asarray(lut, np.uint8)
    read = 0
    for p in sorted(Path(directory).iterdir()):
        if p.suffix == ".mca":
            read += import_region(p, lut, origin, out)
    return out, read
