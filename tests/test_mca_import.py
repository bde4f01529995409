"""The Minecraft region import (Core/NBT/Importer.cpp through enkiMI) of
vpt_import_mca_world against the Python restatement (oracle/mca.py) and, when
it was built here, against the reference's own region / NBT reader
(oracle/_ref/libenkimi_ref.so). Region files are written by the test: the
reference's sample worlds are not part of its tree."""
import ctypes as C
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

REF_LIB = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "libenkimi_ref.so"


# ------------------------------------------------------------ NBT writer --
def _name(s):
    b = s.encode()
    return struct.pack(">H", len(b)) + b


def tag(t, name, payload):
    return bytes([t]) + _name(name) + payload


def compound(fields):
    return b"".join(fields) + b"\x00"


def byte_array(a):
    a = np.ascontiguousarray(a, np.uint8)
    return struct.pack(">i", a.size) + a.tobytes()


def chunk_nbt(cx, cz, sections, y_as_int=False, extra=True):
    secs = []
    for y, blocks, data in sections:
        f = [tag(3, "Y", struct.pack(">i", y)) if y_as_int else tag(1, "Y", struct.pack(">b", y)),
             tag(7, "Blocks", byte_array(blocks))]
        if data is not None:
            f.append(tag(7, "Data", byte_array(data)))
        if extra:
            f.append(tag(7, "SkyLight", byte_array(np.full(2048, 0xFF, np.uint8))))
        secs.append(compound(f))
    level = [tag(3, "xPos", struct.pack(">i", cx)), tag(3, "zPos", struct.pack(">i", cz))]
    if extra:
        level += [tag(4, "LastUpdate", struct.pack(">q", 123456)), tag(8, "Status", _name("postprocessed")),
                  tag(11, "HeightMap", struct.pack(">i", 256) + np.zeros(256, ">i4").tobytes()),
                  tag(9, "Entities", bytes([10]) + struct.pack(">i", 0))]
    level.append(tag(9, "Sections", bytes([10]) + struct.pack(">i", len(secs)) + b"".join(secs)))
    root = [tag(10, "Level", compound(level))]
    if extra:
        root.insert(0, tag(3, "DataVersion", struct.pack(">i", 1343)))
    return tag(10, "", compound(root))


def write_region(path, chunks, level=6, corrupt=()):
    """chunks: {slot: nbt bytes}; corrupt: slots whose zlib data is damaged."""
    header = bytearray(8192)
    body = bytearray()
    sector = 2
    for slot, nbt in sorted(chunks.items()):
        z = bytearray(zlib.compress(nbt, level))
        if slot in corrupt:
            z[-1] ^= 0x5A                      # breaks the Adler-32
        data = struct.pack(">I", len(z) + 1) + bytes([2]) + bytes(z)
        data += b"\0" * (-len(data) % 4096)
        n = len(data) // 4096
        header[4 * slot:4 * slot + 4] = bytes([(sector >> 16) & 255, (sector >> 8) & 255, sector & 255, n])
        body += data
        sector += n
    Path(path).write_bytes(bytes(header) + bytes(body))


def random_sections(rng, ys, data_prob=0.3):
    out = []
    for y in ys:
        blocks = rng.integers(0, 200, 4096).astype(np.uint8)
        blocks[rng.random(4096) < 0.4] = 0
        data = None
        if rng.random() < 0.8:
            nib = (rng.random(4096) < data_prob) * rng.integers(1, 16, 4096)
            data = (nib[0::2] | (nib[1::2] << 4)).astype(np.uint8)
        out.append((y, blocks, data))
    return out


def region_dir(tmp_path, rng, n_regions=2, level=6, corrupt=(), y_as_int=False):
    d = tmp_path / "region"
    d.mkdir()
    for r in range(n_regions):
        chunks = {}
        for slot in rng.choice(1024, 6, replace=False):
            cx, cz = int(rng.integers(-14, 14)), int(rng.integers(-14, 14))
            ys = sorted(rng.choice(np.arange(-1, 9), 3, replace=False).tolist())
            chunks[int(slot)] = chunk_nbt(cx, cz, random_sections(rng, ys), y_as_int=y_as_int)
        write_region(d / f"r.{r}.0.mca", chunks, level=level, corrupt=corrupt if r == 0 else ())
    (d / "notes.txt").write_text("not a region file")
    return d


# ------------------------------------------------------------------ tests --
@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_import_matches_restatement(vpt, tmp_path, level):
    """Every zlib block type (stored at level 0, fixed and dynamic Huffman
    codes above), a random Minecraft-id table and a fractional origin."""
    from oracle import mca
    rng = np.random.default_rng(level)
    d = region_dir(tmp_path, rng, level=level)
    lut = rng.integers(0, 100, 256).astype(np.uint8)
    lut[0] = 0
    origin = (10.7, 3.2, -20.9)
    got, n = vpt.import_mca_world(d, lut, origin)
    ref, n_ref = mca.import_world(d, lut, origin)
    assert n == n_ref == 12
    assert got.shape == (384, 128, 384) and (got > 0).sum() > 10000
    assert np.array_equal(got, ref)


def test_import_int_y_and_duplicate_sections(vpt, tmp_path):
    from oracle import mca
    rng = np.random.default_rng(5)
    d = tmp_path / "region"
    d.mkdir()
    secs = random_sections(rng, [2, 3]) + random_sections(rng, [2])     # Y 2 twice: the last wins
    write_region(d / "r.0.0.mca", {7: chunk_nbt(1, -2, secs, y_as_int=True, extra=False)})
    got, n = vpt.import_mca_world(d)
    ref, n_ref = mca.import_world(d, np.arange(256), (0, 0, 0))
    assert n == n_ref == 1 and np.array_equal(got, ref)


def test_import_skips_damaged_chunks(vpt, tmp_path):
    """Two of six chunks with a broken Adler-32 are skipped; the others import."""
    from oracle import mca
    d2 = tmp_path / "damaged"
    d2.mkdir()
    rng = np.random.default_rng(11)
    chunks = {}
    for slot in rng.choice(1024, 6, replace=False):
        cx, cz = int(rng.integers(-14, 14)), int(rng.integers(-14, 14))
        ys = sorted(rng.choice(np.arange(-1, 9), 3, replace=False).tolist())
        chunks[int(slot)] = chunk_nbt(cx, cz, random_sections(rng, ys))
    bad = sorted(chunks)[:2]
    write_region(d2 / "r.0.0.mca", chunks, corrupt=bad)
    got, n = vpt.import_mca_world(d2)
    ref, n_ref = mca.import_world(d2, np.arange(256), (0, 0, 0))
    assert n == n_ref == 4 and np.array_equal(got, ref)


def test_import_rejects_bad_arguments(vpt, tmp_path):
    with pytest.raises(vpt.VPTError):
        vpt.import_mca_world(tmp_path / "missing")
    d = tmp_path / "short"
    d.mkdir()
    (d / "r.0.0.mca").write_bytes(b"\0" * 100)                       # shorter than the header
    with pytest.raises(vpt.VPTError):
        vpt.import_mca_world(d)
    out = np.zeros(10, np.uint8)
    assert vpt.lib.vpt_import_mca_world(str(tmp_path).encode(), np.zeros(256, np.uint8).ctypes.data,
                                        (C.c_float * 3)(), out.ctypes.data, out.nbytes, None) == vpt.ERR_INVALID_ARG


@pytest.mark.skipif(not REF_LIB.exists(), reason="the reference's region reader was not built here")
@pytest.mark.parametrize("level", [0, 6])
def test_import_matches_reference_reader(vpt, tmp_path, level):
    """The same files through the reference's own enkiMI reader driven as
    Importer.cpp drives it."""
    lib = C.CDLL(str(REF_LIB))
    lib.ref_import_region.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(100 + level)
    d = region_dir(tmp_path, rng, level=level)
    lut = rng.integers(0, 100, 256).astype(np.uint8)
    lut[0] = 0
    origin = (-33.5, 7.9, 41.2)
    got, _ = vpt.import_mca_world(d, lut, origin)
    ref = np.zeros((384, 128, 384), np.uint8)
    org = (C.c_int * 3)(*[int(v) for v in origin])
    for p in sorted(d.glob("*.mca")):
        assert lib.ref_import_region(str(p).encode(), lut.ctypes.data, org, ref.ctypes.data) == 6
    assert np.array_equal(got, ref)
