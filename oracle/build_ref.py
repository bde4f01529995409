"""Builds oracle/_ref/libenkimi_ref.so: the reference's own Minecraft region /
NBT reader (enkiMI and miniz, compiled from the sources where they lie in the
reference tree) with the driver oracle/enkimi_ref.c. TEST INFRASTRUCTURE; a
no-op when the reference tree is absent (the tests that need the library
skip then).

The reference tree is taken from the environment variable VPT_REFERENCE_DIR,
else from the directory `reference` beside this repository's own directory
(`<repo>/../reference`).

    python oracle/build_ref.py
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("VPT_REFERENCE_DIR") or HERE.parent.parent / "reference")
ENKI = REFERENCE / "Dependencies" / "enkiMI"
OUT = HERE / "_ref" / "libenkimi_ref.so"


def build(verbose: bool = False) -> Path | None:
    sources = [ENKI / "enkimi.c", ENKI / "miniz.c", HERE / "enkimi_ref.c"]
    if not all(p.exists() for p in sources[:2]):
        return None
    if OUT.exists() and all(OUT.stat().st_mtime >= p.stat().st_mtime for p in sources):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-w", f"-I{ENKI}", *map(str, sources), "-o",
           str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr)
        return None
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
