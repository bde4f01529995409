"""Builds the parts of the reference that compile standalone into oracle/_ref/:
libenkimi_ref.so, the reference's own Minecraft region / NBT reader (enkiMI
and miniz, compiled from the sources where they lie in the reference tree)
with the driver oracle/enkimi_ref.c, libglm_ref.so, the reference's
vendored glm (header-only) behind oracle/glm_ref.cpp, and libglsl_ref.so, the
reference's own shaders compiled as C++ (oracle/build_glsl_ref.py). TEST INFRASTRUCTURE; a
no-op when the reference tree is absent (the tests that need the libraries
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
GLM = REFERENCE / "Dependencies" / "glm"
OUT = HERE / "_ref" / "libenkimi_ref.so"
OUT_GLM = HERE / "_ref" / "libglm_ref.so"


def _compile(cmd_head, sources, deps, out, verbose):
    if out.exists() and all(out.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return out
    out.parent.mkdir(exist_ok=True)
    tmp = out.with_suffix(".so.tmp")
    r = subprocess.run([*cmd_head, *map(str, sources), "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr)
        return None
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(tmp, out)
    return out


def build_glm(verbose: bool = False) -> Path | None:
    """oracle/glm_ref.cpp against the reference's glm, with the oracle's
    floating-point flags (no contraction, no fast math)."""
    if not (GLM / "glm" / "glm.hpp").exists():
        return None
    src = HERE / "glm_ref.cpp"
    head = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
            "-shared", "-w", f"-I{GLM}"]
    return _compile(head, [src], [src], OUT_GLM, verbose)


def build(verbose: bool = False) -> Path | None:
    build_glm(verbose)
    # the reference's shaders compiled as C++ (oracle/build_glsl_ref.py)
    import importlib.util
    spec = importlib.util.spec_from_file_location("vpt_build_glsl_ref", HERE / "build_glsl_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build(verbose)
    sources = [ENKI / "enkimi.c", ENKI / "miniz.c", HERE / "enkimi_ref.c"]
    if not all(p.exists() for p in sources[:2]):
        return None
    head = [os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-w", f"-I{ENKI}"]
    return _compile(head, sources, sources, OUT, verbose)


if __name__ == "__main__":
    print(build(verbose=True))
