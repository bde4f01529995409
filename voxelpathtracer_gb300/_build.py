"""Builds libvpt (CUDA, sm_103a) and the CPU oracle library.

libvpt: every translation unit under csrc/ is compiled by nvcc in parallel
(one -gencode, device code with -fmad=false and IEEE division / square root,
host code with -ffp-contract=off), then linked into voxelpathtracer_gb300/libvpt.so
with the static CUDA runtime.

Oracle (test infrastructure): oracle/*.cpp compiled by g++ with OpenMP into
oracle/_build/libvpt_oracle.so.

Both are rebuilt only when a source or header is newer than the output.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO / "include"
BUILD = PKG_DIR / "_build"
LIB = PKG_DIR / "libvpt.so"
ORACLE_DIR = REPO / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libvpt_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-O3",
    f"-I{INCLUDE}", f"-I{CSRC}",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; set NVCC or install the CUDA toolkit")


def _newer(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build_libvpt(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    sources = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    objs = []
    todo = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            todo.append((src, obj))
    nv = nvcc()

    def compile_one(item):
        src, obj = item
        cmd = [nv, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [nv, *NVCC_FLAGS, "-x", "c++", "-c", str(src), "-o", str(obj)]
        r = _run(cmd)
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(todo))) as ex:
            list(ex.map(compile_one, todo))
    if todo or _newer(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    out_dir = ORACLE_LIB.parent
    out_dir.mkdir(exist_ok=True)
    # *_ref.* files are compiled against the reference tree (oracle/build_ref.py)
    sources = sorted(p for p in ORACLE_DIR.glob("*.cpp") if not p.stem.endswith("_ref"))
    deps = sources + list(ORACLE_DIR.glob("*.h")) + [Path(__file__)]
    if _newer(ORACLE_LIB, deps):
        cxx = os.environ.get("CXX", "g++")
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               *map(str, sources), "-o", str(tmp)]
        r = _run(cmd)
        if verbose:
            sys.stderr.write(r.stderr)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_libvpt, verbose)
        b = ex.submit(build_oracle, verbose)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
