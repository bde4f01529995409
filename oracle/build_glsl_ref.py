"""Compiles functions of the reference's own shaders as C++ on the host.

TEST INFRASTRUCTURE ONLY. The shader files are read from the reference tree
(VPT_REFERENCE_DIR, else `<repo>/../reference`), turned into C++ by the
mechanical rewrites below, written to oracle/_ref/glsl_ref_gen.inc (a build
output, never committed) and compiled with oracle/glsl_compat.h (GLSL's types
and built-ins) and oracle/glsl_ref.cpp (the drivers that stand in for
the dispatches and draws) into oracle/_ref/libglsl_ref.so. A no-op where the
reference tree is absent; the tests that use the library skip then.

For each shader the top-level items (preprocessor lines, declarations,
structs, interface blocks, functions) are split, the functions reachable from
the entry point are kept, and functions on paths the drivers never take (the
alpha-tested traversal with its texture sampling, the shadow-temporal
helpers of the temporal filter) become stubs that abort.
The rewrites keep the shader's own arithmetic and operation order:
  * parameter qualifiers: `in T x` -> `T x`, `out T x` / `inout T x` -> `T& x`;
  * `uniform`, `in`, `out` and `layout(...)` globals -> namespace variables,
    a `buffer` block -> its members; `layout(...) in;` is dropped;
  * the WORLD_SIZE_* #defines -> variables the drivers set (the shaders hard
    code the reference's 384 x 128 x 384 world);
  * swizzles `.xyzw` / `.xyz` / `.xy` (and `.rgba` / `.rgb` / `.rg`) -> member
    calls, single colour components `.r .g .b .a` -> `.x .y .z .w`, and
    `v.xyz /= s;` -> the three component divisions;
  * array constructors `T[](a, b, ...)` -> brace lists, `T[n] name` -> `T name[n]`,
    a function returning `float[6]` -> the compat header's array type;
  * floating literals without a suffix -> float literals (GLSL's float).

    python oracle/build_glsl_ref.py
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("VPT_REFERENCE_DIR") or HERE.parent.parent / "reference")
SHADERS = REFERENCE / "Core" / "Shaders"
GEN = HERE / "_ref" / "glsl_ref_gen.inc"
OUT = HERE / "_ref" / "libglsl_ref.so"

# namespace, shader file, entry point, functions replaced by aborting stubs
UNITS = [
    ("df_x", "ManhattanDistanceX.comp", "main", ()),
    ("df_y", "ManhattanDistanceY.comp", "main", ()),
    ("df_z", "ManhattanDistanceZ.comp", "main", ()),
    ("primary", "InitialRayTraceFrag.glsl", "main", ("VoxelTraversalDF_AlphaTest",)),
    ("shadow", "ShadowRayTraceFrag.glsl", "main", ("VoxelTraversalDF_AlphaTest",)),
    ("pre3x3", "Spatial3x3Initial.glsl", "main", ()),
    ("variance", "SVGF/VarianceEstimate.glsl", "main", ()),
    ("atrous", "SVGF/SpatialFilter.glsl", "main", ()),
    ("temporal", "SVGF/TemporalFilter.glsl", "main", ()),
    ("plain_atrous", "AtrousSpatialFilter.glsl", "main", ()),
    ("plain_temporal", "TemporalFilter.glsl", "main", ("GetShadowSpatial", "ClipShadow")),
    # the SH / YCoCg encoding of the diffuse trace and its decoding in the colour pass
    ("sh_encode", "DiffuseRayTraceFrag.glsl", "IrridianceToSH", ()),
    ("sh_decode", "ColorPassFrag.glsl", "SHToIrridiance", ()),
    # the Hammon diffuse BRDF of the bounce rays
    ("brdf", "DiffuseRayTraceFrag.glsl", "DiffuseRayBRDF", ()),
]
WORLD_DEFINES = ("WORLD_SIZE_X", "WORLD_SIZE_Y", "WORLD_SIZE_Z")
KEYWORDS = {"if", "else", "for", "while", "return", "const", "void", "float", "int", "bool", "true", "false",
            "struct", "break", "continue", "in", "out", "inout", "uniform", "layout", "buffer", "do"}


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def split_items(src: str) -> list[str]:
    """Top-level items: preprocessor lines, `;`-terminated declarations,
    function definitions (ending at their closing brace)."""
    items, cur, depth, i, n = [], [], 0, 0, len(src)
    while i < n:
        c = src[i]
        if depth == 0 and not "".join(cur).strip() and c == "#":
            j = src.find("\n", i)
            j = n if j < 0 else j
            items.append(src[i:j].strip())
            i = j + 1
            cur = []
            continue
        cur.append(c)
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                text = "".join(cur)
                head = text[:text.index("{")]
                if "(" in head and "=" not in head and not re.match(r"\s*(struct|layout|uniform|buffer)\b", head):
                    items.append(text.strip())
                    cur = []
        elif c == ";" and depth == 0:
            items.append("".join(cur).strip())
            cur = []
        i += 1
    if "".join(cur).strip():
        items.append("".join(cur).strip())
    return [t for t in items if t]


FUNC = re.compile(r"^([\w\s]+?)\s+(\w+)\s*\((.*?)\)\s*(\{.*\}|;)$", re.S)


def classify(item: str):
    """(kind, names) of a top-level item."""
    if item.startswith("#"):
        return "pp", []
    if re.match(r"layout\s*\([^)]*\)\s*in\s*;", item):
        return "drop", []
    m = FUNC.match(item)
    if m and m.group(1).split()[-1] not in ("layout",) and "=" not in m.group(1):
        return ("func" if m.group(4).startswith("{") else "proto"), [m.group(2)]
    if re.match(r"struct\b", item):
        return "struct", [re.match(r"struct\s+(\w+)", item).group(1)]
    if re.search(r"\bbuffer\b", item) and "{" in item:
        body = item[item.index("{") + 1:item.rindex("}")]
        return "block", [d for d in re.findall(r"(\w+)\s*(?:\[[^\]]*\])?\s*;", body)]
    decl = re.sub(r"layout\s*\([^)]*\)", "", item)
    decl = re.sub(r"=.*$", "", decl, flags=re.S)
    decl = re.sub(r"\[[^\]]*\]", "", decl)
    return "global", [re.findall(r"\w+", decl)[-1]]


def rewrite_params(params: str) -> str:
    out = []
    for p in [q.strip() for q in params.split(",")] if params.strip() else []:
        m = re.match(r"(?:const\s+)?(?:(in|out|inout)\s+)?(\w+)\s+(\w+)(\s*\[[^\]]*\])?$", p)
        if not m:
            raise ValueError(f"parameter not understood: {p!r}")
        qual, ty, name, arr = m.group(1), m.group(2), m.group(3), m.group(4) or ""
        ty = "unsigned" if ty == "uint" else ty
        out.append(f"{ty}& {name}{arr}" if qual in ("out", "inout") else f"{ty} {name}{arr}")
    return ", ".join(out)


def rewrite_array_ctors(text: str) -> str:
    while True:
        m = re.search(r"\b\w+\s*\[\s*\d*\s*\]\s*\(", text)
        if not m:
            return text
        start, depth, k = m.end() - 1, 0, m.end() - 1
        while True:
            if text[k] == "(":
                depth += 1
            elif text[k] == ")":
                depth -= 1
                if depth == 0:
                    break
            k += 1
        text = text[:m.start()] + "{" + text[start + 1:k] + "}" + text[k + 1:]


def rewrite_expr(text: str) -> str:
    # GLSL's `T[n] name = ...` array declarations -> `T name[n] = ...`
    text = re.sub(r"\b(\w+)\s*\[\s*(\d+)\s*\]\s+(\w+)\s*=", r"\1 \3[\2] =", text)
    text = rewrite_array_ctors(text)
    # a swizzle assigned through `/=`: each component divided by the value read once
    text = re.sub(r"\b(\w+)\.xyz\s*/=\s*([^;]+);",
                  lambda m: (f"{{ const float d_ = {m.group(2)}; {m.group(1)}.x /= d_; {m.group(1)}.y /= d_; "
                             f"{m.group(1)}.z /= d_; }}"), text)
    swz = {"xyzw": "xyzw", "rgba": "xyzw", "xyz": "xyz", "rgb": "xyz", "xy": "xy", "rg": "xy"}
    text = re.sub(r"\.(xyzw|rgba|xyz|rgb|xy|rg)\b(?!\s*\()", lambda m: f".{swz[m.group(1)]}()", text)
    comp = {"r": "x", "g": "y", "b": "z", "a": "w"}
    text = re.sub(r"(?<=[\w\)\]])\.([rgba])\b(?!\s*\()", lambda m: "." + comp[m.group(1)], text)
    text = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])",
                  lambda m: m.group(1) + "f", text)
    return re.sub(r"\buint\b", "unsigned", text)


def rewrite_item(kind: str, item: str, stub: bool = False) -> str:
    if kind in ("func", "proto"):
        m = FUNC.match(item)
        head = f"{m.group(1).strip()} {m.group(2)}({rewrite_params(m.group(3))})"
        if kind == "proto":
            return rewrite_expr(head) + ";"
        if stub:
            return head + " { std::abort(); }"
        return rewrite_expr(head + " " + m.group(4))
    if kind == "struct":
        return rewrite_expr(item) + ("" if item.endswith(";") else ";")
    if kind == "block":
        body = item[item.index("{") + 1:item.rindex("}")]
        return rewrite_expr(body.strip())
    text = re.sub(r"layout\s*\([^)]*\)\s*", "", item)
    text = re.sub(r"^\s*(uniform|in|out|flat|highp|mediump|lowp)\s+", "", text)
    text = re.sub(r"^\s*(uniform|in|out)\s+", "", text)
    return rewrite_expr(text) + ("" if text.rstrip().endswith(";") else ";")


def translate(ns: str, path: Path, entry: str, stubs) -> str:
    # functions returning arrays (`float[6] F(...)`) return the compat header's array type
    items = [re.sub(r"^(\w+)\s*\[(\d+)\]\s+(\w+\s*\()", r"arr_\1_\2 \3", t)
             for t in split_items(strip_comments(path.read_text()))]
    cls = [classify(t) for t in items]
    by_name = {}
    for k, (kind, names) in enumerate(cls):
        for nm in names:
            by_name.setdefault(nm, []).append(k)
    keep, work = set(), [entry]
    while work:
        nm = work.pop()
        for k in by_name.get(nm, []):
            if k in keep:
                continue
            keep.add(k)
            kind, names = cls[k]
            if kind == "func" and names[0] in stubs:
                continue
            for ident in set(re.findall(r"\b[A-Za-z_]\w*\b", items[k])) - KEYWORDS - {nm}:
                if ident in by_name:
                    work.append(ident)
    out = [f"namespace {ns} {{", "int WORLD_SIZE_X = 0, WORLD_SIZE_Y = 0, WORLD_SIZE_Z = 0;",
           "uvec3 gl_GlobalInvocationID;", "vec4 gl_FragCoord;"]
    for k, item in enumerate(items):
        kind, names = cls[k]
        if kind == "pp":
            if item.startswith("#version") or item.startswith("#extension"):
                continue
            if any(re.match(rf"#define\s+{d}\b", item) for d in WORLD_DEFINES):
                continue
            out.append(rewrite_expr(item) if item.startswith("#define") else item)
        elif k in keep and kind != "drop":
            out.append(rewrite_item(kind, item, stub=kind == "func" and names[0] in stubs))
    out.append(f"}}  // namespace {ns}")
    return "\n".join(out) + "\n"


def build(verbose: bool = False) -> Path | None:
    if not SHADERS.is_dir():
        return None
    sources = [SHADERS / f for _, f, _, _ in UNITS]
    if not all(p.exists() for p in sources):
        return None
    deps = sources + [HERE / "glsl_compat.h", HERE / "glsl_ref.cpp", HERE / "omath.h", Path(__file__)]
    if OUT.exists() and all(OUT.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    gen = ["// generated by oracle/build_glsl_ref.py from the reference's shaders; not part of the repository"]
    for ns, f, entry, stubs in UNITS:
        gen.append(translate(ns, SHADERS / f, entry, set(stubs)))
    GEN.write_text("\n".join(gen))
    tmp = OUT.with_suffix(".so.tmp")
    # -fwrapv: GLSL's integer arithmetic wraps (the shaders' hash seeds overflow)
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fwrapv", "-fPIC",
           "-shared", "-w", f"-I{HERE}", f"-I{GEN.parent}", str(HERE / "glsl_ref.cpp"), "-o", str(tmp)]
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
