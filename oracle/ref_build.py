"""Builds oracle/_ref/libref.so from the reference's own sources (test
infrastructure only; nothing of the product path loads it).

What is compiled, straight from the reference checkout:
- the compute shaders of the path (shaders/glsl/WaveFrontPathTracer/:
  initSeeds, raygenPrimary, computeMortonCodesAila32, reorderRays,
  raygenShadow, raygenPath + geometrytypes.glsl, reconstructSmooth,
  reconstructShadow, countRayHits, interpolateColors; ray.glsl), as C++
  against oracle/glsl_shim.hpp.  Only declarations are rewritten, by the
  regular expressions below: #version/#extension lines dropped, #include
  of .glsl files inlined, buffer_reference blocks turned into
  GLSL_BUFFER_ARRAY/GLSL_BUFFER_SCALAR structs, the push-constant block
  into a struct variable `pc`, `shared` into a static array, `main` into
  `shader_main`, inout/out parameters into references, float literals given
  the `f` suffix (GLSL literals without a suffix are float).  Function
  bodies are compiled as they are.
- the body of PixelTable::recalculate that builds the two lookup tables
  (projects/WaveFrontPathTracer/Ray/PixelTable.cpp:39-99), spliced into a
  function of oracle/ref_entries.cpp;
- the camera header base/camera.hpp, unchanged, against the glm stand-in
  in oracle/glm_shim (glm is an empty submodule in the reference).

Not compiled: trace.comp (rayQuery traversal is done by the Vulkan driver),
the radix sort (shipped only as SPIR-V), everything that needs a Vulkan
device.  Outputs go to oracle/_ref/ only: generated sources under gen/ and
libref.so.  Needs the reference checkout (REFERENCE_ROOT, default
/root/reference); without it build() raises FileNotFoundError.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libref.so"
REF = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))
SHADERS = Path("shaders/glsl/WaveFrontPathTracer")
PIXEL_TABLE = Path("projects/WaveFrontPathTracer/Ray/PixelTable.cpp")
CAMERA_DIR = Path("base")

# (generated name, shader file)
SHADER_LIST = [
    ("initSeeds", "initSeeds.comp"),
    ("raygenPrimary", "raygenPrimary.comp"),
    ("mortonAila32", "computeMortonCodesAila32.comp"),
    ("reorderRays", "reorderRays.comp"),
    ("raygenShadow", "raygenShadow.comp"),
    ("raygenPath", "raygenPath.comp"),
    ("reconstructSmooth", "reconstructSmooth.comp"),
    ("reconstructShadow", "reconstructShadow.comp"),
    ("countRayHits", "countRayHits.comp"),
    ("interpolateColors", "interpolateColors.comp"),
]

# PixelTable.cpp lines 39..99 (1-based, inclusive) with the text expected on
# the first and last lines, so that a changed file is noticed.
PIXEL_TABLE_LINES = (39, 99)
PIXEL_TABLE_ANCHORS = ("// Smart mode.", "}")

_BUFFER = re.compile(
    r"layout\s*\(\s*buffer_reference[^)]*\)\s*(?:(?:readonly|writeonly|restrict|coherent|volatile)\s+)*"
    r"buffer\s+(?:(?:readonly|writeonly|restrict|coherent|volatile)\s+)*(\w+)\s*"
    r"\{\s*(\w+)\s+(\w+)\s*(\[\s*\])?\s*;\s*\}\s*;")
_PUSH = re.compile(r"layout\s*\(\s*push_constant\s*\)\s*uniform\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", re.S)
_LOCAL = re.compile(r"layout\s*\(\s*local_size_x\s*=\s*(\w+)\s*\)\s*in\s*;")
_INCLUDE = re.compile(r'^\s*#include\s+"([^"]+\.glsl)"\s*$', re.M)
_FLOAT = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
_PARAM_REF = re.compile(r"\b(inout|out)\s+(\w+)\s+(\w+)")
_DEFINE = re.compile(r"^\s*#define\s+(\w+)", re.M)


def _read(p: Path) -> str:
    return p.read_text(encoding="utf-8-sig")


def _inline_includes(text: str, base: Path, seen: set[str]) -> str:
    def sub(m):
        name = m.group(1)
        if name in seen:
            return ""
        seen.add(name)
        return _inline_includes(_read(base / name), base, seen)
    return _INCLUDE.sub(sub, text)


def translate_shader(src: Path) -> str:
    """GLSL compute shader text -> C++ text for oracle/glsl_shim.hpp."""
    text = _inline_includes(_read(src), src.parent, set())
    text = "\n".join(line for line in text.split("\n")
                     if not re.match(r"\s*#\s*(version|extension)\b", line))
    n_buf = len(_BUFFER.findall(text))
    text = _BUFFER.sub(lambda m: ("GLSL_BUFFER_ARRAY" if m.group(4) else "GLSL_BUFFER_SCALAR")
                       + f"({m.group(1)}, {m.group(2)}, {m.group(3)});", text)
    text, n_push = _PUSH.subn(lambda m: f"struct {m.group(1)} {{{m.group(2)}}};\nstatic {m.group(1)} {m.group(3)};", text)
    text, n_local = _LOCAL.subn(lambda m: f"static const unsigned kLocalSizeX = {m.group(1)};", text)
    text = re.sub(r"^(\s*)shared\s+", r"\1static ", text, flags=re.M)
    text, n_main = re.subn(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", text)
    text = _PARAM_REF.sub(r"\2& \3", text)
    text = _FLOAT.sub(lambda m: m.group(1) + "f", text)
    code = re.sub(r"//[^\n]*|/\*.*?\*/", "", text, flags=re.S)
    if "layout" in code or n_push != 1 or n_local != 1 or n_main != 1 or n_buf == 0:
        raise RuntimeError(f"{src.name}: unexpected declarations (buffers {n_buf}, push {n_push}, "
                           f"local size {n_local}, main {n_main}, layout left: {'layout' in code})")
    fibers = "subgroup" in code or "barrier(" in code
    names = sorted(set(_DEFINE.findall(text)))
    undef = "".join(f"#undef {n}\n" for n in names)
    head = f"// Generated by oracle/ref_build.py from {src.name}; do not edit.\n{undef}"
    tail = f"\nstatic const bool kUsesFibers = {'true' if fibers else 'false'};\n{undef}"
    return head + text + tail


def pixel_table_body(src: Path) -> str:
    lines = _read(src).split("\n")
    a, b = PIXEL_TABLE_LINES
    body = lines[a - 1:b]
    if body[0].strip() != PIXEL_TABLE_ANCHORS[0] or body[-1].strip() != PIXEL_TABLE_ANCHORS[1]:
        raise RuntimeError(f"{src}: lines {a}-{b} are not the lookup-table loops this recipe expects")
    return f"// Generated by oracle/ref_build.py from {src.name}:{a}-{b}; do not edit.\n" + "\n".join(body) + "\n"


def _stale(deps: list[Path]) -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False) -> Path:
    if not (REF / SHADERS).is_dir():
        raise FileNotFoundError(f"reference checkout not found at {REF}")
    own = [HERE / "ref_build.py", HERE / "ref_entries.cpp", HERE / "glsl_shim.hpp",
           *sorted((HERE / "glm_shim").rglob("*.hpp"))]
    srcs = [REF / SHADERS / f for _, f in SHADER_LIST] + [REF / SHADERS / "ray.glsl",
                                                          REF / SHADERS / "geometrytypes.glsl",
                                                          REF / PIXEL_TABLE, REF / CAMERA_DIR / "camera.hpp"]
    if not force and not _stale(own + srcs):
        return LIB
    GEN.mkdir(parents=True, exist_ok=True)
    for name, f in SHADER_LIST:
        (GEN / f"{name}.inc").write_text(translate_shader(REF / SHADERS / f))
    (GEN / "pixel_table_body.inc").write_text(pixel_table_body(REF / PIXEL_TABLE))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-I", str(HERE), "-I", str(OUT), "-I", str(HERE / "glm_shim"), "-I", str(REF / CAMERA_DIR),
           str(HERE / "ref_entries.cpp"), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference build failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
