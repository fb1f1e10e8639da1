"""Command-line front end: the reference's env.json options, scene loading
and benchmark output, rendering through the C ABI renderer.

Mirrors Environment/AppEnvironment.cpp:10-43 (every registered option with
its default), the JSON key lookup of Environment.cpp (dotted keys in nested
objects, vectors as "x y z" strings), Benchmark::run
(Benchmark/Benchmark.cpp:84-208: warm-up cycles, averaged counts, times and
Mrays/s, the results block) and replaces the window / present.comp with a
headless image file (PFM float or PPM 8-bit).

Options beyond the reference (same file, same style):
  Renderer.bvh            "bvh2" | "bvh8"              (default "bvh8")
  Renderer.mortonKind     "aila32" | "6d48" | "6d64"   (default "aila32")
  Renderer.albedo         float                        (default 0.8)
  Renderer.useGraph       bool                         (default true)
  Renderer.pathSortSkip   int bit mask: bit b set = bounce b+1 traces its
                          path rays unsorted (per-bounce reordering, default 0)
  Renderer.primaryBvh     "bvh2" | "bvh8" | "" (default: Renderer.bvh): BVH of the
                          primary pass (camera rays and their shadow rays)
  Renderer.shadowOverlap  bool: trace each pass's shadow rays concurrently with
                          the next bounce (default true; same image)
  Renderer.accumulateFp64 bool: keep the running mean over frames in double
                          (default false: float, as interpolateColors.comp)
  Benchmark.stageTimes    bool (default true): in benchmark mode, time every
                          stage with CUDA events (the frame is launched
                          directly on one stream), which gives the TRACE
                          times, RT PERF per ray type (rays / trace time, as
                          the reference) and the SORT LOG; false: graph
                          replay and overlap as configured, RENDER KERNELS
                          only
  Benchmark.warmupCycles  int                          (default 3)
  Benchmark.benchmarkCycles int                        (default 10)
  Scene.generator         "soup:<triangles>:<seed>" | "courtyard[:<seed>]" |
                          "city[:<seed>]" | "city:<triangles>:<seed>" -- a
                          seeded synthetic scene instead of Scene.filename
  Output.image            path of a .pfm or .ppm file for the last frame

Usage: python -m vulkanwavefrontpathtracer_gb300.app --env env.json [--out image.pfm]
"""
from __future__ import annotations

import argparse
import base64
import json
import struct
import sys
import time
from pathlib import Path
from typing import Any, Dict, List, Tuple

import numpy as np

# AppEnvironment::registerOptions (AppEnvironment.cpp:10-43) + the options
# above, with their defaults.
DEFAULTS: Dict[str, Any] = {
    "Application.mode": "interactive",
    "Benchmark.printSortLogs": False,
    "Benchmark.warmupCycles": 3,
    "Benchmark.benchmarkCycles": 10,
    "Benchmark.stageTimes": True,
    "Resolution.width": 1024,
    "Resolution.height": 768,
    "Scene.filename": "",
    "Scene.generator": "",
    "Scene.light": [5.0, -2.0, 1.0],
    "Scene.backgroundcolor": [0.0, 0.0, 1.0],
    "Scene.headlight": False,
    "Renderer.numberOfPrimarySamples": 1,
    "Renderer.numberOfShadowSamples": 2,
    "Renderer.shadowRadius": 0.001,
    "Renderer.rayType": "primary",
    "Renderer.recursionDepth": 1,
    "Renderer.keyValue": 0.6,
    "Renderer.whitePoint": 2.0,
    "Renderer.russianRoulette": False,
    "Renderer.sortShadowRays": False,
    "Renderer.reorderShadowRays": False,
    "Renderer.sortPathRays": False,
    "Renderer.reorderPathRays": False,
    "Renderer.bvh": "bvh8",
    "Renderer.mortonKind": "aila32",
    "Renderer.albedo": 0.8,
    "Renderer.useGraph": True,
    "Renderer.pathSortSkip": 0,
    "Renderer.shadowOverlap": True,
    "Renderer.primaryBvh": "",
    "Renderer.accumulateFp64": False,
    "Camera.position": [0.0, 0.0, 0.0],
    "Camera.rotation": [0.0, 0.0, 0.0],
    "Camera.nearPlane": 0.001,
    "Camera.farPlane": 3.0,
    "Camera.fieldOfView": 45.0,
    "Output.image": "",
}

RAY_TYPES = {"primary": 0, "shadow": 1, "path": 2}
MORTON_KINDS = {"aila32": 0, "6d48": 1, "6d64": 2}
BVH_KINDS = {"bvh2": 0, "bvh8": 1}


def _lookup(data: dict, key: str):
    cur = data
    for seg in key.split("."):
        if not isinstance(cur, dict) or seg not in cur:
            return None
        cur = cur[seg]
    return cur


def _as(default, value, key):
    if isinstance(default, bool):
        if isinstance(value, str):
            if value.lower() in ("1", "true", "yes", "on"):
                return True
            if value.lower() in ("0", "false", "no", "off"):
                return False
            raise ValueError(f"{key}: not a bool: {value!r}")
        return bool(value)
    if isinstance(default, int):
        return int(value)
    if isinstance(default, float):
        return float(value)
    if isinstance(default, list):
        v = [float(x) for x in (value.split() if isinstance(value, str) else value)]
        if len(v) != 3:
            raise ValueError(f"{key}: expected 3 components, got {value!r}")
        return v
    return str(value)


def load_env(source) -> Dict[str, Any]:
    """Options from an env.json path, JSON text or dict; missing keys take
    the registered defaults, unknown keys are reported."""
    if isinstance(source, dict):
        data = source
    else:
        p = Path(source)
        data = json.loads(p.read_text() if p.exists() else str(source))
    opts = {}
    for key, default in DEFAULTS.items():
        v = _lookup(data, key)
        opts[key] = default if v is None else _as(default, v, key)
    known_sections = {k.split(".")[0] for k in DEFAULTS}
    unknown = []
    for sec, body in data.items():
        if sec not in known_sections or not isinstance(body, dict):
            unknown.append(sec)
            continue
        unknown += [f"{sec}.{k}" for k in body if f"{sec}.{k}" not in DEFAULTS]
    if unknown:
        raise ValueError(f"unknown options: {', '.join(sorted(unknown))}")
    for key, table in (("Renderer.rayType", RAY_TYPES), ("Renderer.mortonKind", MORTON_KINDS),
                       ("Renderer.bvh", BVH_KINDS), ("Renderer.primaryBvh", dict(BVH_KINDS, **{"": -1}))):
        if opts[key] not in table:
            raise ValueError(f"{key} must be one of {sorted(table)}")
    return opts


def renderer_config(opts: Dict[str, Any]):
    from . import api
    return api.default_config(
        ray_type=RAY_TYPES[opts["Renderer.rayType"]],
        num_primary_samples=opts["Renderer.numberOfPrimarySamples"],
        num_shadow_samples=opts["Renderer.numberOfShadowSamples"],
        shadow_radius=opts["Renderer.shadowRadius"],
        recursion_depth=opts["Renderer.recursionDepth"],
        key_value=opts["Renderer.keyValue"],
        white_point=opts["Renderer.whitePoint"],
        russian_roulette=1 if opts["Renderer.russianRoulette"] else 0,
        sort_shadow_rays=1 if opts["Renderer.sortShadowRays"] else 0,
        reorder_shadow_rays=1 if opts["Renderer.reorderShadowRays"] else 0,
        sort_path_rays=1 if opts["Renderer.sortPathRays"] else 0,
        reorder_path_rays=1 if opts["Renderer.reorderPathRays"] else 0,
        morton_kind=MORTON_KINDS[opts["Renderer.mortonKind"]],
        bvh_kind=BVH_KINDS[opts["Renderer.bvh"]],
        albedo=opts["Renderer.albedo"],
        use_graph=1 if opts["Renderer.useGraph"] else 0,
        path_sort_skip=opts["Renderer.pathSortSkip"],
        shadow_overlap=1 if opts["Renderer.shadowOverlap"] else 0,
        primary_bvh_kind=-1 if opts["Renderer.primaryBvh"] == "" else BVH_KINDS[opts["Renderer.primaryBvh"]],
        timing=1 if opts["Application.mode"] == "benchmark" and opts["Benchmark.stageTimes"] else 0,
        accumulate_fp64=1 if opts["Renderer.accumulateFp64"] else 0)


# ------------------------------------------------------------ scene input
_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}


def load_gltf(path) -> Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Triangles of a glTF 2.0 file (.gltf with external or data-URI
    buffers): positions [V,3], normals [V,3], indices [T,3] and the first
    triangle of each primitive (one reference Geometry per primitive, as
    vkglTF::Model feeds the BLAS, WaveFrontPathTracer.cpp:202-271).  Node
    transforms are not applied: the reference shades with object-space
    normals and builds one BLAS over the untransformed primitives."""
    path = Path(path)
    doc = json.loads(path.read_text())
    buffers = []
    for b in doc.get("buffers", []):
        uri = b["uri"]
        if uri.startswith("data:"):
            buffers.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            buffers.append((path.parent / uri).read_bytes())

    def accessor(i):
        a = doc["accessors"][i]
        view = doc["bufferViews"][a["bufferView"]]
        dt = np.dtype(_COMPONENT[a["componentType"]])
        nc = _NCOMP[a["type"]]
        stride = view.get("byteStride", 0) or dt.itemsize * nc
        start = view.get("byteOffset", 0) + a.get("byteOffset", 0)
        raw = buffers[view["buffer"]]
        out = np.empty((a["count"], nc), dt)
        for r in range(a["count"]):
            out[r] = np.frombuffer(raw, dt, nc, start + r * stride)
        return out

    pos_l, nrm_l, idx_l, first = [], [], [], []
    nv = nt = 0
    for mesh in doc.get("meshes", []):
        for prim in mesh["primitives"]:
            if prim.get("mode", 4) != 4:
                continue  # triangles only
            p = accessor(prim["attributes"]["POSITION"]).astype(np.float32)
            if "NORMAL" in prim["attributes"]:
                n = accessor(prim["attributes"]["NORMAL"]).astype(np.float32)
            else:
                n = np.zeros_like(p)
            if "indices" in prim:
                ix = accessor(prim["indices"]).astype(np.uint32).reshape(-1, 3)
            else:
                ix = np.arange(p.shape[0], dtype=np.uint32).reshape(-1, 3)
            first.append(nt)
            pos_l.append(p)
            nrm_l.append(n)
            idx_l.append(ix + nv)
            nv += p.shape[0]
            nt += ix.shape[0]
    if not pos_l:
        raise ValueError(f"{path}: no triangle primitives")
    return (np.concatenate(pos_l), np.concatenate(nrm_l), np.concatenate(idx_l),
            np.array(first, dtype=np.uint32))


def load_scene(opts: Dict[str, Any]):
    """(positions, normals, indices, geometry_first) from Scene.generator or
    Scene.filename."""
    from . import api
    gen = opts["Scene.generator"]
    if gen:
        parts = gen.split(":")
        name = parts[0]
        if name == "soup":
            ntris = int(parts[1]) if len(parts) > 1 else 65536
            seed = int(parts[2]) if len(parts) > 2 else 1
            pos, nrm, idx = api.generate_scene(0, seed, ntris)
        elif name == "courtyard":
            pos, nrm, idx = api.generate_scene(1, int(parts[1]) if len(parts) > 1 else 1)
        elif name == "city" and len(parts) == 3:
            pos, nrm, idx = api.generate_scene(3, int(parts[2]), int(parts[1]))
        elif name == "city":
            pos, nrm, idx = api.generate_scene(2, int(parts[1]) if len(parts) > 1 else 1)
        else:
            raise ValueError(f"unknown Scene.generator {gen!r}")
        return pos, nrm, idx, np.zeros(1, np.uint32)
    if opts["Scene.filename"]:
        return load_gltf(opts["Scene.filename"])
    raise ValueError("set Scene.filename or Scene.generator")


# ------------------------------------------------------------ image output
def write_pfm(path, rgb: np.ndarray) -> None:
    """Portable float map, 3 channels, little endian; rows bottom to top."""
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(rgb[::-1], dtype="<f4").tobytes())


def read_pfm(path) -> np.ndarray:
    data = Path(path).read_bytes()
    header, rest = data.split(b"\n", 1)
    dims, rest = rest.split(b"\n", 1)
    scale, rest = rest.split(b"\n", 1)
    w, h = map(int, dims.split())
    dt = "<f4" if float(scale) < 0 else ">f4"
    return np.frombuffer(rest, dt).reshape(h, w, 3)[::-1]


def write_ppm(path, rgb: np.ndarray) -> None:
    """8-bit binary PPM of clamped [0, 1] values; NaN (the reference's 0/0
    tone map of black pixels) writes as 0."""
    h, w, _ = rgb.shape
    v = np.nan_to_num(rgb, nan=0.0, posinf=1.0, neginf=0.0)
    b = np.clip(np.rint(np.clip(v, 0.0, 1.0) * 255.0), 0, 255).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(b.tobytes())


def pixels_to_image(pixels: np.ndarray, width: int, height: int) -> np.ndarray:
    """Row-major RGB image (row 0 first) from the pixel buffer (float4 per
    pixel, pixel index y * width + x)."""
    return np.asarray(pixels, np.float32).reshape(height, width, 4)[:, :, :3]


# ------------------------------------------------------------ run
def run(opts: Dict[str, Any], out_image: str = "", device=None, frames=None, quiet=False) -> Dict[str, Any]:
    import torch

    from . import api
    dev = device or torch.device("cuda", 0)
    pos, nrm, idx, first = load_scene(opts)
    t0 = time.perf_counter()
    scene = api.Scene(pos, idx, geometry_first=first if first.shape[0] > 1 else None)
    build_ms = (time.perf_counter() - t0) * 1e3
    geom = api.Geometry(pos, nrm, idx, device=dev, geometry_first=first if first.shape[0] > 1 else None)
    w, h = opts["Resolution.width"], opts["Resolution.height"]
    cfg = renderer_config(opts)
    r = api.Renderer(config=cfg)
    light = opts["Camera.position"] if opts["Scene.headlight"] else opts["Scene.light"]
    r.set_scene(scene, geom, light, opts["Scene.backgroundcolor"])
    cam = api.make_camera(position=opts["Camera.position"], rotation_deg=opts["Camera.rotation"],
                          fov_deg=opts["Camera.fieldOfView"], znear=opts["Camera.nearPlane"],
                          zfar=opts["Camera.farPlane"])
    px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    warm = opts["Benchmark.warmupCycles"]
    cycles = opts["Benchmark.benchmarkCycles"] if frames is None else frames
    if opts["Application.mode"] != "benchmark" and frames is None:
        warm, cycles = 0, 1
    keys = ("primary", "shadow", "path")
    acc = dict(kernels_ms=0.0, absolute_ms=0.0, primary=0, shadow=0, path=0, trace_primary=0.0, trace_shadow=0.0,
               trace_path=0.0, perf_total=0.0, perf_primary=0.0, perf_shadow=0.0, perf_path=0.0)
    depth = opts["Renderer.recursionDepth"]
    fields = ("ray_count", "morton_ms", "sort_ms", "reorder_ms", "trace_sort_ms", "trace_ms")
    shadow_logs = [dict.fromkeys(fields, 0.0) for _ in range(depth + 1)]
    path_logs = [dict.fromkeys(fields, 0.0) for _ in range(depth)]
    timed = False

    def perf(rays, ms):  # Renderer::get*TracePerformance (Renderer.cpp:692-706)
        return rays * 1.0e-3 / ms if ms > 0 else 0.0

    for f in range(warm + cycles):
        t = time.perf_counter()
        r.render(cam, w, h, px, fp)
        st = r.stats()  # waits for the frame
        absolute = (time.perf_counter() - t) * 1e3
        if f < warm:
            continue
        timed = bool(st.timed)
        acc["kernels_ms"] += st.frame_ms
        acc["absolute_ms"] += absolute
        counts = (st.num_primary_rays, st.num_shadow_rays, st.num_path_rays)
        times = (st.primary_trace_ms, st.shadow_trace_ms, st.path_trace_ms)
        for k, c, ms in zip(keys, counts, times):
            acc[k] += c
            acc["trace_" + k] += ms
            acc["perf_" + k] += perf(c, ms)
        acc["perf_total"] += perf(sum(counts), sum(times))
        for logs, src in ((shadow_logs, st.shadow_sort_logs), (path_logs, st.path_sort_logs)):
            for i, lg in enumerate(logs):
                for fld in fields:
                    lg[fld] += getattr(src[i], fld)
    n = max(cycles, 1)
    rays = (acc["primary"] + acc["shadow"] + acc["path"]) / n
    res = {"ray_type": opts["Renderer.rayType"], "total_rays": rays, "primary_rays": acc["primary"] / n,
           "shadow_rays": acc["shadow"] / n, "path_rays": acc["path"] / n,
           "render_kernels_ms": acc["kernels_ms"] / n, "render_absolute_ms": acc["absolute_ms"] / n,
           "stage_times": timed,
           "trace_total_ms": (acc["trace_primary"] + acc["trace_shadow"] + acc["trace_path"]) / n,
           "trace_primary_ms": acc["trace_primary"] / n, "trace_shadow_ms": acc["trace_shadow"] / n,
           "trace_path_ms": acc["trace_path"] / n,
           "rt_perf_total_mrays_s": acc["perf_total"] / n, "rt_perf_primary_mrays_s": acc["perf_primary"] / n,
           "rt_perf_shadow_mrays_s": acc["perf_shadow"] / n, "rt_perf_path_mrays_s": acc["perf_path"] / n,
           "frame_perf_mrays_s": rays * 1e-3 / (acc["kernels_ms"] / n) if acc["kernels_ms"] else 0.0,
           "shadow_sort_logs": [{k: v / n for k, v in lg.items()} for lg in shadow_logs],
           "path_sort_logs": [{k: v / n for k, v in lg.items()} for lg in path_logs],
           "print_sort_logs": bool(opts["Benchmark.printSortLogs"]),
           "frames": warm + cycles, "bvh_build_ms": build_ms, "triangles": int(idx.shape[0])}
    if out_image:
        img = pixels_to_image(px.cpu().numpy(), w, h)
        (write_pfm if str(out_image).endswith(".pfm") else write_ppm)(out_image, img)
        res["image"] = str(out_image)
    if not quiet and opts["Application.mode"] == "benchmark":
        print(benchmark_text(res))
    return res


def benchmark_text(res: Dict[str, Any]) -> str:
    """The results block of Benchmark::run (Benchmark.cpp:128-195): averaged
    counts, TRACE times and RT PERF per ray type (rays / trace time, where a
    trace time covers ray generation, sorting and traversal as in the
    reference; zero without stage times), the overall times, and with
    Benchmark.printSortLogs the SORT LOG of every depth and its total."""
    lines = [
        "=" * 50, " RAY TRACING BENCHMARK RESULTS ", "-" * 50,
        f" RAY TYPE                : {res['ray_type']}", "", " [Count (Average)]",
        f" TOTAL RAYS              : {int(res['total_rays'])}",
        f" PRIMARY RAYS            : {int(res['primary_rays'])}",
        f" SHADOW RAYS             : {int(res['shadow_rays'])}",
        f" PATH RAYS               : {int(res['path_rays'])}", "", " [Time (ms)]",
        f" TRACE TOTAL             : {res['trace_total_ms']:.4f} ms",
        f" TRACE PRIMARY           : {res['trace_primary_ms']:.4f} ms",
        f" TRACE SHADOW            : {res['trace_shadow_ms']:.4f} ms",
        f" TRACE PATH              : {res['trace_path_ms']:.4f} ms", "", " [Performance (Mrays/s)]",
        f" RT PERF TOTAL           : {res['rt_perf_total_mrays_s']:.2f}",
        f" RT PERF PRIMARY         : {res['rt_perf_primary_mrays_s']:.2f}",
        f" RT PERF SHADOW          : {res['rt_perf_shadow_mrays_s']:.2f}",
        f" RT PERF PATH            : {res['rt_perf_path_mrays_s']:.2f}", "", " [Overall Time]",
        f" RENDER KERNELS          : {res['render_kernels_ms']:.4f} ms",
        f" RENDER ABSOLUTE         : {res['render_absolute_ms']:.4f} ms", "-" * 50, "=" * 50]
    if res.get("print_sort_logs"):
        for label, logs, first in (("SHADOW", res["shadow_sort_logs"], 0), ("PATH", res["path_sort_logs"], 1)):
            total = {k: 0.0 for k in ("ray_count", "morton_ms", "sort_ms", "reorder_ms", "trace_sort_ms",
                                      "trace_ms")}
            lines += ["=" * 50, "-" * 50]
            for i, lg in enumerate(logs):
                lines += [f"SORT LOG {label} AT DEPTH {i + first}", *_sort_log_lines(lg), ""]
                for k in total:
                    total[k] += lg[k]
            lines += ["-" * 50, f"SORT LOG {label} TOTAL", *_sort_log_lines(total), "-" * 50, "=" * 50]
    return "\n".join(lines)


def _sort_log_lines(lg: Dict[str, float]) -> List[str]:
    return [f"RAY COUNTS        : {int(lg['ray_count'])}",
            f"MORTONCODES TIME  : {lg['morton_ms']:.4f} ms",
            f"SORT TIME         : {lg['sort_ms']:.4f} ms",
            f"REORDER TIME      : {lg['reorder_ms']:.4f} ms",
            f"TRACE SORT TIME   : {lg['trace_sort_ms']:.4f} ms",
            f"TRACE TIME        : {lg['trace_ms']:.4f} ms\n"]


def main(argv: List[str] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--env", required=True, help="env.json path")
    ap.add_argument("--out", default="", help="image file (.pfm or .ppm); overrides Output.image")
    ap.add_argument("--frames", type=int, default=None, help="frames to render after warm-up")
    ap.add_argument("--json", action="store_true", help="print the results as one JSON line")
    args = ap.parse_args(argv)
    from . import build
    build.build()
    opts = load_env(args.env)
    res = run(opts, args.out or opts["Output.image"], frames=args.frames, quiet=args.json)
    if args.json:
        print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
