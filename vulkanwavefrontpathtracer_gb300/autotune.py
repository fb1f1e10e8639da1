"""Autotuner for the wavefront stages.

Searches, on the GPU it runs on and for a given scene:
  * the persistent BVH8 traversal knobs (warp refill threshold, triangle
    postponing threshold), separately for closest-hit and any-hit rays;
  * the Morton key layout (32-bit Aila, 48- and 64-bit 6-D) and whether to
    reorder the rays, for a path-ray wavefront, by timing the composite
    Morton + radix sort + reorder + trace.
Timings use CUDA events over repeated launches on the current stream.  The
result is a plain dict that `apply()` installs (traversal knobs are
process-wide) and that a renderer configuration can take the key/reorder
choice from.
"""
from __future__ import annotations

import itertools
from typing import Callable, Dict, Iterable

from . import _lib as L
from . import api


def _timeit(fn: Callable[[], None], reps: int = 5, warm: int = 2) -> float:
    import torch
    stream = torch.cuda.current_stream()
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune_traversal(scene: api.Scene, closest_rays, any_rays, refills: Iterable[int] = (1, 2, 4, 8, 16, 32),
                   postpones: Iterable[int] = (0, 4, 8, 12), coops: Iterable[int] = (0, 1),
                   batches: Iterable[int] = (1, 8, 16, 24, 32), steps: Iterable[int] = (1, 2, 3),
                   reps: int = 5) -> Dict:
    """Grid search of refill x (cooperative tests: batch x node steps per
    iteration; per-lane tests: postpone) for BVH8 closest-hit and any-hit
    traversal; returns the best settings and the full table (ms)."""
    import torch
    dev = closest_rays.device
    res_c = torch.empty((closest_rays.shape[0], 4), dtype=torch.int32, device=dev)
    res_a = torch.empty((any_rays.shape[0], 4), dtype=torch.int32, device=dev)
    keys = ("trace.bvh8.refill", "trace.bvh8.postpone", "trace.bvh8.coop", "trace.bvh8.batch", "trace.bvh8.steps")
    kind_keys = ("trace.bvh8.any_batch", "trace.bvh8.any_steps")
    old = [api.tune_get(k) for k in keys]
    old_any = [api.tune_get(k) for k in kind_keys]
    grid = []
    for coop in coops:
        for refill in refills:
            if coop:
                grid += [(refill, 0, 1, b, s) for b, s in itertools.product(batches, steps)]
            else:
                grid += [(refill, p, 0, old[3], old[4]) for p in postpones]
    table = []
    try:
        for setting in grid:
            for k, v in zip(keys, setting):
                api.tune_set(k, v)
            for k, v in zip(kind_keys, setting[3:]):  # both kinds of rays take the setting's batch and steps
                api.tune_set(k, v)
            mc = _timeit(lambda: api.trace(scene, L.BVH8_Q8, closest_rays, res_c, closest_hit=True), reps)
            ma = _timeit(lambda: api.trace(scene, L.BVH8_Q8, any_rays, res_a, closest_hit=False), reps)
            refill, post, coop, batch, stp = setting
            table.append({"refill": refill, "postpone": post, "coop": coop, "batch": batch, "steps": stp,
                          "closest_ms": mc, "any_ms": ma})
    finally:
        for k, v in zip(keys, old):
            api.tune_set(k, v)
        for k, v in zip(kind_keys, old_any):
            api.tune_set(k, v)
    # Refill, postpone and coop are shared by both kinds of rays (the best
    # sum of both times); batch and steps are set per kind, each from the
    # best time of its own kind among the settings with the shared knobs
    # chosen.
    nc, na = closest_rays.shape[0], any_rays.shape[0]
    best = min(table, key=lambda e: e["closest_ms"] + e["any_ms"])
    same = [e for e in table if (e["refill"], e["postpone"], e["coop"]) == (best["refill"], best["postpone"],
                                                                             best["coop"])]
    best_c = min(same, key=lambda e: e["closest_ms"])
    best_a = min(same, key=lambda e: e["any_ms"])
    return {"refill": best["refill"], "postpone": best["postpone"], "coop": best["coop"], "batch": best_c["batch"],
            "steps": best_c["steps"], "any_batch": best_a["batch"], "any_steps": best_a["steps"], "table": table,
            "best_closest_mrays_s": nc / (best_c["closest_ms"] * 1e-3) / 1e6,
            "best_any_mrays_s": na / (best_a["any_ms"] * 1e-3) / 1e6}


KEY_CHOICES = ((L.MORTON_AILA32, 32), (L.MORTON_6D48, 48), (L.MORTON_6D64, 63))


def tune_keys(scene: api.Scene, path_rays, bvh_kind: int = L.BVH8_Q8, reps: int = 5) -> Dict:
    """Times trace alone, and Morton + sort + (reorder | indirect) + trace for
    each key layout; returns the fastest choice and the table (ms)."""
    import torch
    dev = path_rays.device
    m = path_rays.shape[0]
    res = torch.empty((m, 4), dtype=torch.int32, device=dev)
    keys = torch.empty(m, dtype=torch.int64, device=dev)
    ids = torch.empty(m, dtype=torch.int32, device=dev)
    scratch = torch.empty(api.sort_scratch_bytes(m, 64), dtype=torch.uint8, device=dev)
    s2i = torch.arange(m, dtype=torch.int32, device=dev)
    out = torch.empty_like(path_rays)
    os2i = torch.empty(m, dtype=torch.int32, device=dev)
    oi2s = torch.empty(m, dtype=torch.int32, device=dev)
    smin = scene.bounds_min
    ssize = scene.bounds_max - scene.bounds_min
    table = [{"morton": None, "reorder": False,
              "ms": _timeit(lambda: api.trace(scene, bvh_kind, path_rays, res), reps)}]
    for kind, bits in KEY_CHOICES:
        for reorder in (False, True):
            def step(kind=kind, bits=bits, reorder=reorder):
                api.morton(path_rays, smin, ssize, kind, keys, ids)
                api.sort_pairs(keys, ids, bits, scratch=scratch)
                if reorder:
                    api.reorder(ids, path_rays, out, s2i, os2i, oi2s)
                    api.trace(scene, bvh_kind, out, res)
                else:
                    api.trace(scene, bvh_kind, path_rays, res, ray_index=ids)
            table.append({"morton": kind, "key_bits": bits, "reorder": reorder, "ms": _timeit(step, reps)})
    best = min(table, key=lambda e: e["ms"])
    return {"best": best, "table": table}


def tune_sort(keys, key_bits: int, reps: int = 10) -> Dict:
    """Radix digit width (4 or 8 bits) x tile variant (small, large,
    extra-large; 64-bit keys have no extra-large tile, so 3 repeats 2) for
    sorts of `keys` (a device tensor of int32 / int64 keys); returns the
    fastest setting and the table (ms per sort, keys restored before
    every sort)."""
    import torch
    n = keys.shape[0]
    work = keys.clone()
    vals = torch.empty(n, dtype=torch.int32, device=keys.device)
    scratch = torch.empty(api.sort_scratch_bytes(n, 64 if key_bits > 32 else 32), dtype=torch.uint8,
                          device=keys.device)
    old = (api.tune_get("sort.digit_bits"), api.tune_get("sort.tiles"))
    table = []
    try:
        for db, tiles in itertools.product((8, 4), (1, 2) if key_bits > 32 else (1, 2, 3)):
            api.tune_set("sort.digit_bits", db)
            api.tune_set("sort.tiles", tiles)

            def one():
                work.copy_(keys)
                api.sort_pairs(work, vals, key_bits, scratch=scratch)

            copy_ms = _timeit(lambda: work.copy_(keys), reps)
            table.append({"digit_bits": db, "tiles": tiles, "ms": max(_timeit(one, reps) - copy_ms, 0.0)})
    finally:
        api.tune_set("sort.digit_bits", old[0])
        api.tune_set("sort.tiles", old[1])
    best = min(table, key=lambda e: e["ms"])
    return {"digit_bits": best["digit_bits"], "tiles": best["tiles"], "table": table}


def tune_bounce_sort(make_renderer, camera, width: int, height: int, depth: int, frames: int = 3,
                     device=None) -> Dict:
    """Per-bounce reordering: greedy search of the renderer's path_sort_skip
    mask.  make_renderer(path_sort_skip) returns a renderer with its scene
    set (sorting and reordering of path rays on); each bounce's bit is kept
    flipped when whole frames get faster.  Returns the best mask, its frame
    time and the table of tried masks (median ms of `frames` frames)."""
    import statistics

    import torch
    dev = device or torch.device("cuda", 0)
    px = torch.zeros((width * height, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)

    def frame_ms(mask):
        r = make_renderer(mask)
        r.render(camera, width, height, px, fp)  # warm-up (and graph capture)
        times = []
        for _ in range(frames):
            r.render(camera, width, height, px, fp)
            times.append(r.stats().frame_ms)
        r.close()
        return statistics.median(times)

    best_mask, best_ms = 0, frame_ms(0)
    table = [{"path_sort_skip": 0, "ms": best_ms}]
    for b in range(depth):
        mask = best_mask | (1 << b)
        ms = frame_ms(mask)
        table.append({"path_sort_skip": mask, "ms": ms})
        if ms < best_ms:
            best_mask, best_ms = mask, ms
    return {"path_sort_skip": best_mask, "ms": best_ms, "table": table}


def tune_primary_bvh(make_renderer, camera, width: int, height: int, frames: int = 3, device=None) -> Dict:
    """BVH of the primary pass (coherent camera rays and their shadow
    rays): make_renderer(primary_bvh_kind) returns a renderer with its scene
    set; whole frames are timed with the FP32 BVH2 and with the BVH8 there.
    Returns the faster kind and the table (median ms of `frames` frames)."""
    import statistics

    import torch
    dev = device or torch.device("cuda", 0)
    px = torch.zeros((width * height, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)
    table = []
    for kind in (L.BVH2_FP32, L.BVH8_Q8):
        r = make_renderer(kind)
        r.render(camera, width, height, px, fp)
        times = []
        for _ in range(frames):
            r.render(camera, width, height, px, fp)
            times.append(r.stats().frame_ms)
        r.close()
        table.append({"primary_bvh_kind": kind, "ms": statistics.median(times)})
    best = min(table, key=lambda e: e["ms"])
    return {"primary_bvh_kind": best["primary_bvh_kind"], "ms": best["ms"], "table": table}


def tune_bvh_kinds(make_renderer, camera, width: int, height: int, frames: int = 3, device=None) -> Dict:
    """BVH of the bounces and of the primary pass: make_renderer(bvh_kind,
    primary_bvh_kind) returns a renderer with its scene set; whole frames are
    timed with the BVH8 everywhere, the FP32 BVH2 for the primary pass only,
    and the FP32 BVH2 everywhere.  Returns the fastest pair and the table
    (median ms of `frames` frames)."""
    import statistics

    import torch
    dev = device or torch.device("cuda", 0)
    px = torch.zeros((width * height, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)
    table = []
    for kind, pkind in ((L.BVH8_Q8, -1), (L.BVH8_Q8, L.BVH2_FP32), (L.BVH2_FP32, -1)):
        r = make_renderer(kind, pkind)
        r.render(camera, width, height, px, fp)
        times = []
        for _ in range(frames):
            r.render(camera, width, height, px, fp)
            times.append(r.stats().frame_ms)
        r.close()
        table.append({"bvh_kind": kind, "primary_bvh_kind": pkind, "ms": statistics.median(times)})
    best = min(table, key=lambda e: e["ms"])
    return {"bvh_kind": best["bvh_kind"], "primary_bvh_kind": best["primary_bvh_kind"], "ms": best["ms"],
            "table": table}


def measure_work(scene: api.Scene, rays, bvh_kind: int, closest: bool) -> Dict:
    """Node visits and triangle tests per ray (counting kernel variants)."""
    import torch
    res = torch.empty((rays.shape[0], 4), dtype=torch.int32, device=rays.device)
    old = api.tune_get("trace.count")
    api.tune_set("trace.count", 1)
    try:
        api.trace_counters(reset=True)
        api.trace(scene, bvh_kind, rays, res, closest_hit=closest)
        c = api.trace_counters(reset=True)
    finally:
        api.tune_set("trace.count", old)
    n = max(1, c["rays"])
    out = {"rays": c["rays"], "nodes_per_ray": c["nodes"] / n, "tris_per_ray": c["tris"] / n}
    if c["warp_iters"]:
        # lanes busy per warp loop iteration: node steps / iterations
        out["warp_iters"] = c["warp_iters"]
        out["node_steps_per_iter"] = c["nodes"] / c["warp_iters"]
    return out


def apply(traversal: Dict) -> None:
    api.tune_set("trace.bvh8.refill", traversal["refill"])
    api.tune_set("trace.bvh8.postpone", traversal["postpone"])
    if "coop" in traversal:
        api.tune_set("trace.bvh8.coop", traversal["coop"])
    if "batch" in traversal:
        api.tune_set("trace.bvh8.batch", traversal["batch"])
    if "steps" in traversal:
        api.tune_set("trace.bvh8.steps", traversal["steps"])
    if "any_batch" in traversal:
        api.tune_set("trace.bvh8.any_batch", traversal["any_batch"])
    if "any_steps" in traversal:
        api.tune_set("trace.bvh8.any_steps", traversal["any_steps"])
