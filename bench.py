"""Benchmark of the wavefront path tracer on one GB300 (or N replicas).

Workload (default): the courtyard scene -- tessellated 30x12x20 room, 48
cylinders of 2,048 triangles and 50,000 clutter triangles (268,304
triangles, seeded) -- rendered at 1920x1080, 1 spp, path rays with 8
bounces and 2 shadow samples per hit.  A step is one frame
(Renderer::render): primary rays, shadow rays, 8 bounces of path rays with
Morton keys, radix sort, reorder and traversal, shading, accumulation.

Forms:
  chosen  8-wide BVH with 8-bit quantised boxes, 64-bit 6-D Morton keys,
          sort + reorder of the path rays of every bounce
  plain   binary BVH with FP32 boxes, no sorting
The headline value is the chosen form's rays per second over the whole
frame (reference metric Mrays/s = rays * 1e-3 / ms, Renderer.cpp:692-706,
here with everything in the frame timed).  The per-bounce microbenchmark
traces one incoherent bounce wavefront with each form.

Usage:
  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

COURTYARD = dict(
    scene_kind=1, seed=1, width=1920, height=1080,
    camera=dict(position=(15.0, 5.0, 19.4), rotation_deg=(-8.0, 12.0, 0.0), fov_deg=60.0, znear=0.1, zfar=512.0),
    light=(15.0, 11.0, 10.0), background=(0.529, 0.808, 0.98),
    renderer=dict(ray_type=2, num_primary_samples=1, num_shadow_samples=2, shadow_radius=1.0, recursion_depth=8,
                  key_value=0.6, white_point=2.0, albedo=0.8),
)
# Shadow rays are generated in the (already reordered) slot order of their
# path rays and all aim at the light, so the chosen form does not sort them.
# The chosen form replays each frame as one captured graph with persistent
# BVH8 traversal, each pass's shadow rays traced on a second stream while
# the next bounce runs; the plain form launches every stage directly on one
# stream (unbatched) with FP32 BVH2 nodes.
CHOSEN = dict(bvh_kind=1, morton_kind=2, sort_path_rays=1, reorder_path_rays=1, sort_shadow_rays=0,
              reorder_shadow_rays=0, use_graph=1, shadow_overlap=1)
PLAIN = dict(bvh_kind=0, morton_kind=0, sort_path_rays=0, reorder_path_rays=0, sort_shadow_rays=0,
             reorder_shadow_rays=0, use_graph=0, shadow_overlap=0)
# The city block (3,000,320 triangles; its BVH2 does not fit in L2) at
# 3840x2160: the per-bounce comparison on the largest incoherent workload.
CITY = dict(
    scene_kind=2, seed=1, width=3840, height=2160,
    camera=dict(position=(320.0, 90.0, 700.0), rotation_deg=(-25.0, 0.0, 0.0), fov_deg=60.0, znear=0.1,
                zfar=2048.0),
    light=(320.0, 300.0, 320.0), background=(0.529, 0.808, 0.98),
    renderer=dict(num_shadow_samples=2, shadow_radius=4.0),
)
# The reference arm renders every 4th pixel-table slot of the courtyard frame
# per step (a quarter of its rays, spread over the whole image).
REF_PIXEL_STRIDE = 4
WORKLOAD_NAME = ("courtyard: 268,304 triangles, 1920x1080, 1 spp, path rays, 8 bounces, 2 shadow samples; "
                 "chosen form = BVH8-Q8 + persistent graph-captured wavefront + 64-bit 6-D Morton sort/reorder "
                 "of the path rays of every bounce")
METRIC = "Mrays/s per bounce, chosen vs plain form; radix sort+reorder HBM GB/s vs peak"
# DRAM bytes (read + write) per ray of the full-size bounce-1 BVH8 traversal
# launches (2,073,600 sorted closest-hit path rays, 4,147,200 any-hit shadow
# rays), median of 12 launches each from one ncu capture of
# `bench.py --micro-only` (dram__bytes_read.sum + dram__bytes_write.sum,
# cold caches): closest 87.6 MB + 10.2 MB, any-hit 152.9 MB + 40.6 MB.
TRACE_DRAM_BYTES_PER_RAY = {"any": 46.64, "closest": 47.20}
# Warp instructions per ray of the courtyard's bounce-1 BVH8 traversal
# (sm__inst_executed.sum / rays of one launch each, `bench.py --trace-profile`
# under ncu at 960x540: 288,619,160 for 518,400 sorted closest-hit path rays,
# 337,241,928 for 1,036,800 any-hit shadow rays).  With the live launch time
# they give the issue rate; the issue peak is 152 SMs x 4 schedulers x one
# warp instruction per clock at the sampled SM clock.
TRACE_WARP_INST_PER_RAY = {"any": 325.27, "closest": 556.75}
NUM_SMS = 152


def workload_config(triangles, world):
    """The `config` of the bench line, the same for both arms."""
    return {"workload": WORKLOAD_NAME, "resolution": [COURTYARD["width"], COURTYARD["height"]],
            "triangles": int(triangles), "parallelism": f"replicas x{world}",
            "l2": "frame working set (>1 GB of ray/hit/key buffers) exceeds the 129 MB L2"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def setup_dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_over_ranks(ms, rays, world, device):
    """Job-wide result of one timed region: the slowest rank's time and the
    rays all ranks traced.  The ranks meet at a barrier first, so none
    leaves the timed region's accounting early; world == 1 returns the
    inputs.  Replicas share nothing else: no collective touches the data
    path."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    rt = torch.tensor([float(rays)], dtype=torch.float64, device=device)
    if world > 1:
        dist.barrier()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(rt, op=dist.ReduceOp.SUM)
    return float(t.item()), float(rt.item())


# ------------------------------------------------------------------ ours
def city_frames(wf, api, dev, stream, scene, geom, steps=3):
    """Whole city frames (3840x2160, 1 spp, 8 bounces, 2 shadow samples):
    the chosen form as specified (BVH8, sort + reorder of every bounce,
    graph replay, overlapped shadow passes), the plain form, and the chosen
    form as autotuned on this GPU (per-bounce reordering, then the BVH of the
    bounces and of the primary pass, searched on whole frames).  Mrays/s
    over all rays of a frame, CUDA events on the launching stream."""
    import torch

    from vulkanwavefrontpathtracer_gb300 import autotune
    W = CITY
    w, h = W["width"], W["height"]
    cam = api.make_camera(**W["camera"])
    rcfg = dict(COURTYARD["renderer"], **W["renderer"])
    px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)

    def make(form):
        r = api.Renderer(**rcfg, **form)
        r.set_scene(scene, geom, W["light"], W["background"])
        return r

    def timed(form, warm=1):
        r = make(form)
        for _ in range(warm):
            r.render(cam, w, h, px, fp)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            r.render(cam, w, h, px, fp)
        b.record(stream)
        torch.cuda.synchronize()
        st = r.stats()
        r.close()
        ms = a.elapsed_time(b) / steps
        rays = st.num_primary_rays + st.num_shadow_rays + st.num_path_rays
        return ms, rays

    c_ms, rays = timed(CHOSEN)
    p_ms, _ = timed(PLAIN)
    depth = rcfg["recursion_depth"]
    tune = autotune.tune_bounce_sort(lambda m: make(dict(CHOSEN, path_sort_skip=m)), cam, w, h, depth, frames=2,
                                     device=dev)
    mask = int(tune["path_sort_skip"])
    ktune = autotune.tune_bvh_kinds(
        lambda k, pk: make(dict(CHOSEN, path_sort_skip=mask, bvh_kind=k, primary_bvh_kind=pk)), cam, w, h, frames=2,
        device=dev)
    kinds = dict(bvh_kind=int(ktune["bvh_kind"]), primary_bvh_kind=int(ktune["primary_bvh_kind"]))
    t_ms, _ = timed(dict(CHOSEN, path_sort_skip=mask, **kinds))
    mr = lambda ms: round(rays / (ms * 1e-3) / 1e6, 3)
    return {"resolution": [w, h], "rays_per_frame": int(rays),
            "chosen": {"value": mr(c_ms), "unit": "Mrays/s", "ms_per_frame": round(c_ms, 3)},
            "plain": {"value": mr(p_ms), "unit": "Mrays/s", "ms_per_frame": round(p_ms, 3)},
            "chosen_over_plain": round(p_ms / c_ms, 3),
            "autotuned": {"value": mr(t_ms), "unit": "Mrays/s", "ms_per_frame": round(t_ms, 3),
                          "over_plain": round(p_ms / t_ms, 3), "path_sort_skip": mask, **kinds,
                          "search": [{"path_sort_skip": e["path_sort_skip"], "ms": round(e["ms"], 3)}
                                     for e in tune["table"]]
                          + [{"bvh_kind": e["bvh_kind"], "primary_bvh_kind": e["primary_bvh_kind"],
                              "ms": round(e["ms"], 3)} for e in ktune["table"]]}}


def city_bounce(wf, api, dev, stream, frames=True, size=None):
    """The bounce-1 comparison of `bounce_micro` on the city block at
    3840x2160 (8.3M primary rays; `size` = (w, h) for a smaller profiling
    case) and, with `frames`, whole city frames (city_frames).  Returns the
    per-bounce line (with the frames under "frames") and the host-built city
    scene (for the build-time report)."""
    W = dict(CITY, width=size[0], height=size[1]) if size else CITY
    pos, nrm, idx = api.generate_scene(W["scene_kind"], W["seed"])
    scene = api.Scene(pos, idx)
    geom = api.Geometry(pos, nrm, idx, device=dev)
    cam = api.make_camera(**W["camera"])
    micro = bounce_micro(wf, api, dev, scene, geom, cam, W["width"], W["height"], stream, workload=W)
    line = dict(micro["per_bounce"])
    line["triangles"] = int(scene.info.num_triangles)
    line["resolution"] = [W["width"], W["height"]]
    line["sort_gbs"] = round(micro["sort"]["gbs"], 1)
    del micro
    if frames:
        line["frames"] = city_frames(wf, api, dev, stream, scene, geom)
    del geom
    return line, (pos, idx, scene)


def scene_build_times(api, pos, idx, host_scene, city=None):
    """Acceleration-structure build times (BVH2 + BVH8) of the courtyard and
    the 3M-triangle city block: host build (binned SAH + collapse) and device
    build (PLOC + collapse on the GPU; the first device build of the process
    also loads the build kernels, so it is done once untimed).  `city`: the
    city's (positions, indices, host-built scene), when already built."""
    out = {"courtyard_host_ms": round(host_scene.info.build_ms, 1)}
    warm = api.Scene(pos, idx, device_build=True)
    warm.close()
    d = api.Scene(pos, idx, device_build=True)
    out["courtyard_device_ms"] = round(d.info.build_ms, 1)
    d.close()
    if city is None:
        cpos, _, cidx = api.generate_scene(2, 1)
        hsc = api.Scene(cpos, cidx)
    else:
        cpos, cidx, hsc = city
    out["city_host_ms"] = round(hsc.info.build_ms, 1)
    hsc.close()
    # Three device builds, the fastest reported: a single build also times
    # the driver mapping the first allocations of its ~1 GB of temporaries
    # (8-50 ms seen for the same build).
    times = []
    for _ in range(3):
        d = api.Scene(cpos, cidx, device_build=True)
        out["city_triangles"] = int(d.info.num_triangles)
        times.append(d.info.build_ms)
        d.close()
    out["city_device_ms"] = round(min(times), 1)
    out["city_device_ms_all"] = [round(t, 1) for t in times]
    out["city_device_speedup"] = round(out["city_host_ms"] / max(out["city_device_ms"], 1e-3), 1)
    out["note"] = "device-built trees trace the courtyard's bounce-1 rays 10-13 % slower (PLOC vs binned SAH)"
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    import vulkanwavefrontpathtracer_gb300 as wf
    from vulkanwavefrontpathtracer_gb300 import build as wbuild
    wbuild.build()
    world, rank, local = setup_dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    api = wf.api
    lib = wf._lib.load()
    W = COURTYARD
    w, h = W["width"], W["height"]
    pos, nrm, idx = api.generate_scene(W["scene_kind"], W["seed"])
    scene = api.Scene(pos, idx)
    geom = api.Geometry(pos, nrm, idx, device=dev)
    cam = api.make_camera(**W["camera"])
    stream = torch.cuda.current_stream()

    def make(form):
        r = api.Renderer(**W["renderer"], **form)
        r.set_scene(scene, geom, W["light"], W["background"])
        return r

    px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)

    def timed_frames(r, steps, warmup):
        for _ in range(warmup):
            r.render(cam, w, h, px, fp)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = lib.wfpt_kernel_launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rays = 0
        ev0.record(stream)
        for _ in range(steps):
            r.render(cam, w, h, px, fp)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        launches = lib.wfpt_kernel_launch_count() - l0
        st = r.stats()
        rays = (st.num_primary_rays + st.num_shadow_rays + st.num_path_rays) * steps
        ms, rays = reduce_over_ranks(ms, rays, world, dev)
        return ms, rays, st, launches

    # Headline: the courtyard configuration as specified, every bounce's
    # path rays Morton-sorted and reordered.  Beside it, the per-bounce
    # reordering the autotuner picks on this GPU (tune_bounce_sort: greedy
    # over the bounces, whole frames timed, before the timed regions).
    chosen = make(CHOSEN)
    plain = make(PLAIN)
    with ClockSampler(local) as clocks:
        ms_c, rays_c, st_c, launches = timed_frames(chosen, args.steps, args.warmup)
    ms_p, rays_p, st_p, _ = timed_frames(plain, args.steps, max(1, args.warmup // 2))
    value = rays_c / (ms_c * 1e-3) / 1e6
    plain_value = rays_p / (ms_p * 1e-3) / 1e6
    from vulkanwavefrontpathtracer_gb300 import autotune
    tune = autotune.tune_bounce_sort(lambda m: make(dict(CHOSEN, path_sort_skip=m)), cam, w, h,
                                     W["renderer"]["recursion_depth"], frames=3, device=dev)
    mask = int(tune["path_sort_skip"])
    ktune = autotune.tune_bvh_kinds(
        lambda k, pk: make(dict(CHOSEN, path_sort_skip=mask, bvh_kind=k, primary_bvh_kind=pk)), cam, w, h, frames=3,
        device=dev)
    bkind, pkind = int(ktune["bvh_kind"]), int(ktune["primary_bvh_kind"])
    tuned = make(dict(CHOSEN, path_sort_skip=mask, bvh_kind=bkind, primary_bvh_kind=pkind))
    ms_t, rays_t, _, _ = timed_frames(tuned, args.steps, max(1, args.warmup // 2))
    tuned_value = rays_t / (ms_t * 1e-3) / 1e6

    # End to end through the C ABI with host buffers: per step the frame is
    # rendered and the tone-mapped image is read back into pinned memory.
    host_img = torch.empty((w * h, 4), dtype=torch.float32, pin_memory=True)
    for _ in range(2):
        chosen.render(cam, w, h, px, fp)
        host_img.copy_(fp, non_blocking=True)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        chosen.render(cam, w, h, px, fp)
        host_img.copy_(fp, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    rays_per_frame = st_c.num_primary_rays + st_c.num_shadow_rays + st_c.num_path_rays
    e2e_ms, e2e_rays = reduce_over_ranks(e0.elapsed_time(e1), rays_per_frame * args.steps, world, dev)
    e2e_value = e2e_rays / (e2e_ms * 1e-3) / 1e6

    micro = bounce_micro(wf, api, dev, scene, geom, cam, w, h, stream)
    hbm, peak_kind = peaks()
    out = None
    builds = city_line = None
    sort_big = reorder_big = batched = None
    if rank == 0:
        city_line, city = city_bounce(wf, api, dev, stream)
        builds = scene_build_times(api, pos, idx, scene, city=city)
        del city
        torch.cuda.empty_cache()
        sort_big = sort_row(api, dev, stream)
        reorder_big = reorder_row(api, dev, stream)
        batched = batched_serving(api, dev, stream, steps=3, warmup=1)
    if rank == 0:
        cpu = cpu_baseline(args, wf, api, scene, pos, nrm, idx) if world == 1 and not args.no_cpu else None
        if cpu is not None:
            cpu["stages"] = cpu_stages(wf, api, dev, scene, geom, cam)
        def trace_roof(tr, kernel, kind):
            ach = tr["alg_bytes"] / (tr["ms"] * 1e-3) / 1e9
            per_ray = TRACE_DRAM_BYTES_PER_RAY[kind]
            return {"kernel": kernel, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                    "frac": ach / hbm, "traffic": None if per_ray is None else per_ray * tr["rays"],
                    "peak_source": f"{peak_kind} hbm_gbs", "alg_bytes_per_ray": 48,
                    "launch_ms": tr["ms"], "rays_per_launch": tr["rays"],
                    "note": "the BVH and triangles stay in L2, so DRAM carries only the ray and hit records; "
                            "the kernel is bound by instruction issue, not by HBM"}

        def issue_roof(tr, kind):
            mhz = clocks.summary().get("sm_mhz") or clocks.summary().get("sm_max_mhz") or 2070.0
            peak_g = NUM_SMS * 4 * mhz * 1e6 / 1e9
            ach_g = TRACE_WARP_INST_PER_RAY[kind] * tr["rays"] / (tr["ms"] * 1e-3) / 1e9
            return {"bound": "issue", "achieved": round(ach_g, 1), "peak": round(peak_g, 1),
                    "unit": "G warp instructions/s", "frac": round(ach_g / peak_g, 3),
                    "warp_inst_per_ray": TRACE_WARP_INST_PER_RAY[kind], "sm_mhz": mhz,
                    "source": "warp instructions per ray from one ncu launch of the same traversal at 960x540 "
                              "(sm__inst_executed.sum); launch time measured here"}

        roof = trace_roof(micro["trace_shadow"], "k_trace_bvh8_coop<any-hit> (bounce-1 shadow rays, 2 per path ray)",
                          "any")
        roof["issue_roofline"] = issue_roof(micro["trace_shadow"], "any")
        closest_roof = trace_roof(micro["trace_chosen"],
                                  "k_trace_bvh8_coop<closest> (bounce-1 path rays after sort+reorder)", "closest")
        closest_roof["issue_roofline"] = issue_roof(micro["trace_chosen"], "closest")
        srt = micro["sort"]
        sort_roof = {"kernel": "radix sort u64 keys (63 bits, 8 passes) + u32 values", "bound": "hbm",
                     "achieved": srt["gbs"], "peak": hbm, "unit": "GB/s", "frac": srt["gbs"] / hbm,
                     "pairs": srt["n"], "alg_bytes_per_pair": 192}
        out = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_c / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene)",
            "config": workload_config(scene.info.num_triangles, world),
            "rays_per_frame": int(rays_per_frame),
            "path_rays_per_bounce": list(st_c.path_rays_per_bounce),
            "plain": {"value": round(plain_value, 3), "unit": "Mrays/s", "ms_per_step": round(ms_p / args.steps, 4),
                      "rays_per_frame": int(st_p.num_primary_rays + st_p.num_shadow_rays + st_p.num_path_rays)},
            "chosen_over_plain": round(value / plain_value, 3),
            "chosen_over_plain_per_bounce": {
                "courtyard_trace_only": micro["per_bounce"]["chosen_over_plain_trace_only"],
                "courtyard_composite": micro["per_bounce"]["chosen_over_plain_composite"],
                "city_trace_only": city_line["chosen_over_plain_trace_only"] if city_line else None,
                "city_composite": city_line["chosen_over_plain_composite"] if city_line else None,
                "note": "bounce-1 path rays (the incoherent bounce; city = the 3M-triangle block at 3840x2160): "
                        "trace only = BVH8 on the sorted rays vs FP32 BVH2 on the unsorted rays; composite adds "
                        "the Morton keys, sort and reorder to the chosen form"},
            "autotuned": {"value": round(tuned_value, 3), "unit": "Mrays/s", "ms_per_step": round(ms_t / args.steps, 4),
                          "over_plain": round(tuned_value / plain_value, 3), "path_sort_skip": mask,
                          "bvh_kind": bkind, "primary_bvh_kind": pkind,
                          "search": [{"path_sort_skip": e["path_sort_skip"], "ms": round(e["ms"], 3)}
                                     for e in tune["table"]]
                          + [{"bvh_kind": e["bvh_kind"], "primary_bvh_kind": e["primary_bvh_kind"],
                              "ms": round(e["ms"], 3)} for e in ktune["table"]],
                          "note": "chosen form with the per-bounce reordering (autotune.tune_bounce_sort; bit b "
                                  "set: bounce b+1 unsorted) and the BVH of the bounces and of the primary pass "
                                  "(autotune.tune_bvh_kinds; 0 = FP32 BVH2, 1 = BVH8, -1 = as the bounces) "
                                  "picked live on whole frames"},
            "per_bounce": micro["per_bounce"],
            "per_bounce_city": city_line,
            "sort_2p26": sort_big,
            "reorder_2p24": reorder_big,
            "batched": batched,
            "sort_reorder": {"sort_gbs": round(srt["gbs"], 1), "sort_frac": round(srt["gbs"] / hbm, 3),
                             "reorder_gbs": round(micro["reorder"]["gbs"], 1),
                             "reorder_frac": round(micro["reorder"]["gbs"] / hbm, 3)},
            "roofline": roof, "closest_roofline": closest_roof, "sort_roofline": sort_roof,
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 36,
                    "d2h_bytes_per_step": w * h * 16,
                    "note": "camera passed by value through the C ABI; tone-mapped frame read back to pinned host"},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "scene_build": builds,
        }
        print(json.dumps(out))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return out


def bounce_micro(wf, api, dev, scene, geom, cam, w, h, stream, workload=None):
    """One incoherent bounce: primary hits -> cosine bounce rays (bounce 1),
    then traced plain (BVH2, unsorted) and chosen (6-D keys, sort, reorder,
    BVH8).  Also times the sort and reorder kernels alone."""
    W = workload or COURTYARD
    import torch
    n = w * h
    i2p_np, _ = api.pixel_table(w, h)
    i2p = torch.from_numpy(i2p_np).to(dev)
    s2w = api.camera_screen_to_world(cam.position, cam.rotation_deg, cam.fov_deg, w / h, cam.znear, cam.zfar)
    prim = torch.empty((n, 8), dtype=torch.float32, device=dev)
    api.raygen_primary(s2w, i2p, prim, list(cam.position), 0, w, h, cam.zfar)
    hits = torch.empty((n, 4), dtype=torch.int32, device=dev)
    api.trace(scene, wf.BVH8_Q8, prim, hits)
    seeds = torch.empty(n, dtype=torch.int32, device=dev)
    api.init_seeds(seeds, 1)
    dec = torch.ones((n, 4), dtype=torch.float32, device=dev)
    path = torch.empty((n, 8), dtype=torch.float32, device=dev)
    p_i2p = torch.empty(n, dtype=torch.int32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    api.raygen_path(seeds, geom.table, prim, path, i2p, p_i2p, hits, dec, cnt)
    m = int(cnt.item())
    path = path[:m].contiguous()
    res = torch.empty((m, 4), dtype=torch.int32, device=dev)
    smin = scene.bounds_min
    ssize = scene.bounds_max - scene.bounds_min
    keys = torch.empty(m, dtype=torch.int64, device=dev)
    ids = torch.empty(m, dtype=torch.int32, device=dev)
    scratch = torch.empty(api.sort_scratch_bytes(m, 64), dtype=torch.uint8, device=dev)
    s2i = torch.arange(m, dtype=torch.int32, device=dev)
    out = torch.empty_like(path)
    os2i = torch.empty(m, dtype=torch.int32, device=dev)
    oi2s = torch.empty(m, dtype=torch.int32, device=dev)

    def timeit(fn, reps=10):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    ms_plain = timeit(lambda: api.trace(scene, wf.BVH2_FP32, path, res))
    ms_bvh8_unsorted = timeit(lambda: api.trace(scene, wf.BVH8_Q8, path, res))

    def sort_part():
        api.morton(path, smin, ssize, wf.MORTON_6D64, keys, ids)
        api.sort_pairs(keys, ids, 63, scratch=scratch)

    def composite():
        sort_part()
        api.reorder(ids, path, out, s2i, os2i, oi2s)
        api.trace(scene, wf.BVH8_Q8, out, res)

    ms_comp = timeit(composite)
    sort_part()
    api.reorder(ids, path, out, s2i, os2i, oi2s)
    ms_trace8 = timeit(lambda: api.trace(scene, wf.BVH8_Q8, out, res))
    ms_trace2_sorted = timeit(lambda: api.trace(scene, wf.BVH2_FP32, out, res))
    # The bounce's shadow rays (2 per path ray, toward the area light): the
    # any-hit traversal that takes the largest share of a frame.
    S = W["renderer"]["num_shadow_samples"]
    srays = torch.empty((S * m, 8), dtype=torch.float32, device=dev)
    ss2i = torch.empty(S * m, dtype=torch.int32, device=dev)
    si2s = torch.empty(S * m, dtype=torch.int32, device=dev)
    sres = torch.empty((S * m, 4), dtype=torch.int32, device=dev)
    api.raygen_shadow(seeds, out, res, srays, ss2i, si2s, W["light"], W["renderer"]["shadow_radius"], 0, m, S)
    ms_shadow8 = timeit(lambda: api.trace(scene, wf.BVH8_Q8, srays, sres, closest_hit=False))
    ms_shadow2 = timeit(lambda: api.trace(scene, wf.BVH2_FP32, srays, sres, closest_hit=False))
    ms_sort = timeit(lambda: api.sort_pairs(keys, ids, 63, scratch=scratch))
    ms_morton = timeit(lambda: api.morton(path, smin, ssize, wf.MORTON_6D64, keys, ids))
    ms_reorder = timeit(lambda: api.reorder(ids, path, out, s2i, os2i, oi2s))
    mr = lambda ms: round(m / (ms * 1e-3) / 1e6, 2)
    return {
        "per_bounce": {"bounce": 1, "rays": m,
                       "plain_mrays_s": mr(ms_plain), "chosen_composite_mrays_s": mr(ms_comp),
                       "chosen_trace_only_mrays_s": mr(ms_trace8), "bvh8_unsorted_mrays_s": mr(ms_bvh8_unsorted),
                       "bvh2_sorted_mrays_s": mr(ms_trace2_sorted),
                       "chosen_over_plain_composite": round(ms_plain / ms_comp, 3),
                       "chosen_over_plain_trace_only": round(ms_plain / ms_trace8, 3),
                       "morton_ms": round(ms_morton, 4), "sort_ms": round(ms_sort, 4),
                       "reorder_ms": round(ms_reorder, 4),
                       "shadow_rays": S * m, "shadow_bvh8_mrays_s": round(S * m / (ms_shadow8 * 1e-3) / 1e6, 2),
                       "shadow_bvh2_mrays_s": round(S * m / (ms_shadow2 * 1e-3) / 1e6, 2)},
        "trace_chosen": {"ms": ms_trace8, "alg_bytes": 48.0 * m, "rays": m},
        "trace_shadow": {"ms": ms_shadow8, "alg_bytes": 48.0 * S * m, "rays": S * m},
        "sort": {"n": m, "ms": ms_sort, "gbs": 192.0 * m / (ms_sort * 1e-3) / 1e9},
        "reorder": {"n": m, "ms": ms_reorder, "gbs": 80.0 * m / (ms_reorder * 1e-3) / 1e9},
    }


def make_wavefronts(wf, api, dev, scene, geom, cam, w, h, light, shadow_samples=2):
    """Bounce-1 path rays (unsorted, as compacted) and the shadow rays of the
    primary hits, built with the stage kernels."""
    import torch
    n = w * h
    i2p_np, _ = api.pixel_table(w, h)
    i2p = torch.from_numpy(i2p_np).to(dev)
    s2w = api.camera_screen_to_world(cam.position, cam.rotation_deg, cam.fov_deg, w / h, cam.znear, cam.zfar)
    prim = torch.empty((n, 8), dtype=torch.float32, device=dev)
    api.raygen_primary(s2w, i2p, prim, list(cam.position), 0, w, h, cam.zfar)
    hits = torch.empty((n, 4), dtype=torch.int32, device=dev)
    api.trace(scene, wf.BVH8_Q8, prim, hits)
    seeds = torch.empty(n, dtype=torch.int32, device=dev)
    api.init_seeds(seeds, 1)
    srays = torch.empty((n * shadow_samples, 8), dtype=torch.float32, device=dev)
    s2i = torch.empty(n * shadow_samples, dtype=torch.int32, device=dev)
    i2s = torch.empty(n * shadow_samples, dtype=torch.int32, device=dev)
    api.raygen_shadow(seeds, prim, hits, srays, s2i, i2s, light, 1.0, 0, n, shadow_samples)
    dec = torch.ones((n, 4), dtype=torch.float32, device=dev)
    path = torch.empty((n, 8), dtype=torch.float32, device=dev)
    p_i2p = torch.empty(n, dtype=torch.int32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    api.raygen_path(seeds, geom.table, prim, path, i2p, p_i2p, hits, dec, cnt)
    m = int(cnt.item())
    return path[:m].contiguous(), srays


def run_trace_profile(args):
    """A small case for kernel profiles: the bounce-1 path rays of the
    courtyard (or, with --city, the city block) at --width x --height
    (default 960x540) and the shadow rays of the bounce's hits (2 per path
    ray, toward the light), each traversal form launched once after the
    primary trace: BVH2 closest (unsorted), BVH8 closest (unsorted), BVH8
    closest (6-D Morton sorted and reordered), BVH8 any hit, BVH2 any hit.
    Prints the ray counts; the timings of these single launches are not
    benchmark numbers."""
    import torch

    import vulkanwavefrontpathtracer_gb300 as wf
    from vulkanwavefrontpathtracer_gb300 import build as wbuild
    wbuild.build()
    dev = torch.device("cuda", 0)
    api = wf.api
    W = CITY if args.city else COURTYARD
    w, h = args.width or 960, args.height or 540
    pos, nrm, idx = api.generate_scene(W["scene_kind"], W["seed"])
    scene = api.Scene(pos, idx)
    geom = api.Geometry(pos, nrm, idx, device=dev)
    cam = api.make_camera(**W["camera"])
    path, _ = make_wavefronts(wf, api, dev, scene, geom, cam, w, h, W["light"])
    m = path.shape[0]
    res = torch.empty((m, 4), dtype=torch.int32, device=dev)
    keys = torch.empty(m, dtype=torch.int64, device=dev)
    ids = torch.empty(m, dtype=torch.int32, device=dev)
    api.morton(path, scene.bounds_min, scene.bounds_max - scene.bounds_min, wf.MORTON_6D64, keys, ids)
    api.sort_pairs(keys, ids, 63)
    srt = torch.empty_like(path)
    api.reorder(ids, path, srt, torch.arange(m, dtype=torch.int32, device=dev),
                torch.empty(m, dtype=torch.int32, device=dev), torch.empty(m, dtype=torch.int32, device=dev))
    S = W["renderer"]["num_shadow_samples"]
    seeds = torch.zeros(m, dtype=torch.int32, device=dev)
    api.trace(scene, wf.BVH8_Q8, srt, res)
    srays = torch.empty((S * m, 8), dtype=torch.float32, device=dev)
    ss2i = torch.empty(S * m, dtype=torch.int32, device=dev)
    si2s = torch.empty(S * m, dtype=torch.int32, device=dev)
    api.raygen_shadow(seeds, srt, res, srays, ss2i, si2s, W["light"], W["renderer"]["shadow_radius"], 0, m, S)
    sres = torch.empty((S * m, 4), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    # The profiled launches, in this order (after the primary trace and the
    # sorted trace that made the shadow rays).
    api.trace(scene, wf.BVH2_FP32, path, res)
    api.trace(scene, wf.BVH8_Q8, path, res)
    api.trace(scene, wf.BVH8_Q8, srt, res)
    api.trace(scene, wf.BVH8_Q8, srays, sres, closest_hit=False)
    api.trace(scene, wf.BVH2_FP32, srays, sres, closest_hit=False)
    torch.cuda.synchronize()
    print(json.dumps({"trace_profile": "city" if args.city else "courtyard", "resolution": [w, h],
                      "path_rays": m, "shadow_rays": S * m}))
    if args.trace_counts:
        # The same five launches through the counting kernels: node visits,
        # triangle tests and (BVH8) persistent-warp loop iterations per ray.
        forms = (("bvh2 closest", wf.BVH2_FP32, path, res, True), ("bvh8 closest unsorted", wf.BVH8_Q8, path, res, True),
                 ("bvh8 closest sorted", wf.BVH8_Q8, srt, res, True), ("bvh8 any", wf.BVH8_Q8, srays, sres, False),
                 ("bvh2 any", wf.BVH2_FP32, srays, sres, False))
        old = api.tune_get("trace.count")
        api.tune_set("trace.count", 1)
        try:
            for label, kind, rays, out, closest in forms:
                api.trace_counters(reset=True)
                api.trace(scene, kind, rays, out, closest_hit=closest)
                torch.cuda.synchronize()
                c = api.trace_counters(reset=True)
                nr = rays.shape[0]
                print(json.dumps({"form": label, "rays": nr, "hit_fraction": round(float((out[:nr, 0] >= 0).float().mean()), 3),
                                  "nodes_per_ray": round(c["nodes"] / nr, 2), "tris_per_ray": round(c["tris"] / nr, 2),
                                  "warp_iters_per_32_rays": round(c["warp_iters"] * 32 / nr, 2)}))
        finally:
            api.tune_set("trace.count", old)


def run_sweep(args):
    """Autotuner searches on the courtyard wavefronts (prints one JSON line)."""
    import torch

    import vulkanwavefrontpathtracer_gb300 as wf
    from vulkanwavefrontpathtracer_gb300 import autotune
    from vulkanwavefrontpathtracer_gb300 import build as wbuild
    wbuild.build()
    dev = torch.device("cuda", 0)
    api = wf.api
    W = COURTYARD
    pos, nrm, idx = api.generate_scene(W["scene_kind"], W["seed"])
    scene = api.Scene(pos, idx)
    geom = api.Geometry(pos, nrm, idx, device=dev)
    cam = api.make_camera(**W["camera"])
    args.width, args.height = args.width or W["width"], args.height or W["height"]
    path, shadow = make_wavefronts(wf, api, dev, scene, geom, cam, args.width, args.height, W["light"])
    keys = autotune.tune_keys(scene, path)
    best = keys["best"]
    if best["morton"] is not None and best["reorder"]:
        # tune traversal on the reordered wavefront the renderer would trace
        m = path.shape[0]
        k = torch.empty(m, dtype=torch.int64, device=dev)
        ids = torch.empty(m, dtype=torch.int32, device=dev)
        api.morton(path, scene.bounds_min, scene.bounds_max - scene.bounds_min, best["morton"], k, ids)
        api.sort_pairs(k, ids, best["key_bits"])
        out = torch.empty_like(path)
        api.reorder(ids, path, out, torch.arange(m, dtype=torch.int32, device=dev),
                    torch.empty(m, dtype=torch.int32, device=dev), torch.empty(m, dtype=torch.int32, device=dev))
        path = out
    trav = autotune.tune_traversal(scene, path, shadow)
    work = {f"{form}_{kind}": autotune.measure_work(scene, rays, bvh, closest)
            for form, bvh in (("bvh2", wf.BVH2_FP32), ("bvh8", wf.BVH8_Q8))
            for kind, rays, closest in (("path", path, True), ("shadow", shadow, False))}

    def make_renderer(mask):
        r = api.Renderer(**W["renderer"], **dict(CHOSEN, path_sort_skip=mask))
        r.set_scene(scene, geom, W["light"], W["background"])
        return r

    bounces = autotune.tune_bounce_sort(make_renderer, cam, args.width, args.height, W["renderer"]["recursion_depth"])
    mk = torch.empty(path.shape[0], dtype=torch.int64, device=dev)
    mi = torch.empty(path.shape[0], dtype=torch.int32, device=dev)
    api.morton(path, scene.bounds_min, scene.bounds_max - scene.bounds_min, wf.MORTON_6D64, mk, mi)
    sort = autotune.tune_sort(mk, 63)
    print(json.dumps({"keys": keys, "traversal": trav, "work": work, "bounce_sort": bounces, "sort": sort,
                      "resolution": [args.width, args.height]}))


def run_micro_only(args):
    import torch

    import vulkanwavefrontpathtracer_gb300 as wf
    from vulkanwavefrontpathtracer_gb300 import build as wbuild
    wbuild.build()
    dev = torch.device("cuda", 0)
    api = wf.api
    size = (args.width, args.height) if args.width and args.height else None
    if args.city:
        line, _ = city_bounce(wf, api, dev, torch.cuda.current_stream(), frames=not args.no_city_frames, size=size)
        print(json.dumps({"per_bounce_city": line}))
        return
    W = COURTYARD
    pos, nrm, idx = api.generate_scene(W["scene_kind"], W["seed"])
    scene = api.Scene(pos, idx)
    geom = api.Geometry(pos, nrm, idx, device=dev)
    cam = api.make_camera(**W["camera"])
    w, h = size or (W["width"], W["height"])
    micro = bounce_micro(wf, api, dev, scene, geom, cam, w, h, torch.cuda.current_stream())
    print(json.dumps({"micro": micro["per_bounce"], "sort_gbs": round(micro["sort"]["gbs"], 1),
                      "reorder_gbs": round(micro["reorder"]["gbs"], 1), "resolution": [w, h]}))


# ---------------------------------------------------------- CPU baseline
def cpu_frame(args, api, scene, pos, nrm, idx, w, h, form):
    import oracle
    W = COURTYARD
    nodes, tris = scene.export_bvh2()
    hg = oracle.HostGeometry(api.gltf_vertices(pos, nrm), idx)
    c = W["camera"]
    s2w = api.camera_screen_to_world(c["position"], c["rotation_deg"], c["fov_deg"], w / h, c["znear"], c["zfar"])
    R = W["renderer"]
    cfg = oracle.FrameCfg(ray_type=2, spp=1, S=R["num_shadow_samples"], depth=R["recursion_depth"],
                          radius=R["shadow_radius"], key=R["key_value"], white=R["white_point"], albedo=R["albedo"],
                          sort_shadow=form["sort_shadow_rays"], reorder_shadow=form["reorder_shadow_rays"],
                          sort_path=form["sort_path_rays"], reorder_path=form["reorder_path_rays"],
                          morton_kind=form["morton_kind"], frame_index=1)
    t0 = time.perf_counter()
    _, _, st = oracle.render_frame(nodes, tris, hg, scene.bounds_min, scene.bounds_max, W["light"],
                                   W["background"], s2w, c["position"], c["zfar"], w, h, cfg)
    dt = time.perf_counter() - t0
    return (st.primary + st.shadow + st.path), dt


def cpu_stages(wf, api, dev, scene, geom, cam, n_sample=1 << 20):
    """Per-stage CPU oracle throughput on a 1M-ray sample of the bounce-1
    path wavefront and its shadow rays (the same rays the GPU per-bounce
    line traces): Morton keys, stable sort, reorder, closest-hit and any-hit
    traversal of the FP32 BVH2."""
    import oracle
    W = COURTYARD
    path, shadow = make_wavefronts(wf, api, dev, scene, geom, cam, W["width"], W["height"], W["light"])
    p = path[:n_sample].cpu().numpy()
    s = shadow[:n_sample].cpu().numpy()
    nodes, tris = scene.export_bvh2()
    smin, ssize = scene.bounds_min, scene.bounds_max - scene.bounds_min
    th = oracle.num_threads()
    out = {}

    def timed(fn):
        t = time.perf_counter()
        r = fn()
        return r, time.perf_counter() - t

    (keys, ids), dt = timed(lambda: oracle.morton(p, smin, ssize, 2))
    out["morton_6d64"] = {"mrays_s": round(p.shape[0] / dt / 1e6, 2), "threads": th}
    (_, order), dt = timed(lambda: oracle.sort_pairs_mt(keys, ids, 63))
    out["sort_u64_63bit"] = {"mpairs_s": round(p.shape[0] / dt / 1e6, 2), "gbs": round(192.0 * p.shape[0] / dt / 1e9, 3),
                             "threads": th, "method": "LSD radix, 8-bit digits, OpenMP"}
    _, dt = timed(lambda: oracle.reorder(order, p, np.arange(p.shape[0], dtype=np.int32)))
    out["reorder"] = {"mrays_s": round(p.shape[0] / dt / 1e6, 2), "gbs": round(80.0 * p.shape[0] / dt / 1e9, 3),
                      "threads": th}
    _, dt = timed(lambda: oracle.trace_bvh2(nodes, tris, p, closest=True))
    out["trace_closest"] = {"mrays_s": round(p.shape[0] / dt / 1e6, 2), "threads": th}
    _, dt = timed(lambda: oracle.trace_bvh2(nodes, tris, s, closest=False))
    out["trace_any"] = {"mrays_s": round(s.shape[0] / dt / 1e6, 2), "threads": th}
    out["sample"] = f"{p.shape[0]} bounce-1 path rays and {s.shape[0]} shadow rays of the courtyard frame"
    return out


def cpu_baseline(args, wf, api, scene, pos, nrm, idx):
    import oracle
    w, h = COURTYARD["width"], COURTYARD["height"]
    rays, dt = cpu_frame(args, api, scene, pos, nrm, idx, w, h, CHOSEN)
    return {"value": round(rays / dt / 1e6, 3), "unit": "Mrays/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"one full {w}x{h} frame of the courtyard workload, chosen-form settings, CPU oracle with "
                      f"FP32 BVH2 traversal; {int(rays)} rays in {dt:.2f} s"}


# ---------------------------------------------------------- reference arm
def run_reference(args):
    """The reference arm: the CPU restatement of the reference's stage chain
    (oracle/, its restatement pinned to the reference's own sources) on the
    host cores, with its own scene generation, BVH2 build and camera: the
    process maps no product library.  The workload and `config` are the
    repo arm's (the courtyard at 1920x1080, chosen-form settings); each
    step renders a sample of that frame, every REF_PIXEL_STRIDE-th slot of
    its pixel table (the same camera rays, spread over the whole image), so
    that --steps 20 --warmup 5 ends within a few minutes."""
    world, rank, local = setup_dist()
    if rank != 0:
        return None
    import oracle
    W = COURTYARD
    pos, nrm, idx = oracle.generate_scene(W["scene_kind"], W["seed"])
    nodes, tris = oracle.bvh2_build(pos, idx)
    hg = oracle.HostGeometry(oracle.gltf_vertices(pos, nrm), idx)
    w, h = W["width"], W["height"]
    c = W["camera"]
    s2w = oracle.camera_screen_to_world(c["position"], c["rotation_deg"], c["fov_deg"], w / h, c["znear"], c["zfar"])
    R, F = W["renderer"], CHOSEN
    cfg = oracle.FrameCfg(ray_type=2, spp=1, S=R["num_shadow_samples"], depth=R["recursion_depth"],
                          radius=R["shadow_radius"], key=R["key_value"], white=R["white_point"], albedo=R["albedo"],
                          sort_shadow=F["sort_shadow_rays"], reorder_shadow=F["reorder_shadow_rays"],
                          sort_path=F["sort_path_rays"], reorder_path=F["reorder_path_rays"],
                          morton_kind=F["morton_kind"], frame_index=1, pixel_stride=REF_PIXEL_STRIDE)
    smin, smax = pos.min(0), pos.max(0)

    def step():
        t0 = time.perf_counter()
        _, _, st = oracle.render_frame(nodes, tris, hg, smin, smax, W["light"], W["background"], s2w, c["position"],
                                       c["zfar"], w, h, cfg)
        return st.primary + st.shadow + st.path, time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    total_rays, total_t = 0, 0.0
    for _ in range(args.steps):
        r, dt = step()
        total_rays += r
        total_t += dt
    value = total_rays / total_t / 1e6
    out = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_t / args.steps * 1e3, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scene)", "config": workload_config(idx.shape[0], world),
           "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": oracle.num_threads(),
                            "kind": "port",
                            "sample": f"each step every {REF_PIXEL_STRIDE}th pixel-table slot of the {w}x{h} "
                                      f"courtyard frame ({int(total_rays / args.steps)} rays), rendered by the CPU "
                                      "restatement of the reference shaders (pinned to their sources) with its own "
                                      "BVH2; the reference's Vulkan/rayQuery path is unavailable on this box"},
           "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return out


# Batched serving workload: 64 requests over 4 seeded scenes (65,536-triangle
# soup, the 268,304-triangle courtyard, a ~1M-triangle and the 3M-triangle
# city block), resolutions drawn from {128^2, 256^2, 512^2, 1024^2}, 1-16
# samples per pixel and depth 1-8, path rays, chosen form.
BATCH_SCENES = [
    dict(kind=0, seed=1, ntris=65536, light=(0.5, 1.6, 0.5), background=(0.53, 0.81, 0.98),
         camera=dict(position=(0.5, 0.5, 2.2), rotation_deg=(0.0, 0.0, 0.0), fov_deg=45.0, znear=0.001,
                     zfar=10.0)),
    dict(kind=1, seed=1, ntris=0, light=COURTYARD["light"], background=COURTYARD["background"],
         camera=COURTYARD["camera"]),
    dict(kind=3, seed=1, ntris=1000000, light=(185.0, 300.0, 185.0), background=(0.53, 0.81, 0.98),
         camera=dict(position=(185.0, 60.0, 420.0), rotation_deg=(-12.0, 0.0, 0.0), fov_deg=60.0, znear=0.1,
                     zfar=2000.0)),
    dict(kind=2, seed=1, ntris=0, light=(320.0, 400.0, 320.0), background=(0.53, 0.81, 0.98),
         camera=dict(position=(320.0, 80.0, 720.0), rotation_deg=(-12.0, 0.0, 0.0), fov_deg=60.0, znear=0.1,
                     zfar=3000.0)),
]


def batch_requests(seed=7, count=64):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        res = int(rng.choice([128, 256, 512, 1024]))
        out.append(dict(scene=int(rng.integers(0, 4)), width=res, height=res, spp=int(rng.integers(1, 17)),
                        depth=int(rng.integers(1, 9))))
    return out


def batched_serving(api, dev, stream, count=64, steps=10, warmup=3):
    """One step = one frame of all `count` requests: batched (one graph
    replay, 4 branches) against the same requests rendered one after another
    through standalone renderers with every stage launched directly."""
    import torch
    scenes = []
    for s in BATCH_SCENES:
        pos, nrm, idx = api.generate_scene(s["kind"], s["seed"], s["ntris"])
        scenes.append((api.Scene(pos, idx), api.Geometry(pos, nrm, idx, device=dev), int(idx.shape[0])))
    specs = batch_requests(count=count)
    reqs, solos = [], []
    for q in specs:
        s = BATCH_SCENES[q["scene"]]
        sc, geom, _ = scenes[q["scene"]]
        over = dict(COURTYARD["renderer"], num_primary_samples=q["spp"], recursion_depth=q["depth"],
                    shadow_radius=COURTYARD["renderer"]["shadow_radius"] if q["scene"] != 0 else 0.1)
        n = q["width"] * q["height"]
        px = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        reqs.append(dict(scene=sc, geometry=geom, light=s["light"], background=s["background"],
                         camera=api.make_camera(**s["camera"]), width=q["width"], height=q["height"],
                         config=api.default_config(**over, **CHOSEN), pixels=px, frame_pixels=fp))
        solo = api.Renderer(**over, **dict(CHOSEN, use_graph=0))
        solo.set_scene(sc, geom, s["light"], s["background"])
        solos.append((solo, api.make_camera(**s["camera"]), q["width"], q["height"], px, fp))
    batch = api.Batch(reqs, streams=4)

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps

    def solo_all():
        for r, cam, w, h, px, fp in solos:
            r.render(cam, w, h, px, fp)

    ms_batch = timed(batch.render, steps, warmup)
    rays = sum(st.num_primary_rays + st.num_shadow_rays + st.num_path_rays
               for st in (batch.stats(i) for i in range(len(reqs))))
    ms_solo = timed(solo_all, max(1, steps // 2), 1)
    out = {"metric": "Mrays/s, batched render requests (chosen form)", "value": round(rays / (ms_batch * 1e-3) / 1e6, 3),
           "unit": "Mrays/s", "ms_per_step": round(ms_batch, 3), "steps": steps, "warmup": warmup,
           "requests": len(reqs), "rays_per_step": int(rays), "graph_kernels": batch.kernels(),
           "unbatched": {"value": round(rays / (ms_solo * 1e-3) / 1e6, 3), "ms_per_step": round(ms_solo, 3)},
           "batched_over_unbatched": round(ms_solo / ms_batch, 3),
           "scenes_triangles": [s[2] for s in scenes],
           "requests_by_resolution": {str(r): sum(1 for q in specs if q["width"] == r) for r in (128, 256, 512, 1024)}}
    batch.close()
    for r, *_ in solos:
        r.close()
    return out


def run_batched(args):
    import torch

    import vulkanwavefrontpathtracer_gb300 as wf
    from vulkanwavefrontpathtracer_gb300 import build as wbuild
    wbuild.build()
    dev = torch.device("cuda", 0)
    print(json.dumps(batched_serving(wf.api, dev, torch.cuda.current_stream(), args.batch_requests, args.steps,
                                     args.warmup)))


def sort_row(api, dev, stream, n=1 << 26, reps=5):
    """Radix sorts of n uniform random pairs, u64 keys (63 bits, 8 passes)
    and u32 keys (4 passes), u32 values: algorithmic GB/s (passes x 2 x
    (key + value bytes) per pair) against the measured HBM peak."""
    import torch
    hbm, _ = peaks()
    gen = torch.Generator(device=dev)
    out = {"pairs": n}
    for bits in (63, 32):
        wide = bits > 32
        gen.manual_seed(n + bits)
        src = torch.randint(0, (1 << 62) if wide else (1 << 32), (n,), generator=gen, device=dev, dtype=torch.int64)
        src = (src * 2 + (src & 1)) if wide else src.to(torch.int32)
        keys = torch.empty_like(src)
        vals = torch.arange(n, dtype=torch.int32, device=dev)
        scratch = torch.empty(api.sort_scratch_bytes(n, 64 if wide else 32), dtype=torch.uint8, device=dev)

        def timed(fn):
            for _ in range(2):
                fn()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            return a.elapsed_time(b) / reps

        ms = timed(lambda: (keys.copy_(src), api.sort_pairs(keys, vals, bits, scratch=scratch)))
        ms -= timed(lambda: keys.copy_(src))
        passes = (bits + 7) // 8
        gbs = passes * 2 * ((8 if wide else 4) + 4) * n / (ms * 1e-3) / 1e9
        out["u64" if wide else "u32"] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / hbm, 3),
                                         "alg_bytes_per_pair": passes * 2 * ((8 if wide else 4) + 4)}
        del src, keys, vals, scratch
        torch.cuda.empty_cache()
    return out


def reorder_row(api, dev, stream, n=1 << 24, reps=5):
    """The reorder gather beyond L2: n random-order rays gathered by the
    permutation that sorts them (32-byte records with the slot maps, 80 B
    per ray; and 48-byte records, 112 B per ray), algorithmic GB/s against
    the measured HBM peak."""
    import torch
    hbm, _ = peaks()
    gen = torch.Generator(device=dev)
    gen.manual_seed(n)
    perm = torch.randperm(n, generator=gen, device=dev).to(torch.int32)
    rays = torch.rand((n, 8), generator=gen, device=dev)
    out = torch.empty_like(rays)
    s2i = torch.arange(n, dtype=torch.int32, device=dev)
    os2i = torch.empty(n, dtype=torch.int32, device=dev)
    oi2s = torch.empty(n, dtype=torch.int32, device=dev)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    res = {"rays": n}
    ms = timed(lambda: api.reorder(perm, rays, out, s2i, os2i, oi2s))
    res["ray32"] = {"ms": round(ms, 4), "gbs": round(80.0 * n / (ms * 1e-3) / 1e9, 1),
                    "frac": round(80.0 * n / (ms * 1e-3) / 1e9 / hbm, 3), "alg_bytes_per_ray": 80}
    del out
    wide = torch.cat([rays, rays[:, :4]], dim=1).contiguous()
    wide_out = torch.empty_like(wide)
    ms = timed(lambda: api.reorder_records(perm, wide, wide_out, s2i, os2i, oi2s))
    res["rec48"] = {"ms": round(ms, 4), "gbs": round(112.0 * n / (ms * 1e-3) / 1e9, 1),
                    "frac": round(112.0 * n / (ms * 1e-3) / 1e9 / hbm, 3), "alg_bytes_per_ray": 112}
    res["note"] = ("random 32/48-byte record gathers and 4-byte slot-map accesses: about 3.7x the algorithmic "
                   "bytes reach DRAM (sector and burst granularity), the kernel's ceiling beyond L2")
    del rays, wide, wide_out, perm, s2i, os2i, oi2s
    torch.cuda.empty_cache()
    return res


def run_sort_micro(args):
    """Sort / reorder microbenchmark: stable key-value sorts of 2^16..2^26
    pairs, u32 and u64 keys, uniform random keys and Morton keys of
    clustered 6-D Gaussian rays (origins and directions), plus the reorder
    gather of 32-byte ray records; algorithmic GB/s against the measured HBM
    peak (passes x 2 x (key + value bytes) per pair for the sort, 80 B per
    ray for the reorder)."""
    import torch

    import vulkanwavefrontpathtracer_gb300 as wf
    from vulkanwavefrontpathtracer_gb300 import build as wbuild
    wbuild.build()
    api = wf.api
    dev = torch.device("cuda", 0)
    hbm, peak_kind = peaks()
    stream = torch.cuda.current_stream()
    sizes = [int(s) for s in args.sort_sizes.split(",")]
    gen = torch.Generator(device=dev)

    def timeit(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    def clustered_rays(n):
        # 64 Gaussian clusters in 6-D: origins in the unit cube, directions
        # around a cluster axis.
        gen.manual_seed(n)
        c = torch.randint(0, 64, (n,), generator=gen, device=dev)
        co = torch.rand((64, 3), generator=gen, device=dev)
        cd = torch.nn.functional.normalize(torch.randn((64, 3), generator=gen, device=dev), dim=1)
        o = (co[c] + 0.05 * torch.randn((n, 3), generator=gen, device=dev)).clamp(0, 1)
        d = torch.nn.functional.normalize(cd[c] + 0.2 * torch.randn((n, 3), generator=gen, device=dev), dim=1)
        r = torch.zeros((n, 8), dtype=torch.float32, device=dev)
        r[:, :3] = o
        r[:, 4:7] = d
        r[:, 7] = 1e30
        return r

    rows = []
    for n in sizes:
        rays = clustered_rays(n)
        reps = 20 if n <= (1 << 22) else 5
        for bits in (32, 63):
            wide = bits > 32
            kdt = torch.int64 if wide else torch.int32
            keys = torch.empty(n, dtype=kdt, device=dev)
            ids = torch.empty(n, dtype=torch.int32, device=dev)
            scratch = torch.empty(api.sort_scratch_bytes(n, 64 if wide else 32), dtype=torch.uint8, device=dev)
            for dist in ("uniform", "clustered"):
                if dist == "uniform":
                    gen.manual_seed(n + bits)
                    src = torch.randint(0, (1 << 62) if wide else (1 << 32), (n,), generator=gen, device=dev,
                                        dtype=torch.int64)
                    src = (src * 2 + (src & 1)) if wide else src.to(torch.int32)
                else:
                    kind = wf.MORTON_6D64 if wide else wf.MORTON_AILA32
                    api.morton(rays, [0, 0, 0], [1, 1, 1], kind, keys, ids)
                    src = keys.clone()
                vals = torch.arange(n, dtype=torch.int32, device=dev)

                def one():
                    keys.copy_(src)
                    api.sort_pairs(keys, vals, bits, scratch=scratch)

                copy_ms = timeit(lambda: keys.copy_(src), reps)
                ms = max(timeit(one, reps) - copy_ms, 1e-6)
                passes = (bits + 7) // 8
                alg = passes * 2 * ((8 if wide else 4) + 4) * n
                rows.append({"n": n, "key_bits": bits, "keys": dist, "ms": round(ms, 4),
                             "gbs": round(alg / (ms * 1e-3) / 1e9, 1), "frac": round(alg / (ms * 1e-3) / 1e9 / hbm, 3)})
        # Reorder gather of 32-byte ray records by a sorted permutation.
        # ... by the permutation that sorts the clustered rays' 64-bit keys,
        # as in the pipeline (Morton -> sort -> reorder).
        api.morton(rays, [0, 0, 0], [1, 1, 1], wf.MORTON_6D64, keys, ids)
        api.sort_pairs(keys, ids, 63, scratch=scratch)
        perm = ids
        out = torch.empty_like(rays)
        s2i = torch.arange(n, dtype=torch.int32, device=dev)
        os2i = torch.empty(n, dtype=torch.int32, device=dev)
        oi2s = torch.empty(n, dtype=torch.int32, device=dev)
        ms = timeit(lambda: api.reorder(perm, rays, out, s2i, os2i, oi2s), reps)
        rows.append({"n": n, "reorder_ms": round(ms, 4), "reorder_gbs": round(80.0 * n / (ms * 1e-3) / 1e9, 1),
                     "reorder_frac": round(80.0 * n / (ms * 1e-3) / 1e9 / hbm, 3)})
        # The same gather of 48-byte records (the ray plus a 16-byte
        # payload) with the slot maps: 4 + 4 + 48 B read, 48 + 4 + 4 B
        # written per ray.
        wide = torch.cat([rays, rays[:, :4]], dim=1).contiguous()
        wide_out = torch.empty_like(wide)
        del out
        ms = timeit(lambda: api.reorder_records(perm, wide, wide_out, s2i, os2i, oi2s), reps)
        rows.append({"n": n, "reorder48_ms": round(ms, 4), "reorder48_gbs": round(112.0 * n / (ms * 1e-3) / 1e9, 1),
                     "reorder48_frac": round(112.0 * n / (ms * 1e-3) / 1e9 / hbm, 3)})
        del rays, keys, ids, scratch, wide, wide_out
        torch.cuda.empty_cache()
    print(json.dumps({"sort_micro": rows, "peak_gbs": hbm, "peak_source": f"{peak_kind} hbm_gbs",
                      "sort_tiles": api.tune_get("sort.tiles")}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--micro-only", action="store_true",
                    help="only the bounce-1 microbenchmark (small profiling case with --width/--height)")
    ap.add_argument("--city", action="store_true",
                    help="with --micro-only: the bounce-1 comparison and whole frames on the city block at 3840x2160")
    ap.add_argument("--no-city-frames", action="store_true", help="with --city: the bounce-1 comparison only")
    ap.add_argument("--width", type=int, default=None, help="with --micro-only: resolution of the bounce")
    ap.add_argument("--height", type=int, default=None)
    ap.add_argument("--sweep", action="store_true", help="run the autotuner searches and print their tables")
    ap.add_argument("--sort-micro", action="store_true", help="sort/reorder microbenchmark over --sort-sizes")
    ap.add_argument("--sort-sizes", default="65536,262144,1048576,2073600,4194304,16777216,67108864")
    ap.add_argument("--scene-build", action="store_true",
                    help="acceleration-structure build times only (host vs device; courtyard and city)")
    ap.add_argument("--batched", action="store_true", help="the 64-request batched serving workload")
    ap.add_argument("--trace-profile", action="store_true",
                    help="each traversal form launched once on a small bounce-1 case (for kernel profiles)")
    ap.add_argument("--trace-counts", action="store_true",
                    help="with --trace-profile: node visits and triangle tests per ray of each form (counting kernels)")
    ap.add_argument("--batch-requests", type=int, default=64)
    args = ap.parse_args()
    if args.batched:
        run_batched(args)
        return
    if args.trace_profile:
        run_trace_profile(args)
        return
    if args.scene_build:
        import torch

        import vulkanwavefrontpathtracer_gb300 as wf
        from vulkanwavefrontpathtracer_gb300 import build as wbuild
        wbuild.build()
        torch.cuda.set_device(0)
        W = COURTYARD
        pos, nrm, idx = wf.api.generate_scene(W["scene_kind"], W["seed"])
        print(json.dumps({"scene_build": scene_build_times(wf.api, pos, idx, wf.api.Scene(pos, idx))}))
        return
    if args.sweep:
        run_sweep(args)
        return
    if args.sort_micro:
        run_sort_micro(args)
        return
    if args.micro_only:
        run_micro_only(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
