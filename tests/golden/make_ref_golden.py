"""Writes tests/golden/ref_vectors.npz: inputs and outputs of the reference's
own shader and host sources, compiled for the CPU (oracle/_ref/libref.so,
built by oracle/ref_build.py from the reference checkout).  The file lets
the oracle (CPU tests) and the CUDA kernels (GPU tests) be checked against
reference-executed outputs where the reference checkout is absent, as on a
GPU machine.

Run from the repository root: python tests/golden/make_ref_golden.py
Every input is seeded; the scene is the library's triangle-soup generator
(kind 0, seed 21, 200 triangles) in its host form.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

OUT = Path(__file__).resolve().parent / "ref_vectors.npz"


def rays_of(rng, n, lo, hi, tmax=10.0):
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, :3], r[:, 4:7], r[:, 7] = o, d, tmax
    return r


def main() -> None:
    import oracle
    import oracle.ref as ref
    import vulkanwavefrontpathtracer_gb300 as wf

    wf._lib.load()
    rng = np.random.default_rng(20260312)
    v: dict[str, np.ndarray] = {}

    v["seeds_n"], v["seeds_frame"] = np.int32(3001), np.int32(5)
    v["seeds_out"] = ref.init_seeds(3001, 5)

    for w, h in ((61, 37), (130, 17)):
        a, b = ref.pixel_table(w, h)
        v[f"pixel_table_{w}x{h}_i2p"], v[f"pixel_table_{w}x{h}_p2i"] = a, b

    cams = np.array([[15, 6, 19.5, 0, 0, 0, 60.0, 16 / 9, 0.1, 512.0],
                     [3, 2, 9, 10, 25, 0, 60.0, 61 / 37, 0.1, 300.0],
                     [-4, 1, 2, 30, -20, 10, 45.0, 1.0, 0.5, 100.0],
                     [0.5, 0.5, 2.5, -10, 20, 5, 45.0, 4 / 3, 0.001, 3.0]], np.float32)
    v["camera_in"] = cams
    v["camera_out"] = np.stack([ref.camera_screen_to_world(c[0:3], c[3:6], c[6], c[7], c[8], c[9])[0] for c in cams])

    i2p, _ = ref.pixel_table(61, 37)
    m = v["camera_out"][1]
    v["primary_out"] = ref.raygen_primary(m, i2p, cams[1, 0:3], 3, 61, 37, 300.0)

    mr = rays_of(rng, 1024, -0.3, 1.3)
    mr[:64, 4:7] *= 3.0  # unnormalised directions
    v["morton_rays"], v["morton_smin"], v["morton_ssize"] = mr, np.float32([0.05, -0.1, 0.2]), np.float32([0.9, 1.1, 0.7])
    v["morton_keys"], v["morton_idx"] = ref.morton_aila32(mr, v["morton_smin"], v["morton_ssize"])

    n = 512
    rr = rays_of(rng, n, 0, 1)
    v["reorder_rays"], v["reorder_idx"] = rr, rng.permutation(n).astype(np.uint32)
    v["reorder_s2i"] = rng.permutation(n).astype(np.int32)
    v["reorder_out"], v["reorder_out_s2i"], v["reorder_out_i2s"] = ref.reorder(v["reorder_idx"], rr, v["reorder_s2i"])

    pos, nrm, idx = wf.api.generate_scene(0, 21, 200)
    v["scene_pos"], v["scene_nrm"], v["scene_idx"] = pos, nrm, idx
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, tris = sc.export_bvh2()
    geom = oracle.HostGeometry(wf.api.gltf_vertices(pos, nrm), idx)

    sr = rays_of(rng, 512, -0.5, 1.5)
    sres = oracle.trace_bvh2(nodes, tris, sr)
    v["shadow_rays"], v["shadow_res"] = sr, sres
    v["shadow_seeds"] = rng.integers(0, 2**32, 512, dtype=np.uint32)
    v["shadow_light"], v["shadow_radius"] = np.float32([0.3, 2.0, 0.4]), np.float32(0.25)
    v["shadow_bb"], v["shadow_bs"], v["shadow_S"] = np.int32(100), np.int32(300), np.int32(3)
    v["shadow_out"], v["shadow_out_s2i"], v["shadow_out_i2s"] = ref.raygen_shadow(
        v["shadow_seeds"], sr, sres, v["shadow_light"], 0.25, 100, 300, 3)

    pr = rays_of(rng, n, -0.5, 1.5)
    pres = oracle.trace_bvh2(nodes, tris, pr)
    v["path_rays"], v["path_res"] = pr, pres
    v["path_seeds"] = rng.integers(0, 2**32, n, dtype=np.uint32)
    v["path_i2p"] = rng.permutation(n).astype(np.int32)
    v["path_dec"] = rng.uniform(0.1, 1.0, (n, 4)).astype(np.float32)
    s, o, oi, d, c = ref.raygen_path(v["path_seeds"], geom.table, pr, v["path_i2p"], pres, v["path_dec"])
    v["path_out_seeds"], v["path_out_rays"], v["path_out_i2p"], v["path_out_dec"] = s, o, oi, d
    v["path_count"] = np.int32(c)

    v["smooth_pixels"] = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    v["smooth_light"], v["smooth_bg"], v["smooth_spp"] = np.float32([0.5, 3.0, 0.2]), np.float32([0.2, 0.3, 0.9]), np.int32(2)
    v["smooth_out"] = ref.reconstruct_smooth(pr, pres, v["path_i2p"], v["smooth_pixels"], v["path_dec"], geom.table,
                                             v["smooth_light"], v["smooth_bg"], 2)

    bs, S = 350, 3
    ns = bs * S
    shres = np.full((ns, 4), -1, np.int32)
    shres[rng.uniform(size=ns) < 0.4, 0] = 5
    v["rshadow_res"], v["rshadow_i2s"] = shres, rng.permutation(ns).astype(np.int32)
    v["rshadow_i2p"] = rng.permutation(n).astype(np.int32)
    v["rshadow_in"] = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    v["rshadow_prev"] = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    v["rshadow_bb"], v["rshadow_bs"], v["rshadow_S"] = np.int32(100), np.int32(bs), np.int32(S)
    v["rshadow_out"] = ref.reconstruct_shadow(shres, v["rshadow_i2p"], v["rshadow_i2s"], v["rshadow_in"],
                                              v["rshadow_prev"], 100, bs, S, False)
    v["count_hits"] = np.int32(ref.count_hits(shres))

    fp = rng.uniform(0, 4, (n, 4)).astype(np.float32)
    fp[:8] = 0.0  # black pixels: the tone map's 0/0
    pp = rng.uniform(0, 4, (n, 4)).astype(np.float32)
    v["interp_frame"], v["interp_prev"] = fp, pp
    for frame in (1, 3):
        a, b = ref.interpolate_colors(fp, pp, frame, 0.18, 3.0)
        v[f"interp_out_frame_{frame}"], v[f"interp_out_pixels_{frame}"] = a, b

    np.savez_compressed(OUT, **v)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(v)} arrays)")


if __name__ == "__main__":
    main()
