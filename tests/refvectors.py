"""Comparison of one implementation of the stage functions against
tests/golden/ref_vectors.npz, the outputs of the reference's own sources
compiled for the CPU (written by tests/golden/make_ref_golden.py).

`impl` maps stage names to callables taking numpy inputs and returning numpy
outputs; the oracle (CPU tests) and the CUDA kernels through the C ABI (GPU
tests) each provide one.  Bars: bit-exact everywhere except the bounce
direction of raygen_path (the reference calls sinf/cosf on a rounded
argument: each direction component within 2^-20, the origin within 2^-21
relative to the hit point) and the camera matrix (within 1e-6 of its
largest element).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_vectors.npz"


def load():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def same_bits_nan_aware(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(bits(np.where(na, 0, a)), bits(np.where(nb, 0, b)))


def check_all(impl, v=None):
    """Runs every stage `impl` provides against the vectors; returns the
    names of the stages checked."""
    v = load() if v is None else v
    done = []

    if "init_seeds" in impl:
        assert np.array_equal(impl["init_seeds"](int(v["seeds_n"]), int(v["seeds_frame"])), v["seeds_out"])
        done.append("init_seeds")

    if "pixel_table" in impl:
        for w, h in ((61, 37), (130, 17)):
            a, b = impl["pixel_table"](w, h)
            assert np.array_equal(a, v[f"pixel_table_{w}x{h}_i2p"]) and np.array_equal(b, v[f"pixel_table_{w}x{h}_p2i"])
        done.append("pixel_table")

    if "camera" in impl:
        for c, ref in zip(v["camera_in"], v["camera_out"]):
            m = np.asarray(impl["camera"](c[0:3], c[3:6], float(c[6]), float(c[7]), float(c[8]), float(c[9])),
                           np.float32).reshape(16)
            assert np.abs(m - ref).max() <= 1e-6 * np.abs(ref).max()
        done.append("camera")

    if "raygen_primary" in impl:
        i2p = v["pixel_table_61x37_i2p"]
        rays = impl["raygen_primary"](v["camera_out"][1], i2p, v["camera_in"][1, 0:3], 3, 61, 37, 300.0)
        assert np.array_equal(bits(rays), bits(v["primary_out"]))
        done.append("raygen_primary")

    if "morton_aila32" in impl:
        k, i = impl["morton_aila32"](v["morton_rays"], v["morton_smin"], v["morton_ssize"])
        assert np.array_equal(k, v["morton_keys"]) and np.array_equal(i, v["morton_idx"])
        done.append("morton_aila32")

    if "reorder" in impl:
        o, s, i = impl["reorder"](v["reorder_idx"], v["reorder_rays"], v["reorder_s2i"])
        assert np.array_equal(bits(o), bits(v["reorder_out"]))
        assert np.array_equal(s, v["reorder_out_s2i"]) and np.array_equal(i, v["reorder_out_i2s"])
        done.append("reorder")

    if "raygen_shadow" in impl:
        o, s, i = impl["raygen_shadow"](v["shadow_seeds"], v["shadow_rays"], v["shadow_res"], v["shadow_light"],
                                        float(v["shadow_radius"]), int(v["shadow_bb"]), int(v["shadow_bs"]),
                                        int(v["shadow_S"]))
        assert np.array_equal(bits(o), bits(v["shadow_out"]))
        assert np.array_equal(s, v["shadow_out_s2i"]) and np.array_equal(i, v["shadow_out_i2s"])
        done.append("raygen_shadow")

    if "raygen_path" in impl:
        seeds, rays, i2p, dec, cnt = impl["raygen_path"](v["scene_pos"], v["scene_nrm"], v["scene_idx"],
                                                         v["path_seeds"], v["path_rays"], v["path_i2p"],
                                                         v["path_res"], v["path_dec"])
        assert cnt == int(v["path_count"])
        assert np.array_equal(seeds, v["path_out_seeds"])
        assert np.array_equal(i2p, v["path_out_i2p"])
        assert np.array_equal(bits(dec), bits(v["path_out_dec"]))
        ref = v["path_out_rays"]
        assert np.array_equal(bits(rays[:, 3]), bits(ref[:, 3])) and np.array_equal(bits(rays[:, 7]), bits(ref[:, 7]))
        assert np.abs(rays[:, 4:7] - ref[:, 4:7]).max() <= 2.0**-20
        scale = np.maximum(np.abs(ref[:, 0:3]), 1.0)
        assert (np.abs(rays[:, 0:3] - ref[:, 0:3]) / scale).max() <= 2.0**-21
        done.append("raygen_path")

    if "reconstruct_smooth" in impl:
        px = impl["reconstruct_smooth"](v["scene_pos"], v["scene_nrm"], v["scene_idx"], v["path_rays"], v["path_res"],
                                        v["path_i2p"], v["smooth_pixels"], v["path_dec"], v["smooth_light"],
                                        v["smooth_bg"], int(v["smooth_spp"]))
        assert np.array_equal(bits(px), bits(v["smooth_out"]))
        done.append("reconstruct_smooth")

    if "reconstruct_shadow" in impl:
        out = impl["reconstruct_shadow"](v["rshadow_res"], v["rshadow_i2p"], v["rshadow_i2s"], v["rshadow_in"],
                                         v["rshadow_prev"], int(v["rshadow_bb"]), int(v["rshadow_bs"]),
                                         int(v["rshadow_S"]))
        assert np.array_equal(bits(out), bits(v["rshadow_out"]))
        done.append("reconstruct_shadow")

    if "count_hits" in impl:
        assert impl["count_hits"](v["rshadow_res"]) == int(v["count_hits"])
        done.append("count_hits")

    if "interpolate_colors" in impl:
        for frame in (1, 3):
            a, b = impl["interpolate_colors"](v["interp_frame"], v["interp_prev"], frame, 0.18, 3.0)
            assert same_bits_nan_aware(a, v[f"interp_out_frame_{frame}"])
            assert same_bits_nan_aware(b, v[f"interp_out_pixels_{frame}"])
        done.append("interpolate_colors")
    return done


ALL_STAGES = ["init_seeds", "pixel_table", "camera", "raygen_primary", "morton_aila32", "reorder", "raygen_shadow",
              "raygen_path", "reconstruct_smooth", "reconstruct_shadow", "count_hits", "interpolate_colors"]
