"""The CPU oracle against the known-answer vectors in tests/golden/
(generated by tests/golden/make_golden.py from the shader formulas)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def test_tea_seeds(orc):
    for i, frame, expect in GOLDEN["tea"]:
        if i >= 1 << 20:
            continue
        seeds = orc.init_seeds(i + 1, frame)
        assert int(seeds[i]) == expect


def test_sobol2d(orc):
    for i, x, y in GOLDEN["sobol2d"]:
        assert orc.sobol2d(i) == (pytest.approx(x, abs=0), pytest.approx(y, abs=0))


def test_pixel_table(orc):
    for key, expect in GOLDEN["pixel_table"].items():
        w, h = map(int, key.split("x"))
        i2p, p2i = orc.pixel_table(w, h)
        assert i2p.tolist() == expect
        assert np.array_equal(p2i[i2p], np.arange(w * h))


def test_morton_aila32(orc):
    for o, d, smin, ssize, expect in GOLDEN["morton_aila32"]:
        rays = np.zeros((1, 8), np.float32)
        rays[0, :3] = o
        rays[0, 4:7] = d
        keys, idx = orc.morton(rays, smin, ssize, 0)
        assert int(keys[0]) == expect
        assert int(idx[0]) == 0


def test_morton_6d_layout(orc):
    # Origin at the scene minimum, direction +x: only the direction bits of
    # x (all ones) and y, z (mid-scale) survive.
    rays = np.zeros((1, 8), np.float32)
    rays[0, 4] = 1.0
    k64, _ = orc.morton(rays, [0, 0, 0], [1, 1, 1], 2)
    ibx, iby = 1023, int(np.float32(0.5) * np.float32(1023))
    expect = 0
    for lvl in range(10):
        expect |= ((ibx >> lvl) & 1) << (6 * lvl + 2)
        expect |= ((iby >> lvl) & 1) << (6 * lvl + 1)
        expect |= ((iby >> lvl) & 1) << (6 * lvl + 0)
    assert int(k64[0]) == expect
    # Origin at the maximum: every origin bit set, including level 10.
    rays[0, :3] = 1.0
    k64, _ = orc.morton(rays, [0, 0, 0], [1, 1, 1], 2)
    for lvl in range(10):
        assert (int(k64[0]) >> (6 * lvl + 3)) & 7 == 7
    assert (int(k64[0]) >> 60) & 7 == 7
    k48, _ = orc.morton(rays, [0, 0, 0], [1, 1, 1], 1)
    for lvl in range(8):
        assert (int(k48[0]) >> (6 * lvl + 3)) & 7 == 7
    assert int(k48[0]) < (1 << 48)


def test_sort_is_stable(orc):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 16, size=5000, dtype=np.uint32)
    vals = np.arange(5000, dtype=np.uint32)
    k, v = orc.sort_pairs(keys, vals, 32)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, order.astype(np.uint32))
    # only the low key_bits bits count
    k2, v2 = orc.sort_pairs(keys | np.uint32(0xF0), vals, 4)
    assert np.array_equal(v2, order.astype(np.uint32))


def test_reorder_records_matches_reorder(orc):
    # The wide-record gather is the 32-byte reorder at record_bytes 32, and a
    # plain row gather (with the same slot maps) at 48.
    rng = np.random.default_rng(5)
    n = 1000
    idx = rng.permutation(n).astype(np.uint32)
    s2i = rng.permutation(n).astype(np.int32)
    rays = rng.standard_normal((n, 8)).astype(np.float32)
    a, a_s2i, a_i2s = orc.reorder(idx, rays, s2i)
    b, b_s2i, b_i2s = orc.reorder_records(idx, rays, s2i)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(a_s2i, b_s2i) and np.array_equal(a_i2s, b_i2s)
    wide = rng.integers(0, 2**32, size=(n, 12), dtype=np.uint32)
    c, c_s2i, c_i2s = orc.reorder_records(idx, wide, s2i)
    assert np.array_equal(c, wide[idx]) and np.array_equal(c_s2i, a_s2i) and np.array_equal(c_i2s, a_i2s)
    d, d_s2i, _ = orc.reorder_records(idx, wide)
    assert np.array_equal(d, wide[idx]) and d_s2i is None


def test_reinhard(orc):
    for c, key, white, expect in GOLDEN["reinhard"]:
        fp = np.array([[*c, 1.0]], np.float32)
        out, px = orc.interpolate_colors(fp, np.zeros((1, 4), np.float32), 1, key, white)
        assert np.allclose(out[0, :3], expect, rtol=2e-5, atol=2e-6)
        assert np.array_equal(px[0], fp[0])


def test_sincos_2pi(orc):
    for r, s, c in GOLDEN["sincos_2pi"]:
        got = orc.sincos_2pi(r)
        assert abs(got[0] - s) < 4e-7 and abs(got[1] - c) < 4e-7


def test_shadow_ray_layout(orc):
    # raygenShadow.comp:100-133: S rays per input, slot maps identity, a
    # miss produces dummy rays with tmax = -1.
    rays = np.zeros((2, 8), np.float32)
    rays[:, 4] = 1.0
    rays[:, 7] = 100.0
    res = np.array([[5, 0, np.float32(2.0).view(np.int32), 0], [-1, -1, np.float32(-1.0).view(np.int32), 0]], np.int32)
    seeds = np.array([11, 22], np.uint32)
    out, s2i, i2s = orc.raygen_shadow(seeds, rays, res, [0, 10, 0], 1.0, 0, 2, 3)
    assert out.shape == (6, 8)
    assert np.array_equal(s2i, np.arange(6)) and np.array_equal(i2s, np.arange(6))
    assert np.allclose(out[:3, 0], 2.0 - 1e-5)
    assert np.all(out[:3, 3] == np.float32(1e-5))
    lens = np.linalg.norm(out[:3, 4:7], axis=1)
    assert np.allclose(lens, 1.0, atol=1e-6)
    assert np.all(out[3:, 7] == -1.0) and np.all(out[3:, 4] == 1.0) and np.all(out[3:, :3] == 0)


def test_oracle_matches_reference_vectors(wf, orc):
    """The oracle against outputs of the reference's own sources compiled for
    the CPU (tests/golden/ref_vectors.npz), stage by stage."""
    import refvectors as rv

    def geom(pos, nrm, idx):
        return orc.HostGeometry(wf.api.gltf_vertices(pos, nrm), idx)

    impl = {
        "init_seeds": orc.init_seeds,
        "pixel_table": orc.pixel_table,
        "camera": orc.camera_screen_to_world,
        "raygen_primary": orc.raygen_primary,
        "morton_aila32": lambda r, a, b: orc.morton(r, a, b, 0),
        "reorder": orc.reorder,
        "raygen_shadow": orc.raygen_shadow,
        "raygen_path": lambda pos, nrm, idx, s, r, i2p, res, dec: orc.raygen_path(s, geom(pos, nrm, idx), r, i2p, res,
                                                                                  dec, albedo=0.8),
        "reconstruct_smooth": lambda pos, nrm, idx, r, res, i2p, px, dec, light, bg, spp: orc.reconstruct_smooth(
            r, res, i2p, px, dec, geom(pos, nrm, idx), light, bg, spp),
        "reconstruct_shadow": orc.reconstruct_shadow,
        "count_hits": orc.count_hits,
        "interpolate_colors": orc.interpolate_colors,
    }
    assert rv.check_all(impl) == rv.ALL_STAGES
