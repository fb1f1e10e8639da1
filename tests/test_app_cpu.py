"""Front end without a GPU: env.json options (the reference's registered
keys and defaults), the glTF loader and the image writers."""
import base64
import json

import numpy as np
import pytest


@pytest.fixture(scope="module")
def app(wf):
    from vulkanwavefrontpathtracer_gb300 import app
    return app


ENV = {
    "Application": {"mode": "benchmark"},
    "Benchmark": {"printSortLogs": True},
    "Resolution": {"width": 320, "height": 200},
    "Scene": {"generator": "soup:4096:3", "light": "1.0 2.0 3.0", "backgroundcolor": "0.1 0.2 0.3",
              "headlight": False},
    "Renderer": {"numberOfPrimarySamples": 2, "numberOfShadowSamples": 3, "shadowRadius": 0.5, "rayType": "path",
                 "recursionDepth": 5, "keyValue": 0.5, "whitePoint": 1.5, "russianRoulette": False,
                 "sortShadowRays": True, "reorderShadowRays": False, "sortPathRays": True,
                 "reorderPathRays": True, "mortonKind": "6d64", "bvh": "bvh8"},
    "Camera": {"position": "0.5 0.5 2.2", "rotation": "0 0 0", "nearPlane": 0.01, "farPlane": 9.0,
               "fieldOfView": 50.0},
}


def test_env_options_and_defaults(app):
    o = app.load_env(ENV)
    assert o["Resolution.width"] == 320 and o["Scene.light"] == [1.0, 2.0, 3.0]
    assert o["Renderer.rayType"] == "path" and o["Renderer.sortPathRays"] is True
    assert o["Camera.fieldOfView"] == 50.0
    d = app.load_env({})
    assert d["Resolution.width"] == 1024 and d["Resolution.height"] == 768
    assert d["Scene.light"] == [5.0, -2.0, 1.0] and d["Renderer.shadowRadius"] == 0.001
    assert d["Renderer.rayType"] == "primary" and d["Camera.farPlane"] == 3.0
    cfg = app.renderer_config(o)
    assert (cfg.ray_type, cfg.num_primary_samples, cfg.num_shadow_samples, cfg.recursion_depth) == (2, 2, 3, 5)
    assert (cfg.sort_shadow_rays, cfg.reorder_shadow_rays, cfg.sort_path_rays, cfg.reorder_path_rays) == (1, 0, 1, 1)
    assert (cfg.morton_kind, cfg.bvh_kind) == (2, 1)
    assert abs(cfg.shadow_radius - 0.5) < 1e-7
    assert cfg.primary_bvh_kind == -1 and cfg.shadow_overlap == 1
    o2 = app.load_env(dict(ENV, Renderer=dict(ENV["Renderer"], primaryBvh="bvh2")))
    assert app.renderer_config(o2).primary_bvh_kind == 0
    # Stage timing follows the benchmark mode (Benchmark.stageTimes, default on); FP64 accumulation
    # is an option of its own.
    assert cfg.timing == 1 and cfg.accumulate_fp64 == 0  # ENV is in benchmark mode
    assert app.renderer_config(app.load_env(dict(ENV, Application={"mode": "interactive"}))).timing == 0
    fp64_env = dict(ENV, Renderer=dict(ENV["Renderer"], accumulateFp64=True))
    assert app.renderer_config(app.load_env(fp64_env)).accumulate_fp64 == 1
    assert app.renderer_config(app.load_env(dict(ENV, Benchmark={"stageTimes": False}))).timing == 0


@pytest.mark.parametrize("bad", [{"Renderer": {"rayType": "photon"}}, {"Renderer": {"numberOfBounces": 3}},
                                 {"Renderer": {"primaryBvh": "bvh4"}},
                                 {"Camera": {"position": "1 2"}}, {"Nope": {"x": 1}}])
def test_env_rejects_bad_options(app, bad):
    with pytest.raises(ValueError):
        app.load_env(bad)


def _write_gltf(path, data_uri):
    # Two primitives: an indexed quad (uint16 indices) and a non-indexed
    # triangle, interleaved-free, positions and normals as float32.
    p0 = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    n0 = np.tile(np.array([[0, 0, 1]], np.float32), (4, 1))
    i0 = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    p1 = np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1]], np.float32)
    n1 = np.tile(np.array([[0, 0, -1]], np.float32), (3, 1))
    blobs = [p0.tobytes(), n0.tobytes(), i0.tobytes() + b"\0\0", p1.tobytes(), n1.tobytes()]
    offs = np.cumsum([0] + [len(b) for b in blobs])[:-1]
    raw = b"".join(blobs)
    views = [{"buffer": 0, "byteOffset": int(o), "byteLength": len(b)} for o, b in zip(offs, blobs)]
    acc = [{"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
           {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC3"},
           {"bufferView": 2, "componentType": 5123, "count": 6, "type": "SCALAR"},
           {"bufferView": 3, "componentType": 5126, "count": 3, "type": "VEC3"},
           {"bufferView": 4, "componentType": 5126, "count": 3, "type": "VEC3"}]
    if data_uri:
        buf = {"byteLength": len(raw), "uri": "data:application/octet-stream;base64," + base64.b64encode(raw).decode()}
    else:
        (path.parent / "mesh.bin").write_bytes(raw)
        buf = {"byteLength": len(raw), "uri": "mesh.bin"}
    doc = {"asset": {"version": "2.0"}, "buffers": [buf], "bufferViews": views, "accessors": acc,
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1}, "indices": 2},
                                      {"attributes": {"POSITION": 3, "NORMAL": 4}}]}]}
    path.write_text(json.dumps(doc))
    return p0, p1


@pytest.mark.parametrize("data_uri", [False, True])
def test_gltf_loader(app, tmp_path, data_uri):
    p0, p1 = _write_gltf(tmp_path / "scene.gltf", data_uri)
    pos, nrm, idx, first = app.load_gltf(tmp_path / "scene.gltf")
    assert np.array_equal(pos, np.concatenate([p0, p1]))
    assert np.array_equal(idx, np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6]], np.uint32))
    assert np.array_equal(first, [0, 2])
    assert np.allclose(nrm[:4, 2], 1.0) and np.allclose(nrm[4:, 2], -1.0)


def test_image_writers(app, tmp_path):
    rng = np.random.default_rng(1)
    img = rng.uniform(-0.5, 2.0, (5, 7, 3)).astype(np.float32)
    img[0, 0, 0] = np.nan
    app.write_pfm(tmp_path / "a.pfm", img)
    back = app.read_pfm(tmp_path / "a.pfm")
    assert np.array_equal(np.isnan(back), np.isnan(img))
    assert np.array_equal(np.nan_to_num(back), np.nan_to_num(img))
    app.write_ppm(tmp_path / "a.ppm", img)
    data = (tmp_path / "a.ppm").read_bytes()
    assert data.startswith(b"P6\n7 5\n255\n")
    px = np.frombuffer(data[len(b"P6\n7 5\n255\n"):], np.uint8).reshape(5, 7, 3)
    ref = np.clip(np.rint(np.clip(np.nan_to_num(img, nan=0.0), 0, 1) * 255), 0, 255).astype(np.uint8)
    assert np.array_equal(px, ref)
    flat = rng.uniform(0, 1, (6 * 4, 4)).astype(np.float32)
    assert np.array_equal(app.pixels_to_image(flat, 4, 6)[2, 3], flat[2 * 4 + 3, :3])


def test_benchmark_text(app):
    log = dict(ray_count=60, morton_ms=0.01, sort_ms=0.02, reorder_ms=0.0, trace_sort_ms=0.1, trace_ms=0.12)
    res = {"ray_type": "path", "total_rays": 100, "primary_rays": 10, "shadow_rays": 60, "path_rays": 30,
           "render_kernels_ms": 1.5, "render_absolute_ms": 2.0, "trace_total_ms": 1.2, "trace_primary_ms": 0.2,
           "trace_shadow_ms": 0.6, "trace_path_ms": 0.4, "rt_perf_total_mrays_s": 83.33,
           "rt_perf_primary_mrays_s": 50.0, "rt_perf_shadow_mrays_s": 100.0, "rt_perf_path_mrays_s": 75.0,
           "print_sort_logs": True, "shadow_sort_logs": [log, log], "path_sort_logs": [dict(log, ray_count=30)]}
    t = app.benchmark_text(res)
    assert " RAY TRACING BENCHMARK RESULTS " in t and " TOTAL RAYS              : 100" in t
    for line in (" TRACE TOTAL             : 1.2000 ms", " TRACE SHADOW            : 0.6000 ms",
                 " RT PERF TOTAL           : 83.33", " RT PERF PRIMARY         : 50.00",
                 " RT PERF SHADOW          : 100.00", " RT PERF PATH            : 75.00",
                 "SORT LOG SHADOW AT DEPTH 1", "SORT LOG PATH AT DEPTH 1", "SORT LOG SHADOW TOTAL"):
        assert line in t, line
    total = t[t.index("SORT LOG SHADOW TOTAL"):]
    assert "RAY COUNTS        : 120" in total and "TRACE TIME        : 0.2400 ms" in total
    assert "SORT LOG" not in app.benchmark_text(dict(res, print_sort_logs=False))
