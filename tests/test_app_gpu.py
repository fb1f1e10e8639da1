"""Front end on the GPU: an env.json run writes the same image a directly
driven renderer produces, and a two-primitive glTF scene (two geometries,
primitive ids relative to their geometry) renders exactly like the same
triangles as one geometry."""
import base64
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _canon(a):
    a = np.array(a, np.float32, copy=True)
    a[np.isnan(a)] = np.float32(np.nan)
    return a.view(np.uint32)


ENV = {
    "Application": {"mode": "benchmark"},
    "Benchmark": {"warmupCycles": 1, "benchmarkCycles": 2},
    "Resolution": {"width": 64, "height": 48},
    "Scene": {"generator": "soup:3000:5", "light": "0.5 1.6 0.5", "backgroundcolor": "0.53 0.81 0.98"},
    "Renderer": {"rayType": "path", "recursionDepth": 3, "numberOfShadowSamples": 2, "shadowRadius": 0.1,
                 "sortPathRays": True, "reorderPathRays": True, "mortonKind": "6d64", "bvh": "bvh8"},
    "Camera": {"position": "0.5 0.5 2.2", "rotation": "0 0 0", "nearPlane": 0.001, "farPlane": 10.0,
               "fieldOfView": 45.0},
}


def test_env_run_matches_direct_renderer(wf, dev, tmp_path):
    import torch
    from vulkanwavefrontpathtracer_gb300 import app
    opts = app.load_env(ENV)
    res = app.run(opts, str(tmp_path / "out.pfm"), device=dev, quiet=True)
    assert res["frames"] == 3 and res["total_rays"] > 64 * 48
    # Benchmark mode times every stage: trace times per ray type, RT PERF
    # from them (not from the frame time), sort logs of the sorted bounces.
    assert res["stage_times"]
    assert 0 < res["trace_total_ms"] < res["render_kernels_ms"]
    for k in ("primary", "shadow", "path"):
        assert res[f"trace_{k}_ms"] > 0 and res[f"rt_perf_{k}_mrays_s"] > 0
    assert res["rt_perf_total_mrays_s"] > res["frame_perf_mrays_s"]
    assert res["path_sort_logs"][0]["sort_ms"] > 0 and res["path_sort_logs"][0]["ray_count"] > 0
    assert "RT PERF PATH" in app.benchmark_text(res)
    img = app.read_pfm(tmp_path / "out.pfm")
    pos, nrm, idx = wf.api.generate_scene(0, 5, 3000)
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    r = wf.api.Renderer(config=app.renderer_config(opts))
    r.set_scene(sc, geom, (0.5, 1.6, 0.5), (0.53, 0.81, 0.98))
    cam = wf.api.make_camera(position=(0.5, 0.5, 2.2), fov_deg=45.0, znear=0.001, zfar=10.0)
    px = torch.zeros((64 * 48, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)
    for _ in range(3):
        r.render(cam, 64, 48, px, fp)
    ref = app.pixels_to_image(px.cpu().numpy(), 64, 48)
    assert np.array_equal(_canon(img), _canon(ref))


def _gltf_two_primitives(path, pos, nrm, idx):
    half = idx.shape[0] // 2
    parts = [(pos, nrm, idx[:half]), (pos, nrm, idx[half:])]
    blobs, acc, views, prims = [], [], [], []
    for p, n, ix in parts:
        for arr, typ, comp in ((p, "VEC3", 5126), (n, "VEC3", 5126), (ix.reshape(-1), "SCALAR", 5125)):
            views.append({"buffer": 0, "byteOffset": sum(len(b) for b in blobs), "byteLength": arr.nbytes})
            acc.append({"bufferView": len(views) - 1, "componentType": comp,
                        "count": int(arr.shape[0]), "type": typ})
            blobs.append(np.ascontiguousarray(arr).tobytes())
        k = len(acc)
        prims.append({"attributes": {"POSITION": k - 3, "NORMAL": k - 2}, "indices": k - 1})
    raw = b"".join(blobs)
    doc = {"asset": {"version": "2.0"},
           "buffers": [{"byteLength": len(raw),
                        "uri": "data:application/octet-stream;base64," + base64.b64encode(raw).decode()}],
           "bufferViews": views, "accessors": acc, "meshes": [{"primitives": prims}]}
    path.write_text(json.dumps(doc))
    return half


def test_gltf_two_geometries_render_like_one(wf, dev, tmp_path):
    import torch
    from vulkanwavefrontpathtracer_gb300 import app
    pos, nrm, idx = wf.api.generate_scene(0, 6, 2000)
    _gltf_two_primitives(tmp_path / "two.gltf", pos.astype(np.float32), nrm.astype(np.float32),
                         idx.astype(np.uint32))
    env = json.loads(json.dumps(ENV))
    env["Scene"] = {"filename": str(tmp_path / "two.gltf"), "light": "0.5 1.6 0.5",
                    "backgroundcolor": "0.53 0.81 0.98"}
    opts = app.load_env(env)
    app.run(opts, str(tmp_path / "two.pfm"), device=dev, quiet=True)
    two = app.read_pfm(tmp_path / "two.pfm")
    # The same triangles and vertices as a single geometry.
    p2, n2, i2, first = app.load_gltf(tmp_path / "two.gltf")
    assert first.shape[0] == 2
    sc = wf.api.Scene(p2, i2)
    geom = wf.api.Geometry(p2, n2, i2, device=dev)
    r = wf.api.Renderer(config=app.renderer_config(opts))
    r.set_scene(sc, geom, (0.5, 1.6, 0.5), (0.53, 0.81, 0.98))
    cam = wf.api.make_camera(position=(0.5, 0.5, 2.2), fov_deg=45.0, znear=0.001, zfar=10.0)
    px = torch.zeros((64 * 48, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)
    for _ in range(3):
        r.render(cam, 64, 48, px, fp)
    one = app.pixels_to_image(px.cpu().numpy(), 64, 48)
    assert np.array_equal(_canon(two), _canon(one))
    assert np.isfinite(one).mean() > 0.5
