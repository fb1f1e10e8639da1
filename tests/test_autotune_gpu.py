"""The autotuner's whole-frame searches (per-bounce reordering, the BVH of
the bounces and of the primary pass) on a small scene: each returns a
setting from its table, and the BVH choices leave the image bit-identical.
(The reordering choice does change the image, as in the reference: a path
ray's random sequence belongs to its wavefront slot, so frames are checked
against the oracle per reordering setting in test_renderer_gpu.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAM = dict(position=(0.5, 0.5, 2.2), rotation_deg=(0.0, 0.0, 0.0), fov_deg=45.0, znear=0.001, zfar=10.0)
LIGHT = (0.5, 1.6, 0.5)
BG = (0.53, 0.81, 0.98)
BASE = dict(num_primary_samples=1, num_shadow_samples=2, shadow_radius=0.1, recursion_depth=3, key_value=0.6,
            white_point=2.0, albedo=0.8, bvh_kind=1, morton_kind=2, sort_path_rays=1, reorder_path_rays=1,
            use_graph=1)
W, H = 96, 64


def _canon(a):
    a = np.array(a, dtype=np.float32, copy=True)
    a[np.isnan(a)] = np.float32(np.nan)
    return a.view(np.uint32)


def test_frame_searches_keep_the_image(wf, dev):
    import torch

    from vulkanwavefrontpathtracer_gb300 import autotune
    api = wf.api
    pos, nrm, idx = api.generate_scene(0, 21, 20000)
    sc = api.Scene(pos, idx)
    geom = api.Geometry(pos, nrm, idx, device=dev)
    cam = api.make_camera(**CAM)

    def make(**form):
        r = api.Renderer(**dict(BASE, ray_type=wf.PATH_RAYS, **form))
        r.set_scene(sc, geom, LIGHT, BG)
        return r

    bounce = autotune.tune_bounce_sort(lambda m: make(path_sort_skip=m), cam, W, H, BASE["recursion_depth"], frames=1,
                                       device=dev)
    mask = bounce["path_sort_skip"]
    assert 0 <= mask < (1 << BASE["recursion_depth"])
    assert len(bounce["table"]) == 1 + BASE["recursion_depth"]
    assert any(e["path_sort_skip"] == mask for e in bounce["table"])
    kinds = autotune.tune_bvh_kinds(lambda k, pk: make(path_sort_skip=mask, bvh_kind=k, primary_bvh_kind=pk), cam, W,
                                    H, frames=1, device=dev)
    assert [(e["bvh_kind"], e["primary_bvh_kind"]) for e in kinds["table"]] == [(1, -1), (1, 0), (0, -1)]
    assert (kinds["bvh_kind"], kinds["primary_bvh_kind"]) in [(1, -1), (1, 0), (0, -1)]
    assert all(e["ms"] > 0 for e in kinds["table"])
    prim = autotune.tune_primary_bvh(lambda k: make(path_sort_skip=mask, primary_bvh_kind=k), cam, W, H, frames=1,
                                     device=dev)
    assert prim["primary_bvh_kind"] in (0, 1)

    def frame(r):
        px = torch.zeros((W * H, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros_like(px)
        r.render(cam, W, H, px, fp)
        out = fp.cpu().numpy()
        r.close()
        return out

    ref = frame(make(path_sort_skip=mask))
    tuned = frame(make(path_sort_skip=mask, bvh_kind=kinds["bvh_kind"], primary_bvh_kind=kinds["primary_bvh_kind"]))
    assert np.array_equal(_canon(ref), _canon(tuned))
    for k, pk in ((0, -1), (0, 1), (1, 0)):
        assert np.array_equal(_canon(ref), _canon(frame(make(path_sort_skip=mask, bvh_kind=k, primary_bvh_kind=pk))))
    assert api.device_status() == 0
