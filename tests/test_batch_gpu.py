"""Batched render requests (wfpt_batch_*): one captured graph over several
branches renders many requests -- different scenes, resolutions, sample
counts, depths, sort settings and BVH forms -- and every request's output,
frame after frame, is bit-identical to a standalone renderer's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIGHT = (0.5, 1.6, 0.5)
BG = (0.53, 0.81, 0.98)


def cam(wf, f, i):
    return wf.api.make_camera(position=(0.5 + 0.03 * i, 0.5 - 0.02 * f, 2.2), rotation_deg=(0.0, 2.0 * i, 0.0),
                              fov_deg=45.0, znear=0.001, zfar=10.0)


def _canon(a):
    a = np.array(a, np.float32, copy=True)
    a[np.isnan(a)] = np.float32(np.nan)
    return a.view(np.uint32)


def test_batch_matches_standalone_renderers(wf, dev):
    import torch
    scenes = []
    for seed, ntris in ((4, 6000), (5, 3000)):
        pos, nrm, idx = wf.api.generate_scene(0, seed, ntris)
        scenes.append((wf.api.Scene(pos, idx), wf.api.Geometry(pos, nrm, idx, device=dev)))
    specs = [  # (scene, w, h, overrides)
        (0, 48, 32, dict(ray_type=wf.PATH_RAYS, recursion_depth=4, num_primary_samples=2)),
        (1, 64, 64, dict(ray_type=wf.PATH_RAYS, recursion_depth=2, sort_path_rays=1, reorder_path_rays=1,
                         bvh_kind=wf.BVH8_Q8, morton_kind=2)),
        (0, 40, 40, dict(ray_type=wf.SHADOW_RAYS, num_shadow_samples=3, sort_shadow_rays=1)),
        (1, 33, 17, dict(ray_type=wf.PRIMARY_RAYS, num_primary_samples=3)),
        (0, 96, 64, dict(ray_type=wf.PATH_RAYS, recursion_depth=8, bvh_kind=wf.BVH8_Q8, sort_path_rays=1,
                         morton_kind=0)),
    ]
    reqs, solo = [], []
    for i, (si, w, h, ov) in enumerate(specs):
        cfg = wf.api.default_config(shadow_radius=0.1, **ov)
        sc, geom = scenes[si]
        px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        reqs.append(dict(scene=sc, geometry=geom, light=LIGHT, background=BG, camera=cam(wf, 0, i), width=w,
                         height=h, config=cfg, pixels=px, frame_pixels=fp))
        r = wf.api.Renderer(config=wf.api.default_config(shadow_radius=0.1, **ov))
        r.set_scene(sc, geom, LIGHT, BG)
        solo.append((r, torch.zeros_like(px), torch.zeros_like(fp)))
    batch = wf.api.Batch(reqs, streams=3)
    assert batch.kernels() > 0
    for f in range(3):
        cams = [cam(wf, f, i) for i in range(len(specs))]
        batch.render(cams)
        for i, (r, px, fp) in enumerate(solo):
            r.render(cams[i], specs[i][1], specs[i][2], px, fp)
        torch.cuda.synchronize()
        for i, (r, px, fp) in enumerate(solo):
            q = reqs[i]
            assert np.array_equal(_canon(q["pixels"].cpu().numpy()), _canon(px.cpu().numpy())), (f, i)
            assert np.array_equal(_canon(q["frame_pixels"].cpu().numpy()), _canon(fp.cpu().numpy())), (f, i)
            a, b = batch.stats(i), r.stats()
            assert (a.num_primary_rays, a.num_shadow_rays, a.num_path_rays) == \
                   (b.num_primary_rays, b.num_shadow_rays, b.num_path_rays)
    assert wf.api.device_status() == 0
    batch.close()
