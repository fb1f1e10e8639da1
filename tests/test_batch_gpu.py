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


def test_batch_on_large_scenes_matches_oracle(wf, orc, dev):
    """Batched requests on the batched workload's two city scenes (about 1M
    and the 3,000,320-triangle block, their cameras and lights), chosen form,
    small resolutions: every request's frame and ray counts equal the
    oracle's CPU frame (FP32 BVH2 traversal of the same scene), bit for
    bit."""
    import sys
    from pathlib import Path

    import torch
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    specs = [(2, 96, 64, 3, 1), (3, 64, 64, 2, 2)]  # (BATCH_SCENES index, w, h, depth, spp)
    reqs, cases = [], []
    for si, w, h, depth, spp in specs:
        S = bench.BATCH_SCENES[si]
        pos, nrm, idx = wf.api.generate_scene(S["kind"], S["seed"], S["ntris"])
        sc = wf.api.Scene(pos, idx)
        geom = wf.api.Geometry(pos, nrm, idx, device=dev)
        over = dict(bench.COURTYARD["renderer"], recursion_depth=depth, num_primary_samples=spp)
        cfg = wf.api.default_config(**over, **bench.CHOSEN)
        px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros_like(px)
        reqs.append(dict(scene=sc, geometry=geom, light=S["light"], background=S["background"],
                         camera=wf.api.make_camera(**S["camera"]), width=w, height=h, config=cfg, pixels=px,
                         frame_pixels=fp))
        cases.append((S, pos, nrm, idx, sc, w, h, over))
    batch = wf.api.Batch(reqs, streams=2)
    batch.render()
    torch.cuda.synchronize()
    assert wf.api.device_status() == 0
    for i, (S, pos, nrm, idx, sc, w, h, over) in enumerate(cases):
        nodes, tris = sc.export_bvh2()
        hg = orc.HostGeometry(wf.api.gltf_vertices(pos, nrm), idx)
        c = S["camera"]
        s2w = wf.api.camera_screen_to_world(c["position"], c["rotation_deg"], c["fov_deg"], w / h, c["znear"],
                                            c["zfar"])
        F = bench.CHOSEN
        cfg = orc.FrameCfg(ray_type=2, spp=over["num_primary_samples"], S=over["num_shadow_samples"],
                           depth=over["recursion_depth"], radius=over["shadow_radius"], key=over["key_value"],
                           white=over["white_point"], albedo=over["albedo"], sort_shadow=F["sort_shadow_rays"],
                           reorder_shadow=F["reorder_shadow_rays"], sort_path=F["sort_path_rays"],
                           reorder_path=F["reorder_path_rays"], morton_kind=F["morton_kind"], frame_index=1)
        o_px, o_fp, o_st = orc.render_frame(nodes, tris, hg, sc.bounds_min, sc.bounds_max, S["light"],
                                            S["background"], s2w, c["position"], c["zfar"], w, h, cfg)
        st = batch.stats(i)
        assert (st.num_primary_rays, st.num_shadow_rays, st.num_path_rays) == (o_st.primary, o_st.shadow, o_st.path)
        assert np.array_equal(_canon(reqs[i]["frame_pixels"].cpu().numpy()), _canon(o_fp)), i
        assert np.array_equal(_canon(reqs[i]["pixels"].cpu().numpy()), _canon(o_px)), i
    batch.close()
