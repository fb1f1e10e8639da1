"""Whole frames through the C ABI renderer against the oracle's CPU frame
(Renderer::render restated), bit-exact: same pixel table, seeds, rays,
traversal, compaction order, shading and tone map."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def N(t):
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def small(wf, orc, dev):
    pos, nrm, idx = wf.api.generate_scene(0, 1, 65536)
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    nodes, tris = sc.export_bvh2()
    hg = orc.HostGeometry(wf.api.gltf_vertices(pos, nrm), idx)
    return sc, geom, nodes, tris, hg


CAM = dict(position=(0.5, 0.5, 2.2), rotation_deg=(0.0, 0.0, 0.0), fov_deg=45.0, znear=0.001, zfar=10.0)
LIGHT = (0.5, 1.6, 0.5)
BG = (0.53, 0.81, 0.98)


def run_pair(wf, orc, dev, small, w, h, frames=1, **opts):
    import torch
    sc, geom, nodes, tris, hg = small
    base = dict(ray_type=wf.PATH_RAYS, num_primary_samples=1, num_shadow_samples=2, shadow_radius=0.1,
                recursion_depth=4, key_value=0.6, white_point=2.0, sort_shadow_rays=0, reorder_shadow_rays=0,
                sort_path_rays=0, reorder_path_rays=0, morton_kind=0, bvh_kind=wf.BVH2_FP32, albedo=0.8)
    base.update(opts)
    r = wf.api.Renderer(**base)
    r.set_scene(sc, geom, LIGHT, BG)
    cam = wf.api.make_camera(**CAM)
    px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    s2w = wf.api.camera_screen_to_world(CAM["position"], CAM["rotation_deg"], CAM["fov_deg"], w / h, CAM["znear"],
                                        CAM["zfar"])
    cfg = orc.FrameCfg(ray_type=base["ray_type"], spp=base["num_primary_samples"], S=base["num_shadow_samples"],
                       depth=base["recursion_depth"], radius=base["shadow_radius"], key=0.6, white=2.0, albedo=0.8,
                       sort_shadow=base["sort_shadow_rays"], reorder_shadow=base["reorder_shadow_rays"],
                       sort_path=base["sort_path_rays"], reorder_path=base["reorder_path_rays"],
                       morton_kind=base["morton_kind"], frame_index=1,
                       path_sort_skip=base.get("path_sort_skip", 0))
    o_px = None
    for f in range(1, frames + 1):
        r.render(cam, w, h, px, fp)
        st = r.stats()
        cfg.frame_index = f
        o_px, o_fp, o_st = orc.render_frame(nodes, tris, hg, sc.bounds_min, sc.bounds_max, LIGHT, BG, s2w,
                                            CAM["position"], CAM["zfar"], w, h, cfg, pixels=o_px)
    assert wf.api.device_status() == 0
    return N(px), N(fp), st, o_px, o_fp, o_st


def _canon_nan(a):
    # Reinhard of a black pixel divides 0/0 (interpolateColors.comp:31-32);
    # GPU and CPU produce NaNs with different payload bits, so NaNs are
    # compared by position only.
    a = np.array(a, dtype=np.float32, copy=True)
    a[np.isnan(a)] = np.float32(np.nan)
    return a


class same_bits:
    """Truthy when the two float arrays are bit-identical (NaN payloads
    aside); its repr reports how many pixels differ, by how much, and the
    first few."""

    def __init__(self, a, b):
        a, b = _canon_nan(a), _canon_nan(b)
        self.ok = np.array_equal(a.view(np.uint32), b.view(np.uint32))
        bad = np.nonzero((a.view(np.uint32) != b.view(np.uint32)).any(axis=1))[0]
        self.msg = "identical"
        if bad.size:
            d = np.abs(a[bad] - b[bad]).max()
            first = ", ".join(f"{i}: {a[i]} vs {b[i]}" for i in bad[:3])
            self.msg = f"{bad.size} of {len(a)} pixels differ (max abs diff {d:.3g}); {first}"

    def __bool__(self):
        return bool(self.ok)

    def __repr__(self):
        return self.msg


@pytest.mark.parametrize("opts", [
    dict(),
    dict(sort_path_rays=1, sort_shadow_rays=1),
    dict(sort_path_rays=1, reorder_path_rays=1, sort_shadow_rays=1, reorder_shadow_rays=1),
    dict(sort_path_rays=1, reorder_path_rays=1, morton_kind=2, bvh_kind=1),
    dict(sort_path_rays=1, reorder_path_rays=1, sort_shadow_rays=1, reorder_shadow_rays=1, morton_kind=1,
         num_shadow_samples=3),
    # per-bounce reordering: bounces 1 and 3 unsorted, 2 and 4 sorted + reordered
    dict(sort_path_rays=1, reorder_path_rays=1, morton_kind=2, bvh_kind=1, path_sort_skip=0b0101),
    # shadow passes on the frame's stream in the reference's order (the
    # other cases overlap them with the next bounce)
    dict(sort_path_rays=1, reorder_path_rays=1, morton_kind=2, bvh_kind=1, shadow_overlap=0),
    dict(sort_path_rays=1, reorder_path_rays=1, sort_shadow_rays=1, reorder_shadow_rays=1, shadow_overlap=0),
    # the primary pass on the other BVH than the bounces
    dict(sort_path_rays=1, reorder_path_rays=1, morton_kind=2, bvh_kind=1, primary_bvh_kind=0),
    dict(bvh_kind=0, primary_bvh_kind=1),
])
def test_path_frame_bit_exact(wf, orc, dev, small, opts):
    px, fp, st, o_px, o_fp, o_st = run_pair(wf, orc, dev, small, 96, 64, **opts)
    assert st.num_primary_rays == o_st.primary
    assert st.num_path_rays == o_st.path
    assert st.num_shadow_rays == o_st.shadow
    assert list(st.path_rays_per_bounce) == list(o_st.path_per_bounce)
    assert same_bits(fp, o_fp) and same_bits(px, o_px)


def test_small_config_full_size(wf, orc, dev, small):
    """256x256, 4 bounces, 32-bit keys with reordering (the small config)."""
    px, fp, st, o_px, o_fp, o_st = run_pair(wf, orc, dev, small, 256, 256, sort_path_rays=1, reorder_path_rays=1,
                                            sort_shadow_rays=1, bvh_kind=1)
    assert st.num_path_rays == o_st.path and st.num_shadow_rays == o_st.shadow
    assert same_bits(fp, o_fp)


@pytest.mark.parametrize("ray_type", [0, 1])
def test_primary_and_shadow_frames(wf, orc, dev, small, ray_type):
    px, fp, st, o_px, o_fp, o_st = run_pair(wf, orc, dev, small, 80, 50, ray_type=ray_type)
    assert same_bits(fp, o_fp) and same_bits(px, o_px)


def test_accumulation_over_frames_and_spp(wf, orc, dev, small):
    px, fp, st, o_px, o_fp, o_st = run_pair(wf, orc, dev, small, 40, 40, frames=3, num_primary_samples=2,
                                            sort_path_rays=1, reorder_path_rays=1)
    assert same_bits(fp, o_fp) and same_bits(px, o_px)


@pytest.mark.parametrize("opts", [
    dict(),
    dict(sort_path_rays=1, reorder_path_rays=1, morton_kind=2, bvh_kind=1),
    dict(ray_type=1, sort_shadow_rays=1, reorder_shadow_rays=1),
    dict(sort_path_rays=1, reorder_path_rays=1, sort_shadow_rays=1, reorder_shadow_rays=1, morton_kind=2,
         bvh_kind=1, num_primary_samples=2),
    dict(sort_path_rays=1, reorder_path_rays=1, morton_kind=2, bvh_kind=1, shadow_overlap=0),
])
def test_graph_frames_match_direct_frames(wf, dev, small, opts):
    """use_graph=1 replays one captured frame with the camera and frame
    index read from device memory; frames must equal directly launched ones
    while the camera moves and the frame index advances."""
    import torch
    sc, geom, nodes, tris, hg = small
    base = dict(ray_type=wf.PATH_RAYS, num_primary_samples=1, num_shadow_samples=2, shadow_radius=0.1,
                recursion_depth=4, key_value=0.6, white_point=2.0, bvh_kind=wf.BVH2_FP32, albedo=0.8)
    base.update(opts)
    w, h = 72, 48
    outs = []
    for use_graph in (0, 1):
        r = wf.api.Renderer(use_graph=use_graph, **base)
        r.set_scene(sc, geom, LIGHT, BG)
        px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        seq = []
        for f in range(4):
            cam = wf.api.make_camera(**dict(CAM, position=(0.5 + 0.05 * (f % 2), 0.5, 2.2)))
            r.render(cam, w, h, px, fp)
            st = r.stats()
            seq.append((N(px).copy(), N(fp).copy(), st.num_path_rays, st.num_shadow_rays))
        outs.append(seq)
    assert wf.api.device_status() == 0
    for (pa, fa, na, sa), (pb, fb, nb, sb) in zip(*outs):
        assert na == nb and sa == sb
        assert same_bits(pa, pb) and same_bits(fa, fb)


def test_renderer_rejects_missing_bvh_kind(wf, dev):
    """A renderer whose primary pass (or bounces) asks for a BVH the scene
    was built without is refused at set_scene and at render, before any
    traversal launch."""
    import torch
    pos, nrm, idx = wf.api.generate_scene(0, 6, 2000)
    only8 = wf.api.Scene(pos, idx, bvh2=False)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    r = wf.api.Renderer(ray_type=wf.PATH_RAYS, bvh_kind=wf.BVH8_Q8, primary_bvh_kind=wf.BVH2_FP32)
    with pytest.raises(wf.WfptError):
        r.set_scene(only8, geom, LIGHT, BG)
    r2 = wf.api.Renderer(ray_type=wf.PATH_RAYS, bvh_kind=wf.BVH8_Q8)
    r2.set_scene(only8, geom, LIGHT, BG)
    r2.set_config(wf.api.default_config(ray_type=wf.PATH_RAYS, bvh_kind=wf.BVH8_Q8, primary_bvh_kind=wf.BVH2_FP32))
    px = torch.zeros((16 * 16, 4), dtype=torch.float32, device=dev)
    with pytest.raises(wf.WfptError):
        r2.render(wf.api.make_camera(**CAM), 16, 16, px, px.clone())
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("workload", ["COURTYARD", "CITY"])
def test_full_size_frames_identical_across_forms(wf, dev, workload):
    """Whole frames at the benchmark's sizes (courtyard 1920x1080, city
    block 3840x2160, 8 bounces, sorted path rays): BVH8 or FP32 BVH2 for the
    bounces and the camera rays, graph replay or direct launches, shadow
    passes overlapped or not -- the same pixels bit for bit (the CPU oracle
    frame is checked at small sizes above; here the forms check each
    other at full size)."""
    import sys
    from pathlib import Path

    import torch
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    W = getattr(bench, workload)
    pos, nrm, idx = wf.api.generate_scene(W["scene_kind"], W["seed"])
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    cam = wf.api.make_camera(**W["camera"])
    w, h = W["width"], W["height"]
    rcfg = dict(bench.COURTYARD["renderer"], **W["renderer"])

    def frame(**form):
        r = wf.api.Renderer(**dict(rcfg, morton_kind=2, sort_path_rays=1, reorder_path_rays=1, **form))
        r.set_scene(sc, geom, W["light"], W["background"])
        px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros_like(px)
        r.render(cam, w, h, px, fp)
        st = r.stats()
        out = _canon_nan(N(fp)).view(np.uint32)
        r.close()
        return out, (st.num_primary_rays, st.num_shadow_rays, st.num_path_rays)

    ref, counts = frame(bvh_kind=wf.BVH8_Q8, use_graph=1, shadow_overlap=1)
    assert counts[2] > 0
    for form in (dict(bvh_kind=wf.BVH2_FP32, use_graph=0, shadow_overlap=0),
                 dict(bvh_kind=wf.BVH8_Q8, primary_bvh_kind=wf.BVH2_FP32, use_graph=1, shadow_overlap=1),
                 dict(bvh_kind=wf.BVH8_Q8, use_graph=0, shadow_overlap=0)):
        got, c = frame(**form)
        assert c == counts
        assert np.array_equal(got, ref)
    assert wf.api.device_status() == 0
