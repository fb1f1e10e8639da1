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


def _workload_frame_vs_oracle(wf, orc, dev, W, w, h, form, cfg_over=None):
    """One frame of a benchmark workload rendered by the GPU renderer in
    `form` and by the oracle's CPU frame (FP32 BVH2 traversal, the
    reference's pass order and batch cap), compared pixel by pixel (tone
    mapped and accumulated) and in every ray count."""
    import sys
    from pathlib import Path

    import torch
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    pos, nrm, idx = wf.api.generate_scene(W["scene_kind"], W["seed"])
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    rcfg = dict(bench.COURTYARD["renderer"], **W["renderer"])
    rcfg.update(cfg_over or {})
    rcfg.update(form)
    r = wf.api.Renderer(**rcfg)
    r.set_scene(sc, geom, W["light"], W["background"])
    cam = wf.api.make_camera(**W["camera"])
    px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)
    r.render(cam, w, h, px, fp)
    st = r.stats()
    g_px, g_fp = N(px), N(fp)
    r.close()
    assert wf.api.device_status() == 0
    nodes, tris = sc.export_bvh2()
    hg = orc.HostGeometry(wf.api.gltf_vertices(pos, nrm), idx)
    c = W["camera"]
    s2w = wf.api.camera_screen_to_world(c["position"], c["rotation_deg"], c["fov_deg"], w / h, c["znear"], c["zfar"])
    cfg = orc.FrameCfg(ray_type=rcfg["ray_type"], spp=rcfg["num_primary_samples"], S=rcfg["num_shadow_samples"],
                       depth=rcfg["recursion_depth"], radius=rcfg["shadow_radius"], key=rcfg["key_value"],
                       white=rcfg["white_point"], albedo=rcfg["albedo"], sort_shadow=rcfg.get("sort_shadow_rays", 0),
                       reorder_shadow=rcfg.get("reorder_shadow_rays", 0), sort_path=rcfg.get("sort_path_rays", 0),
                       reorder_path=rcfg.get("reorder_path_rays", 0), morton_kind=rcfg.get("morton_kind", 0),
                       frame_index=1, path_sort_skip=rcfg.get("path_sort_skip", 0))
    o_px, o_fp, o_st = orc.render_frame(nodes, tris, hg, sc.bounds_min, sc.bounds_max, W["light"], W["background"],
                                        s2w, c["position"], c["zfar"], w, h, cfg)
    sc.close()
    assert st.num_primary_rays == o_st.primary
    assert st.num_shadow_rays == o_st.shadow
    assert st.num_path_rays == o_st.path
    assert list(st.path_rays_per_bounce) == list(o_st.path_per_bounce)
    assert same_bits(g_fp, o_fp) and same_bits(g_px, o_px)
    return st


def test_courtyard_1080p_chosen_frame_matches_oracle(wf, orc, dev):
    """The benchmark frame itself: courtyard, 1920x1080, 8 bounces, chosen
    form (BVH8-Q8, 6-D 64-bit Morton sort + reorder of every bounce's path
    rays, graph replay, overlapped shadow passes) against the oracle frame,
    bit for bit."""
    import bench
    st = _workload_frame_vs_oracle(wf, orc, dev, bench.COURTYARD, 1920, 1080, bench.CHOSEN)
    assert st.num_path_rays > 10_000_000


def test_city_frame_matches_oracle(wf, orc, dev):
    """The 3,000,320-triangle city block at 960x540 (a sixteenth of its
    benchmark pixels; the BVH, scene and camera are the benchmark's), chosen
    form, against the oracle frame, bit for bit."""
    import bench
    _workload_frame_vs_oracle(wf, orc, dev, bench.CITY, 960, 540, bench.CHOSEN)


@pytest.mark.parametrize("overlap", [0, 1])
def test_multi_batch_shadow_frame_matches_oracle(wf, orc, dev, overlap):
    """A frame whose primary shadow pass needs two batches under the
    reference's cap of 8M rays per batch (1024x1024 pixels x 9 shadow
    samples = 9.4M rays: batches of 932,067 and 116,509 inputs, each batch's
    seeds indexed from its own start as raygenShadow.comp:85 does), the
    bounces one batch each, against the oracle frame."""
    import bench
    st = _workload_frame_vs_oracle(wf, orc, dev, bench.COURTYARD, 1024, 1024,
                                   dict(bench.CHOSEN, shadow_overlap=overlap),
                                   cfg_over=dict(num_shadow_samples=9, recursion_depth=2))
    assert st.num_primary_rays * 9 > 8 * 1024 * 1024
    # The memory planner runs the two batches on two slots when passes
    # overlap (a GB300 has the memory for both).
    assert st.shadow_batch_slots == (2 if overlap else 1)


@pytest.mark.parametrize("slots,sort_shadow", [(1, 0), (2, 0), (0, 0), (2, 1)])
def test_shadow_batch_slots_identical_frames(wf, dev, slots, sort_shadow):
    """17 shadow samples at 1024x1024: the primary shadow pass is three
    batches (493,447 + 493,447 + 61,682 inputs).  Run one after another on
    the frame's stream, on 1 or 2 slots (the third batch reuses slot 0) or on
    as many as the planner gives (3), with and without sorted shadow rays,
    the frames and ray counts are the same bit for bit."""
    import bench
    import torch
    W = bench.COURTYARD
    pos, nrm, idx = wf.api.generate_scene(W["scene_kind"], W["seed"])
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    cam = wf.api.make_camera(**W["camera"])
    w = h = 1024

    def frame(overlap, knob):
        old = wf.api.tune_get("renderer.shadow_slots")
        try:
            wf.api.tune_set("renderer.shadow_slots", knob)
            r = wf.api.Renderer(**dict(bench.COURTYARD["renderer"], num_shadow_samples=17, recursion_depth=1,
                                       bvh_kind=wf.BVH8_Q8, use_graph=1, shadow_overlap=overlap,
                                       sort_shadow_rays=sort_shadow))
            r.set_scene(sc, geom, W["light"], W["background"])
            px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
            fp = torch.zeros_like(px)
            for _ in range(2):  # graph replay of the captured frame, frame index 1 and 2
                r.render(cam, w, h, px, fp)
            st = r.stats()
            out = (_canon_nan(N(px)).view(np.uint32), _canon_nan(N(fp)).view(np.uint32),
                   (st.num_primary_rays, st.num_shadow_rays, st.num_path_rays), st.shadow_batch_slots)
            r.close()
            return out
        finally:
            wf.api.tune_set("renderer.shadow_slots", old)

    ref = frame(0, 0)
    got = frame(1, slots)
    assert got[3] == (slots if slots else 3) and ref[3] == 1
    assert got[2] == ref[2]
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert wf.api.device_status() == 0


def test_fp64_accumulation_frames_match_oracle(wf, orc, dev, small):
    """accumulate_fp64: four frames (graph replay), each frame's pixels and
    tone-mapped image bit-exact against the oracle keeping the same double
    running mean; frame 1 equals the float mode's."""
    import torch
    sc, geom, nodes, tris, hg = small
    w, h = 64, 48
    base = dict(ray_type=wf.PATH_RAYS, num_primary_samples=1, num_shadow_samples=2, shadow_radius=0.1,
                recursion_depth=3, key_value=0.6, white_point=2.0, bvh_kind=wf.BVH8_Q8, albedo=0.8, use_graph=1,
                sort_path_rays=1, reorder_path_rays=1, morton_kind=2)
    r = wf.api.Renderer(accumulate_fp64=1, **base)
    r.set_scene(sc, geom, LIGHT, BG)
    cam = wf.api.make_camera(**CAM)
    px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
    fp = torch.zeros_like(px)
    s2w = wf.api.camera_screen_to_world(CAM["position"], CAM["rotation_deg"], CAM["fov_deg"], w / h, CAM["znear"],
                                        CAM["zfar"])
    cfg = orc.FrameCfg(ray_type=2, spp=1, S=2, depth=3, radius=0.1, key=0.6, white=2.0, albedo=0.8, sort_path=1,
                       reorder_path=1, morton_kind=2, frame_index=1, accumulate_fp64=1)
    o_px, acc = None, None
    for f in range(1, 5):
        r.render(cam, w, h, px, fp)
        cfg.frame_index = f
        o_px, o_fp, _, acc = orc.render_frame(nodes, tris, hg, sc.bounds_min, sc.bounds_max, LIGHT, BG, s2w,
                                              CAM["position"], CAM["zfar"], w, h, cfg, pixels=o_px, accum=acc)
        assert same_bits(N(fp), o_fp) and same_bits(N(px), o_px), f
        if f == 1:
            r32 = wf.api.Renderer(**base)
            r32.set_scene(sc, geom, LIGHT, BG)
            px32, fp32 = torch.zeros_like(px), torch.zeros_like(px)
            r32.render(cam, w, h, px32, fp32)
            assert same_bits(N(px32), N(px))
    assert wf.api.device_status() == 0


def test_timing_stats_fill_trace_times_and_sort_logs(wf, dev, small):
    """timing=1 (the reference's benchmark mode with printSortLogs): the
    frame is unchanged (pixels and ray counts equal the graph-replayed,
    overlapped frame's), the per-type trace times are positive and add up to
    less than the frame, and every sorted pass has a sort log with its
    Morton, sort, reorder, sorted-trace and unsorted-trace times."""
    import torch
    sc, geom, nodes, tris, hg = small
    w, h = 128, 96
    base = dict(ray_type=wf.PATH_RAYS, num_primary_samples=2, num_shadow_samples=2, shadow_radius=0.1,
                recursion_depth=4, key_value=0.6, white_point=2.0, bvh_kind=wf.BVH8_Q8, albedo=0.8,
                sort_path_rays=1, reorder_path_rays=1, morton_kind=2, sort_shadow_rays=1, reorder_shadow_rays=0,
                use_graph=1, shadow_overlap=1, path_sort_skip=0b0010)
    out = []
    for timing in (0, 1):
        r = wf.api.Renderer(timing=timing, **base)
        r.set_scene(sc, geom, LIGHT, BG)
        px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros_like(px)
        r.render(wf.api.make_camera(**CAM), w, h, px, fp)
        out.append((N(px), N(fp), r.stats()))
        r.close()
    (pa, fa, s0), (pb, fb, st) = out
    assert same_bits(pa, pb) and same_bits(fa, fb)
    assert (s0.num_primary_rays, s0.num_shadow_rays, s0.num_path_rays) == \
        (st.num_primary_rays, st.num_shadow_rays, st.num_path_rays)
    assert s0.timed == 0 and s0.primary_trace_ms == 0.0
    assert st.timed == 1
    assert st.primary_trace_ms > 0 and st.shadow_trace_ms > 0 and st.path_trace_ms > 0
    assert st.primary_trace_ms + st.shadow_trace_ms + st.path_trace_ms < st.frame_ms
    for b in range(4):
        lg = st.path_sort_logs[b]
        assert lg.ray_count == st.path_rays_per_bounce[b] > 0
        if b == 1:  # path_sort_skip: bounce 2 traces unsorted, no sort-log times
            assert lg.morton_ms == lg.sort_ms == lg.trace_sort_ms == lg.trace_ms == 0.0
        else:
            assert min(lg.morton_ms, lg.sort_ms, lg.reorder_ms, lg.trace_sort_ms, lg.trace_ms) > 0
    for i in range(5):
        lg = st.shadow_sort_logs[i]
        assert lg.ray_count == 2 * st.shadow_hits_per_pass[i]
        assert lg.reorder_ms == 0.0  # shadow rays sorted, traced through the indirect index
        assert min(lg.morton_ms, lg.sort_ms, lg.trace_sort_ms, lg.trace_ms) > 0
    assert wf.api.device_status() == 0
