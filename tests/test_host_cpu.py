"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared entry point, host helpers match the oracle, the BVH builders
produce valid (conservative) structures, argument errors are reported
without touching a device, and the CPU traversal agrees with FP64."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import random_rays

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "wfpt.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wfpt_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(wf):
    lib = wf._lib.load()
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(wf._lib.EXPORTED)
    assert lib.wfpt_abi_version() == 1


def test_status_strings(wf):
    lib = wf._lib.load()
    for code in range(8):
        assert lib.wfpt_status_string(code)


def test_invalid_arguments_rejected_on_host(wf):
    lib = wf._lib.load()
    buf = C.c_void_p(0x1000)
    assert lib.wfpt_sort_pairs(buf, buf, 10, None, 0, buf, 1 << 20, None) == 1
    assert lib.wfpt_sort_pairs(buf, buf, 10, None, 65, buf, 1 << 20, None) == 1
    assert lib.wfpt_sort_pairs(buf, buf, 10, None, 32, None, 0, None) == 1
    assert lib.wfpt_sort_pairs(buf, buf, 1000, None, 32, buf, 16, None) == 6  # scratch too small
    assert lib.wfpt_morton(None, 5, None, wf._lib.fvec([0, 0, 0]), wf._lib.fvec([1, 1, 1]), 0, None, None, None) == 1
    assert lib.wfpt_morton(buf, 5, None, wf._lib.fvec([0, 0, 0]), wf._lib.fvec([1, 1, 1]), 7, buf, buf, None) == 1
    assert lib.wfpt_reorder(buf, buf, buf, buf, buf, buf, 4, None, None) == 1  # in place
    other = C.c_void_p(0x2000)
    assert lib.wfpt_reorder_records(buf, buf, other, 40, None, None, None, 4, None, None) == 1  # width
    assert lib.wfpt_reorder_records(buf, buf, other, 48, buf, None, None, 4, None, None) == 1  # partial maps
    assert lib.wfpt_reorder_records(buf, C.c_void_p(0x1008), other, 48, None, None, None, 4, None, None) == 1
    assert b"aligned" in lib.wfpt_last_error_message()
    assert lib.wfpt_reorder_records(buf, buf, buf, 48, None, None, None, 4, None, None) == 1  # in place
    assert lib.wfpt_reorder_records(None, None, None, 48, None, None, None, 0, None, None) == 0  # empty
    assert lib.wfpt_selftest_wait_timeout(2) == 1  # no such self-test
    out = C.c_void_p()
    assert lib.wfpt_scene_create_device(None, 3, None, 5, None, 0, 3, None, C.byref(out)) == 1  # null mesh
    assert lib.wfpt_scene_create_device(buf, 3, buf, 5, None, 0, 3 | 0x100, None, C.byref(out)) == 1  # host-only
    assert lib.wfpt_scene_create_device(buf, 0, buf, 5, None, 0, 3, None, C.byref(out)) == 1  # no vertices
    assert lib.wfpt_scene_create_device(buf, 3, buf, 5, None, 0, 0, None, C.byref(out)) == 1  # no BVH kind
    assert lib.wfpt_raygen_shadow(buf, buf, buf, buf, buf, buf, wf._lib.fvec([0, 0, 0]), 1.0, 0, 4, None, 0,
                                  None) == 1
    assert lib.wfpt_trace(None, 0, buf, buf, None, 4, None, 1, None) == 1
    assert b"null" in lib.wfpt_last_error_message()
    big = wf.api.RAYGEN_PATH_STATIC_MAX_RAYS + 1
    assert lib.wfpt_raygen_path_static(buf, buf, buf, buf, buf, buf, buf, buf, buf, big, None, 0, 0.8, None) == 1
    assert b"WFPT_RAYGEN_PATH_STATIC_MAX_RAYS" in lib.wfpt_last_error_message()


def test_pixel_table_matches_oracle(wf, orc):
    for w, h in [(256, 256), (1920, 1080), (13, 10), (1, 1), (7, 9), (1560, 720)]:
        a, b = wf.api.pixel_table(w, h)
        oa, ob = orc.pixel_table(w, h)
        assert np.array_equal(a, oa) and np.array_equal(b, ob)
        assert np.array_equal(np.sort(a), np.arange(w * h))


def test_camera_matrix_matches_glm_restatement(wf, orc):
    cases = [((15, 6, 19.5), (0, 0, 0), 60.0, 16 / 9, 0.1, 512.0),
             ((8.287917, 3.804885, 34.659367), (1.075014, -303.599152, 0.0), 60.0, 1560 / 720, 0.1, 512.0),
             ((0.5, 0.5, 2.5), (-10, 20, 5), 45.0, 1.0, 0.001, 3.0)]
    # The float (glm-style) inverse is ill-conditioned for large far/near, so
    # compare what the matrix is used for: unprojected primary-ray directions.
    ndc = np.array([[x, y, 0.0, 1.0] for x in (-1, -0.3, 0, 0.7, 1) for y in (-1, 0.2, 1)], np.float64)
    for c in cases:
        m = wf.api.camera_screen_to_world(*c).astype(np.float64).reshape(4, 4).T
        o = orc.camera_screen_to_world(*c).astype(np.float64).reshape(4, 4).T
        eye = np.array(c[0], np.float64)
        wm = ndc @ m.T
        wo = ndc @ o.T
        dm = wm[:, :3] / wm[:, 3:] - eye
        do = wo[:, :3] / wo[:, 3:] - eye
        dm /= np.linalg.norm(dm, axis=1, keepdims=True)
        do /= np.linalg.norm(do, axis=1, keepdims=True)
        assert np.abs(dm - do).max() < 2e-4


def test_scene_generators_are_deterministic(wf):
    p1, n1, i1 = wf.api.generate_scene(0, 5, 1000)
    p2, n2, i2 = wf.api.generate_scene(0, 5, 1000)
    assert i1.shape == (1000, 3) and np.array_equal(p1, p2) and np.array_equal(i1, i2)
    assert np.allclose(np.linalg.norm(n1, axis=1), 1.0, atol=1e-5)
    pc, _, ic = wf.api.generate_scene(1, 1)
    assert ic.shape[0] == 268304
    assert pc.min() >= -1e-3 and pc[:, 0].max() <= 30.001 and pc[:, 1].max() <= 12.001
    _, _, ik = wf.api.generate_scene(3, 2, 60000)
    assert 40000 < ik.shape[0] < 90000


def _bvh2_arrays(nodes_u8, tris_u8):
    nodes = nodes_u8.view(np.float32).reshape(-1, 16)
    links = nodes_u8.view(np.int32).reshape(-1, 16)[:, 12:14]
    tris = tris_u8.view(np.float32).reshape(-1, 12)
    tri_ids = tris_u8.view(np.uint32).reshape(-1, 12)[:, 11]
    return nodes, links, tris, tri_ids


def test_bvh2_is_valid(wf):
    pos, _, idx = wf.api.generate_scene(0, 9, 3000)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, links, tris, ids = _bvh2_arrays(*sc.export_bvh2())
    assert np.array_equal(np.sort(ids), np.arange(3000))
    seen = 0
    stack = [0]
    while stack:
        n = stack.pop()
        f = nodes[n]
        boxes = [(f[[0, 2, 8]], f[[1, 3, 9]]), (f[[4, 6, 10]], f[[5, 7, 11]])]
        for c in range(2):
            lo, hi = boxes[c]
            link = int(links[n, c])
            if np.isinf(lo[0]):
                continue
            if link >= 0:
                stack.append(link)
                continue
            code = ~link & 0xFFFFFFFF
            first, cnt = code >> 3, (code & 7) + 1
            assert cnt <= 4
            v = tris[first:first + cnt][:, [0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(-1, 3)
            assert np.all(v >= lo) and np.all(v <= hi)
            seen += cnt
    assert seen == 3000


@pytest.mark.parametrize("ntris", [0, 1, 2, 9])
def test_tiny_and_empty_scenes_build(wf, ntris):
    """Scene creation for empty and few-triangle scenes (the empty BVHs
    carry one placeholder record)."""
    pos = np.arange(3 * 3 * max(ntris, 1), dtype=np.float32).reshape(-1, 3) * 0.1
    pos[:, 1] = np.sin(pos[:, 0])
    idx = np.arange(3 * ntris, dtype=np.uint32).reshape(-1, 3)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes_u8, tris_u8 = sc.export_bvh8()
    ids = tris_u8.view(np.uint32).reshape(-1, 12)[:, 11]
    if ntris:
        assert sorted(ids.tolist()) == list(range(ntris))
    else:
        assert ids.shape[0] == 1
    sc.close()


@pytest.mark.parametrize("collapse,tri_cost", [(1, 20), (1, 100), (0, 100)])
def test_bvh8_boxes_are_conservative(wf, collapse, tri_cost):
    """Every child box holds its subtree's triangles, every triangle appears
    once, for the SAH collapse (two cost ratios) and the greedy one."""
    pos, _, idx = wf.api.generate_scene(0, 4, 4000)
    old = wf.api.tune_get("build.bvh8.collapse"), wf.api.tune_get("build.bvh8.tri_cost")
    try:
        wf.api.tune_set("build.bvh8.collapse", collapse)
        wf.api.tune_set("build.bvh8.tri_cost", tri_cost)
        sc = wf.api.Scene(pos, idx, host_only=True)
    finally:
        wf.api.tune_set("build.bvh8.collapse", old[0])
        wf.api.tune_set("build.bvh8.tri_cost", old[1])
    nodes_u8, tris_u8 = sc.export_bvh8()
    nb = nodes_u8.reshape(-1, 80)
    tris = tris_u8.view(np.float32).reshape(-1, 12)
    ids = tris_u8.view(np.uint32).reshape(-1, 12)[:, 11]
    assert np.array_equal(np.sort(ids), np.arange(4000))

    def node(i):
        b = nb[i]
        p = b[0:12].view(np.float32)
        e = b[12:15].astype(np.int32)
        imask = int(b[15])
        child_base, tri_base = b[16:24].view(np.uint32)
        meta = b[24:32]
        q = b[32:80].reshape(6, 8).astype(np.float32)
        scale = np.ldexp(np.float32(1), e - 127).astype(np.float32)
        return p, scale, imask, int(child_base), int(tri_base), meta, q

    def subtree_tris(i, out):
        p, scale, imask, cb, tb, meta, q = node(i)
        for s in range(8):
            m = int(meta[s])
            if m == 0:
                continue
            if imask >> s & 1:
                subtree_tris(cb + bin(imask & ((1 << s) - 1)).count("1"), out)
            else:
                cnt = bin(m >> 5).count("1")
                out.extend(range(tb + (m & 31), tb + (m & 31) + cnt))

    total = 0
    for i in range(nb.shape[0]):
        p, scale, imask, cb, tb, meta, q = node(i)
        for s in range(8):
            m = int(meta[s])
            if m == 0:
                continue
            lo = (p + q[0:3, s] * scale).astype(np.float32)
            hi = (p + q[3:6, s] * scale).astype(np.float32)
            tl = []
            if imask >> s & 1:
                subtree_tris(cb + bin(imask & ((1 << s) - 1)).count("1"), tl)
            else:
                cnt = bin(m >> 5).count("1")
                assert (m >> 5) in (1, 3, 7) and (m & 31) + cnt <= 24
                tl = list(range(tb + (m & 31), tb + (m & 31) + cnt))
                total += cnt
            v = tris[tl][:, [0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(-1, 3)
            assert np.all(v >= lo) and np.all(v <= hi)
    assert total == 4000


def test_cpu_traversal_agrees_with_fp64(wf, orc):
    pos, _, idx = wf.api.generate_scene(0, 7, 20000)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, tris = sc.export_bvh2()
    rays = random_rays(np.random.default_rng(1), 20000)
    res = orc.trace_bvh2(nodes, tris, rays, closest=True)
    t64, tri64 = orc.Fp64Scene(pos, idx).trace(rays, closest=True)
    hit = res[:, 0] >= 0
    assert np.array_equal(hit, tri64 >= 0)
    assert np.mean(res[hit, 0] == tri64[hit]) > 0.9999
    t32 = res[hit, 2].view(np.float32).astype(np.float64)
    # FP32 hit distances: within 1e-5 relative, or 1e-6 of the scene scale
    # (the absolute floor set by FP32 coordinates).
    assert np.all(np.abs(t32 - t64[hit]) <= 1e-5 * t64[hit] + 1e-6 * 1.0)
    anyr = orc.trace_bvh2(nodes, tris, rays, closest=False)
    assert np.array_equal(anyr[:, 0] >= 0, hit)


def adversarial_rays(rng, pos, idx, n):
    """Rays that start on triangles (tmin 0), half of them on an edge, and
    rays aimed at edges and vertices from in front of the surface."""
    tri = rng.integers(0, idx.shape[0], n)
    v = pos[idx[tri]]
    w = rng.dirichlet((1, 1, 1), n).astype(np.float32)
    w[: n // 4, 2] = 0.0
    w[n // 8: n // 4, 1] = 0.0  # a vertex
    w /= np.maximum(w.sum(1, keepdims=True), 1e-30)
    p = np.einsum("nk,nkd->nd", w, v).astype(np.float32)
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = p
    rays[n // 2:, :3] -= 2.0 * rays[n // 2:, 4:7]
    return rays


@pytest.mark.parametrize("scene", [(0, 9, 3000), (1, 1, 0)])
def test_bvh2_culling_is_conservative(wf, orc, scene):
    """The oracle's BVH2 traversal over the product's BVH (boxes grown by
    the build margin) returns the brute-force closest hit on rays that start
    on surfaces or hit edges and vertices, where culling with exact-fit boxes
    drops tied triangles."""
    kind, seed, ntris = scene
    pos, _, idx = wf.api.generate_scene(kind, seed, ntris)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, tris = sc.export_bvh2()
    rng = np.random.default_rng(31)
    n = 3000 if kind == 0 else 300
    rays = adversarial_rays(rng, pos, idx, n)
    a = orc.trace_bvh2(nodes, tris, rays)
    b = orc.trace_brute(tris, rays)
    assert np.array_equal(a, b)


def test_cpu_frame_runs(wf, orc):
    pos, nrm, idx = wf.api.generate_scene(0, 3, 4000)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, tris = sc.export_bvh2()
    geom = orc.HostGeometry(wf.api.gltf_vertices(pos, nrm), idx)
    cam = dict(position=(0.5, 0.5, 2.2), rotation=(0, 0, 0), fov=45.0, zn=0.001, zf=10.0)
    w, h = 32, 24
    s2w = wf.api.camera_screen_to_world(cam["position"], cam["rotation"], cam["fov"], w / h, cam["zn"], cam["zf"])
    cfg = orc.FrameCfg(ray_type=2, spp=1, S=2, depth=3, radius=0.1, key=0.6, white=2.0, albedo=0.8,
                       sort_shadow=1, reorder_shadow=1, sort_path=1, reorder_path=1, morton_kind=0, frame_index=1)
    px, fp, st = orc.render_frame(nodes, tris, geom, sc.bounds_min, sc.bounds_max, [0.5, 1.5, 0.5], [0.2, 0.3, 0.9],
                                  s2w, cam["position"], cam["zf"], w, h, cfg)
    assert st.primary == w * h
    assert 0 < st.path <= 3 * w * h
    assert np.all(np.isfinite(fp)) and np.all(fp[:, 3] == 1.0)


def test_tuning_knobs(wf):
    api = wf.api
    old = (api.tune_get("trace.bvh8.refill"), api.tune_get("trace.bvh8.postpone"), api.tune_get("trace.bvh8.coop"),
           api.tune_get("trace.bvh8.batch"), api.tune_get("trace.bvh8.steps"), api.tune_get("trace.bvh8.any_batch"),
           api.tune_get("trace.bvh8.any_steps"))
    # cooperative tests by default: batched over two node steps for closest-hit rays, after every
    # iteration of three node steps for any-hit rays
    assert old[2] == 1 and old[3] == 24 and old[4] == 2 and old[5] == 1 and old[6] == 3
    try:
        api.tune_set("trace.bvh8.refill", 4)
        api.tune_set("trace.bvh8.postpone", 6)
        api.tune_set("trace.bvh8.coop", 0)
        api.tune_set("trace.bvh8.batch", 9)
        api.tune_set("trace.bvh8.steps", 3)
        api.tune_set("trace.bvh8.any_batch", 7)
        api.tune_set("trace.bvh8.any_steps", 5)
        assert api.tune_get("trace.bvh8.any_batch") == 7 and api.tune_get("trace.bvh8.any_steps") == 5
        assert api.tune_get("trace.bvh8.batch") == 9  # the kinds are independent
        assert api.tune_get("trace.bvh8.refill") == 4 and api.tune_get("trace.bvh8.postpone") == 6
        assert api.tune_get("trace.bvh8.coop") == 0 and api.tune_get("trace.bvh8.batch") == 9
        assert api.tune_get("trace.bvh8.steps") == 3
        for key, bad in (("trace.bvh8.refill", 0), ("trace.bvh8.refill", 33), ("trace.bvh8.postpone", -1),
                         ("trace.bvh8.batch", 0), ("trace.bvh8.batch", 33), ("trace.bvh8.steps", 0),
                         ("trace.bvh8.steps", 9), ("trace.bvh8.any_batch", 0), ("trace.bvh8.any_batch", 33),
                         ("trace.bvh8.any_steps", 0), ("trace.bvh8.any_steps", 9),
                         ("trace.bvh8.coop", 2), ("sort.tiles", 4), ("sort.tiles", -1), ("sort.digit_bits", 5), ("sort.digit_bits", 16), ("build.bvh8.collapse", 2),
                         ("build.bvh8.tri_cost", 0), ("build.bvh8.tri_cost", 10001), ("build.ploc.radius", 0),
                         ("build.ploc.radius", 65), ("debug.fail_alloc_after", -2), ("no.such.knob", 1)):
            with pytest.raises(wf.WfptError):
                api.tune_set(key, bad)
    finally:
        api.tune_set("trace.bvh8.refill", old[0])
        api.tune_set("trace.bvh8.postpone", old[1])
        api.tune_set("trace.bvh8.coop", old[2])
        api.tune_set("trace.bvh8.batch", old[3])
        api.tune_set("trace.bvh8.steps", old[4])
        api.tune_set("trace.bvh8.any_batch", old[5])
        api.tune_set("trace.bvh8.any_steps", old[6])


def test_batch_arguments_rejected_on_host(wf):
    lib = wf._lib.load()
    out = C.c_void_p()
    req = (wf._lib.Request * 1)()
    assert lib.wfpt_batch_create(req, 0, 1, C.byref(out)) == 1
    assert lib.wfpt_batch_create(req, 1, 0, C.byref(out)) == 1
    assert lib.wfpt_batch_create(req, 1, 17, C.byref(out)) == 1
    assert lib.wfpt_batch_create(req, 1, 2, C.byref(out)) == 1  # null scene
    assert b"null scene" in lib.wfpt_last_error_message()
    assert not out
    st = wf._lib.RenderStats()
    assert lib.wfpt_batch_get_stats(None, 0, C.byref(st)) == 1
    assert lib.wfpt_batch_render(None, None, None) == 1
