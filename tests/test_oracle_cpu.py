"""CPU checks of the oracle pieces that let a CPU run stand alone (the
reference arm of the bench maps no product library): its own BVH2 build,
the multi-threaded sort, the scene generator and the strided frame sample."""
import numpy as np

from conftest import random_rays


def test_parallel_sort_equals_stable_sort(orc):
    rng = np.random.default_rng(1)
    for n, bits in ((1, 32), (1000, 32), (300001, 32), (200003, 63), (100000, 48), (50000, 20)):
        if bits <= 32:
            keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
            keys[: n // 3] = keys[0]  # runs of equal keys: stability shows
        else:
            keys = rng.integers(0, 2**63, n, dtype=np.uint64)
            keys[: n // 3] &= np.uint64(0xFFFF)
        vals = np.arange(n, dtype=np.uint32)
        a = orc.sort_pairs(keys, vals, bits)
        b = orc.sort_pairs_mt(keys, vals, bits)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (n, bits)


def test_scene_generator_equals_product(wf, orc):
    for kind, seed, nt in ((0, 3, 1000), (1, 1, 0)):
        a = orc.generate_scene(kind, seed, nt)
        b = wf.api.generate_scene(kind, seed, nt)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_own_bvh2_hits_equal_product_bvh2(wf, orc):
    """The oracle's binned-SAH BVH2 and the product's BVH2 (both culling
    conservatively) give the same closest and any hits, including for rays
    that start on a surface."""
    pos, nrm, idx = orc.generate_scene(1, 1)
    nodes_o, tris_o = orc.bvh2_build(pos, idx)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes_p, tris_p = sc.export_bvh2()
    rng = np.random.default_rng(2)
    n = 60000
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = rng.uniform(sc.bounds_min, sc.bounds_max, (n, 3)).astype(np.float32)
    tri = rng.integers(0, idx.shape[0], n // 4)
    w = rng.dirichlet((1, 1, 1), n // 4).astype(np.float32)
    rays[: n // 4, :3] = np.einsum("nk,nkd->nd", w, pos[idx[tri]]).astype(np.float32)  # on a triangle
    for closest in (True, False):
        a = orc.trace_bvh2(nodes_o, tris_o, rays, closest=closest)
        b = orc.trace_bvh2(nodes_p, tris_p, rays, closest=closest)
        if closest:
            assert np.array_equal(a, b)
        else:
            assert np.array_equal(a[:, 0] >= 0, b[:, 0] >= 0)


def test_strided_frame_sample(wf, orc):
    """pixel_stride k renders every k-th slot of the full frame's pixel table:
    stride 1 is the full frame; with stride 3 the primary rays are the
    sampled slots and only their pixels receive colour."""
    pos, nrm, idx = orc.generate_scene(0, 1, 4000)
    nodes, tris = orc.bvh2_build(pos, idx)
    hg = orc.HostGeometry(orc.gltf_vertices(pos, nrm), idx)
    w, h = 40, 30
    s2w = orc.camera_screen_to_world((0.5, 0.5, 2.2), (0, 0, 0), 45.0, w / h, 0.001, 10.0)
    smin, smax = pos.min(0), pos.max(0)
    outs = []
    for stride in (0, 1, 3):
        cfg = orc.FrameCfg(ray_type=2, spp=1, S=2, depth=2, radius=0.1, key=0.6, white=2.0, albedo=0.8,
                           frame_index=1, pixel_stride=stride)
        outs.append(orc.render_frame(nodes, tris, hg, smin, smax, (0.5, 1.6, 0.5), (0.5, 0.8, 0.9), s2w,
                                     (0.5, 0.5, 2.2), 10.0, w, h, cfg))
    assert np.array_equal(outs[0][0], outs[1][0])
    st3 = outs[2][2]
    i2p, _ = orc.pixel_table(w, h)
    assert st3.primary == len(i2p[::3])
    lit = np.zeros(w * h, bool)
    lit[i2p[::3]] = True
    px3 = outs[2][0]  # frame 1: the accumulated colour before tone mapping
    assert np.all(px3[~lit, :3] == 0) and np.mean(px3[lit, :3].sum(1) > 0) > 0.5  # some are in full shadow
