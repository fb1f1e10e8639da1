"""Traversal through the C ABI.

Plain form (BVH2 FP32) is bit-exact against the oracle's CPU traversal of
the same BVH; the chosen form (BVH8 with 8-bit boxes) returns the same
closest hits as the plain form (same watertight test and tie rule); both
agree with the FP64 oracle: primitive ids except at ties, hit distance
within 1e-5 relative or 1e-6 of the scene scale (the FP32 coordinate floor).
"""
import numpy as np
import pytest

from conftest import random_rays

pytestmark = pytest.mark.gpu


def _fp64_pair(rays, pos, idx, tri):
    """t and barycentrics (u, v) of given (ray, triangle) pairs in double
    (Moller-Trumbore on the float inputs taken as exact)."""
    v = pos[idx[tri]].astype(np.float64)
    o, d = rays[:, 0:3].astype(np.float64), rays[:, 4:7].astype(np.float64)
    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    p = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, p)
    tv = o - v[:, 0]
    u = np.einsum("ij,ij->i", tv, p) / det
    q = np.cross(tv, e1)
    w = np.einsum("ij,ij->i", d, q) / det
    return np.einsum("ij,ij->i", e2, q) / det, u, w


def assert_fp64_parity(g, rays, pos, idx, t64, tri64):
    """The FP64 gate for FP32 closest hits g against the FP64 oracle's
    (t64, tri64):
    - at least 99.9 % of hits have |t - t64| <= 1e-5 * t64 (measured 99.96 %
      on the soup, 99.98 % on the city);
    - every hit is within 1e-5 * t64 + 2^-24 * (|o|_inf + |p|_inf), p the
      hit point: the FP32 floor of a distance computed from coordinates of
      that size (measured at most 0.09 of the floor term beyond 1e-5 t64);
    - a different primitive is only accepted at a t-tie: the GPU's triangle,
      intersected in double, lies within the same bound of t64 and its
      barycentrics within [-1e-6, 1 + 1e-6];
    - a hit on one side and a miss on the other only where the hit triangle
      is grazed within 1e-6 of an edge (barycentric)."""
    hit, hit64 = g[:, 0] >= 0, tri64 >= 0
    p64 = rays[:, 0:3].astype(np.float64) + np.where(hit64, t64, 0.0)[:, None] * rays[:, 4:7]
    floor = 2.0**-24 * (np.abs(rays[:, 0:3]).max(1) + np.abs(p64).max(1))
    both = hit & hit64
    t32 = g[:, 2].view(np.float32).astype(np.float64)
    err = np.abs(t32 - t64)
    assert np.mean(err[both] <= 1e-5 * t64[both]) >= 0.999
    assert np.all(err[both] <= 1e-5 * t64[both] + floor[both])
    mm = np.nonzero(both & (g[:, 0] != tri64))[0]
    if mm.size:
        tg, ug, vg = _fp64_pair(rays[mm], pos, idx, g[mm, 0])
        assert np.all(np.abs(tg - t64[mm]) <= 1e-5 * t64[mm] + floor[mm])
        assert np.all(np.minimum(np.minimum(ug, vg), 1 - ug - vg) >= -1e-6)
    hm = np.nonzero(hit != hit64)[0]
    if hm.size:
        tri = np.where(hit[hm], g[hm, 0], tri64[hm])
        _, u, v = _fp64_pair(rays[hm], pos, idx, tri)
        assert np.all(np.abs(np.minimum(np.minimum(u, v), 1 - u - v)) <= 1e-6)
    assert mm.size + hm.size <= 1e-4 * len(g)


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def N(t):
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def soup(wf):
    pos, nrm, idx = wf.api.generate_scene(0, 1, 65536)
    sc = wf.api.Scene(pos, idx)
    return pos, idx, sc


@pytest.fixture(scope="module")
def courtyard(wf):
    pos, nrm, idx = wf.api.generate_scene(1, 1)
    sc = wf.api.Scene(pos, idx)
    return pos, idx, sc


def gpu_trace(wf, dev, sc, kind, rays, closest=True, ray_index=None):
    import torch
    out = torch.full((rays.shape[0], 4), 77, dtype=torch.int32, device=dev)
    wf.api.trace(sc, kind, T(rays, dev), out, ray_index=None if ray_index is None else T(ray_index, dev),
                 closest_hit=closest)
    return N(out)


def test_bvh2_bit_exact_vs_cpu_traversal(wf, orc, dev, soup):
    pos, idx, sc = soup
    nodes, tris = sc.export_bvh2()
    rays = random_rays(np.random.default_rng(2), 200000)
    g = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays)
    c = orc.trace_bvh2(nodes, tris, rays)
    assert np.array_equal(g, c)
    ga = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays, closest=False)
    ca = orc.trace_bvh2(nodes, tris, rays, closest=False)
    assert np.array_equal(ga, ca)
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("scene", ["soup", "courtyard"])
def test_bvh8_equals_bvh2(wf, dev, scene, request):
    pos, idx, sc = request.getfixturevalue(scene)
    lo, hi = sc.bounds_min, sc.bounds_max
    rng = np.random.default_rng(3)
    n = 300000
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = o
    g2 = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays)
    g8 = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays)
    assert np.array_equal(g2, g8)
    a8 = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays, closest=False)
    assert np.array_equal(a8[:, 0] >= 0, g2[:, 0] >= 0)
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("collapse,tri_cost", [(0, 100), (1, 100), (1, 5)])
def test_bvh8_collapse_policies_equal_bvh2(wf, dev, collapse, tri_cost):
    """The greedy and SAH collapses (different tree shapes and leaf sizes)
    give the BVH2's closest hits on the courtyard."""
    pos, nrm, idx = wf.api.generate_scene(1, 1)
    old = wf.api.tune_get("build.bvh8.collapse"), wf.api.tune_get("build.bvh8.tri_cost")
    try:
        wf.api.tune_set("build.bvh8.collapse", collapse)
        wf.api.tune_set("build.bvh8.tri_cost", tri_cost)
        sc = wf.api.Scene(pos, idx)
    finally:
        wf.api.tune_set("build.bvh8.collapse", old[0])
        wf.api.tune_set("build.bvh8.tri_cost", old[1])
    lo, hi = sc.bounds_min, sc.bounds_max
    rng = np.random.default_rng(13)
    n = 200000
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    g2 = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays)
    g8 = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays)
    assert np.array_equal(g2, g8)
    a8 = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays, closest=False)
    assert np.array_equal(a8[:, 0] >= 0, g2[:, 0] >= 0)
    sc.close()
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("kind", [0, 1])
def test_against_fp64(wf, orc, dev, soup, kind):
    pos, idx, sc = soup
    rays = random_rays(np.random.default_rng(5 + kind), 100000)
    g = gpu_trace(wf, dev, sc, kind, rays)
    t64, tri64 = orc.Fp64Scene(pos, idx).trace(rays)
    assert_fp64_parity(g, rays, pos, idx, t64, tri64)


def test_indirect_index_and_empty_interval(wf, dev, soup):
    pos, idx, sc = soup
    rng = np.random.default_rng(8)
    rays = random_rays(rng, 50000)
    rays[::9, 7] = -1.0  # tmax < tmin: miss (raygenShadow.comp:129 dummy rays)
    direct = gpu_trace(wf, dev, sc, 1, rays)
    assert np.all(direct[::9, 0] == -1) and np.all(direct[::9, 2].view(np.float32) == -1.0)
    perm = rng.permutation(50000).astype(np.uint32)
    ind = gpu_trace(wf, dev, sc, 1, rays, ray_index=perm.view(np.int32))
    assert np.array_equal(ind, direct)


def test_miss_record_and_device_count(wf, dev, soup):
    import torch
    pos, idx, sc = soup
    rays = random_rays(np.random.default_rng(1), 1000)
    rays[:, :3] += 10.0  # outside the scene, pointing anywhere: mostly misses
    out = torch.full((1000, 4), 5, dtype=torch.int32, device=dev)
    cnt = torch.tensor([600], dtype=torch.int32, device=dev)
    wf.api.trace(sc, 1, T(rays, dev), out, n_dev=cnt)
    o = N(out)
    miss = o[:600, 0] == -1
    assert np.all(o[:600][miss][:, 1] == -1) and np.all(o[:600][miss][:, 3] == 0)
    assert np.all(o[600:] == 5)


@pytest.mark.parametrize("batch,steps", [(1, 1), (16, 2), (32, 3)])
@pytest.mark.parametrize("closest", [True, False])
def test_bvh8_batched_tests_indirect_device_count(wf, dev, soup, batch, steps, closest):
    """Batched cooperative tests with an indirect index, empty intervals and
    a device-side count below n: the first count rays (through the index)
    get the BVH2's hit (any hit: its hit flag), the rest are untouched."""
    import torch
    pos, idx, sc = soup
    rng = np.random.default_rng(31 + batch + steps)
    n, count = 40000, 27777
    rays = random_rays(rng, n)
    rays[::7, 7] = -1.0  # tmax < tmin: miss
    perm = rng.permutation(n).astype(np.uint32)
    ref = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays, closest=closest)
    keys = ("trace.bvh8.batch", "trace.bvh8.steps", "trace.bvh8.any_batch", "trace.bvh8.any_steps")
    old = [wf.api.tune_get(k) for k in keys]
    try:
        for k, v in zip(keys, (batch, steps, batch, steps)):
            wf.api.tune_set(k, v)
        out = torch.full((n, 4), 77, dtype=torch.int32, device=dev)
        cnt = torch.tensor([count], dtype=torch.int32, device=dev)
        wf.api.trace(sc, wf.BVH8_Q8, T(rays, dev), out, ray_index=T(perm.view(np.int32), dev), n_dev=cnt,
                     closest_hit=closest)
        o = N(out)
    finally:
        for k, v in zip(keys, old):
            wf.api.tune_set(k, v)
    done = perm[:count]
    rest = np.setdiff1d(np.arange(n), done)
    if closest:
        assert np.array_equal(o[done], ref[done])
    else:
        assert np.array_equal(o[done, 0] >= 0, ref[done, 0] >= 0)
    assert np.all(o[rest] == 77)
    assert wf.api.device_status() == 0


def test_empty_and_tiny_scenes(wf, dev):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    idx = np.array([[0, 1, 2]], np.uint32)
    sc = wf.api.Scene(pos, idx)
    rays = np.zeros((2, 8), np.float32)
    rays[:, :3] = [[0.2, 0.2, 1.0], [2.0, 2.0, 1.0]]
    rays[:, 6] = -1.0
    rays[:, 7] = 10.0
    for kind in (0, 1):
        o = gpu_trace(wf, dev, sc, kind, rays)
        assert o[0, 0] == 0 and o[0, 1] == 0 and abs(o[0, 2].view(np.float32) - 1.0) < 1e-6
        u, v = (o[0, 3] & 0xFFFF) / 65535.0, (o[0, 3] >> 16) / 65535.0
        assert abs(u - 0.2) < 1e-4 and abs(v - 0.2) < 1e-4
        assert o[1, 0] == -1
    empty = wf.api.Scene(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    for kind in (0, 1):
        assert np.all(gpu_trace(wf, dev, empty, kind, rays)[:, 0] == -1)


def test_multi_geometry_ids(wf, dev):
    pos, nrm, idx = wf.api.generate_scene(0, 3, 3000)
    sc = wf.api.Scene(pos, idx, geometry_first=[0, 1000, 2500])
    rays = random_rays(np.random.default_rng(4), 20000)
    o = gpu_trace(wf, dev, sc, 1, rays)
    hit = o[o[:, 0] >= 0]
    glob = np.where(hit[:, 1] == 0, hit[:, 0], np.where(hit[:, 1] == 1, hit[:, 0] + 1000, hit[:, 0] + 2500))
    assert np.all((glob >= 0) & (glob < 3000))
    assert set(np.unique(hit[:, 1])) <= {0, 1, 2}
    assert np.all(hit[hit[:, 1] == 1, 0] < 1500) and np.all(hit[hit[:, 1] == 2, 0] < 500)


@pytest.mark.parametrize("coop,batch,steps", [(0, 16, 2), (1, 1, 1), (1, 7, 1), (1, 16, 2), (1, 32, 3), (1, 24, 8)])
@pytest.mark.parametrize("refill,postpone", [(1, 0), (32, 0), (8, 8), (4, 16)])
def test_bvh8_knobs_do_not_change_hits(wf, dev, soup, refill, postpone, coop, batch, steps):
    pos, idx, sc = soup
    rays = random_rays(np.random.default_rng(12), 60000)
    ref = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays)
    ref_any = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays, closest=False)
    keys = ("trace.bvh8.refill", "trace.bvh8.postpone", "trace.bvh8.coop", "trace.bvh8.batch", "trace.bvh8.steps",
            "trace.bvh8.any_batch", "trace.bvh8.any_steps")
    old = [wf.api.tune_get(k) for k in keys]
    try:
        for k, v in zip(keys, (refill, postpone, coop, batch, steps, batch, steps)):
            wf.api.tune_set(k, v)
        assert np.array_equal(gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays), ref)
        a8 = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays, closest=False)
        assert np.array_equal(a8[:, 0] >= 0, ref_any[:, 0] >= 0)
        hit = a8[:, 0] >= 0
        # An any-hit result is a genuine hit: same record layout, t inside
        # the ray interval.
        t = a8[hit, 2].view(np.float32)
        assert np.all((t >= rays[hit, 3]) & (t <= rays[hit, 7]))
    finally:
        for k, v in zip(keys, old):
            wf.api.tune_set(k, v)
    assert wf.api.device_status() == 0


def test_bvh8_coop_courtyard_and_ties(wf, orc, dev, courtyard):
    """Cooperative and per-lane triangle tests give identical closest hits
    on the courtyard, including rays that start on a triangle (tmin 0) and
    rays through shared edges."""
    pos, idx, sc = courtyard
    rng = np.random.default_rng(21)
    n = 200000
    tri = rng.integers(0, idx.shape[0], n)
    v = pos[idx[tri]]  # [n, 3, 3]
    w = rng.dirichlet((1, 1, 1), n).astype(np.float32)
    w[: n // 4, 2] = 0.0  # on an edge
    w[: n // 4] /= w[: n // 4].sum(1, keepdims=True)
    p = np.einsum("nk,nkd->nd", w, v).astype(np.float32)
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = p
    rays[n // 2:, :3] -= 3.0 * rays[n // 2:, 4:7]  # in front of the surface, looking at it
    old = wf.api.tune_get("trace.bvh8.coop")
    try:
        wf.api.tune_set("trace.bvh8.coop", 0)
        lane = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays)
        wf.api.tune_set("trace.bvh8.coop", 1)
        coop = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays)
    finally:
        wf.api.tune_set("trace.bvh8.coop", old)
    assert np.array_equal(lane, coop)
    # Both BVH forms cull conservatively (boxes grown by the build margin), so rays that
    # start on a surface with tmin 0 and rays through shared edges resolve
    # their ties the same way in both, and the same as the oracle.
    plain = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays)
    assert np.array_equal(coop, plain)
    nodes, tris = sc.export_bvh2()
    sub = np.random.default_rng(22).choice(n, 20000, replace=False)
    assert np.array_equal(plain[sub], orc.trace_bvh2(nodes, tris, rays[sub]))


def test_city_3m_triangles_against_fp64(wf, orc, dev):
    """City block of 3,000,320 triangles: 1M sampled incoherent rays.  BVH8
    and BVH2 return identical hits, which pass the FP64 gate of
    assert_fp64_parity."""
    pos, nrm, idx = wf.api.generate_scene(2, 1)
    assert idx.shape[0] == 3000320
    sc = wf.api.Scene(pos, idx)
    rng = np.random.default_rng(9)
    n = 1 << 20
    lo, hi = sc.bounds_min, sc.bounds_max
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    g8 = gpu_trace(wf, dev, sc, wf.BVH8_Q8, rays)
    g2 = gpu_trace(wf, dev, sc, wf.BVH2_FP32, rays)
    assert np.array_equal(g8, g2)
    t64, tri64 = orc.Fp64Scene(pos, idx).trace(rays)
    assert_fp64_parity(g8, rays, pos, idx, t64, tri64)
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("morton_kind", [0, 1, 2])
@pytest.mark.parametrize("kind", [0, 1])
def test_trace_sort_composite(wf, dev, courtyard, kind, morton_kind):
    """wfpt_trace_sort (Tracer::traceSort): indirect results equal a plain
    trace at every slot; reordered results equal the plain hit of the ray
    that sorted into each slot, and the slot maps follow the rays."""
    import torch
    pos, idx, sc = courtyard
    rng = np.random.default_rng(40 + morton_kind)
    n = 123457
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = rng.uniform(sc.bounds_min, sc.bounds_max, (n, 3)).astype(np.float32)
    plain = gpu_trace(wf, dev, sc, kind, rays)
    d_rays = T(rays, dev)
    res = torch.empty((n, 4), dtype=torch.int32, device=dev)
    keys = torch.empty(n, dtype=torch.int64, device=dev)
    ids = torch.empty(n, dtype=torch.int32, device=dev)
    wf.api.trace_sort(sc, kind, d_rays, res, sc.bounds_min, sc.bounds_max, morton_kind, False, keys, ids)
    assert np.array_equal(N(res), plain)
    out = torch.empty_like(d_rays)
    # Slot -> index map: a permutation of [0, n) (pixel indices in the
    # renderer); the reorder writes index_to_slot_out at these values.
    perm = rng.permutation(n).astype(np.int32)
    s2i = T(perm, dev)
    os2i = torch.empty(n, dtype=torch.int32, device=dev)
    oi2s = torch.empty(n, dtype=torch.int32, device=dev)
    wf.api.trace_sort(sc, kind, d_rays, res, sc.bounds_min, sc.bounds_max, morton_kind, True, keys, ids,
                      rays_out=out, slot_to_index=s2i, slot_to_index_out=os2i, index_to_slot_out=oi2s)
    order = N(ids).view(np.uint32)
    assert np.array_equal(np.sort(order), np.arange(n))
    assert np.array_equal(N(res), plain[order])
    assert np.array_equal(N(out), rays[order])
    assert np.array_equal(N(os2i), perm[order])
    assert np.array_equal(N(oi2s)[perm[order]], np.arange(n))
    assert wf.api.device_status() == 0
