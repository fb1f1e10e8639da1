"""Device BVH build (PLOC BVH2 + SAH collapse into the BVH8) through the C
ABI: a device-built scene returns exactly the hits of the host-built scene
of the same mesh (closest hits do not depend on the tree: watertight test,
smallest-t-then-index tie rule, conservative boxes), and its exported BVHs
hold every triangle once inside conservative child boxes."""
import numpy as np
import pytest

from conftest import random_rays

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def trace(wf, dev, sc, kind, rays, closest=True):
    import torch
    out = torch.full((rays.shape[0], 4), 77, dtype=torch.int32, device=dev)
    wf.api.trace(sc, kind, T(rays, dev), out, closest_hit=closest)
    return out.cpu().numpy()


def scene_rays(sc, n, seed):
    rng = np.random.default_rng(seed)
    rays = random_rays(rng, n, tmax=1e30)
    rays[:, :3] = rng.uniform(sc.bounds_min, sc.bounds_max, (n, 3)).astype(np.float32)
    return rays


def check_bvh2(nodes_u8, tris_u8, ntris):
    nodes = nodes_u8.view(np.float32).reshape(-1, 16)
    links = nodes_u8.view(np.int32).reshape(-1, 16)[:, 12:14]
    tris = tris_u8.view(np.float32).reshape(-1, 12)
    ids = tris_u8.view(np.uint32).reshape(-1, 12)[:, 11]
    assert np.array_equal(np.sort(ids), np.arange(ntris))
    seen = np.zeros(tris.shape[0], np.int32)
    stack = [0]
    while stack:
        i = stack.pop()
        f = nodes[i]
        for c in range(2):
            lo = np.array([f[0], f[2], f[8]] if c == 0 else [f[4], f[6], f[10]], np.float32)
            hi = np.array([f[1], f[3], f[9]] if c == 0 else [f[5], f[7], f[11]], np.float32)
            link = int(links[i, c])
            if link >= 0:
                stack.append(link)
                continue
            code = ~link & 0xFFFFFFFF
            first, cnt = code >> 3, (code & 7) + 1
            for r in range(first, first + cnt):
                seen[r] += 1
                v = tris[r][[0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(3, 3)
                assert np.all(v >= lo) and np.all(v <= hi)
    assert np.all(seen == 1)


@pytest.fixture(scope="module")
def courtyard_pair(wf):
    pos, nrm, idx = wf.api.generate_scene(1, 1)
    host = wf.api.Scene(pos, idx)
    devb = wf.api.Scene(pos, idx, device_build=True)
    return pos, idx, host, devb


def test_device_build_equals_host_hits(wf, dev, courtyard_pair):
    pos, idx, host, devb = courtyard_pair
    assert devb.info.num_triangles == idx.shape[0]
    assert np.array_equal(devb.bounds_min, host.bounds_min) and np.array_equal(devb.bounds_max, host.bounds_max)
    rays = scene_rays(host, 300000, 1)
    ref = trace(wf, dev, host, wf.BVH2_FP32, rays)
    for kind in (wf.BVH2_FP32, wf.BVH8_Q8):
        assert np.array_equal(trace(wf, dev, devb, kind, rays), ref)
        occl = trace(wf, dev, devb, kind, rays, closest=False)
        assert np.array_equal(occl[:, 0] >= 0, ref[:, 0] >= 0)
    assert wf.api.device_status() == 0


def test_device_built_bvhs_are_valid(wf, courtyard_pair):
    pos, idx, host, devb = courtyard_pair
    nodes, tris = devb.export_bvh2()
    assert nodes.size == 64 * devb.info.bvh2_nodes and devb.info.bvh2_nodes == idx.shape[0] - 1
    check_bvh2(nodes, tris, idx.shape[0])
    nodes8, tris8 = devb.export_bvh8()
    assert nodes8.size == 80 * devb.info.bvh8_nodes
    ids = tris8.view(np.uint32).reshape(-1, 12)[:, 11]
    assert np.array_equal(np.sort(ids), np.arange(idx.shape[0]))


@pytest.mark.parametrize("ntris", [2, 3, 17, 4097])
def test_device_build_small_scenes(wf, dev, ntris):
    pos, _, idx = wf.api.generate_scene(0, 11, ntris)
    host = wf.api.Scene(pos, idx)
    devb = wf.api.Scene(pos, idx, device_build=True)
    rays = scene_rays(host, 20000, ntris)
    assert np.array_equal(trace(wf, dev, devb, wf.BVH8_Q8, rays), trace(wf, dev, host, wf.BVH2_FP32, rays))
    nodes, tris = devb.export_bvh2()
    check_bvh2(nodes, tris, ntris)


def test_device_build_from_device_tensors_and_geometries(wf, dev):
    import torch
    pos, _, idx = wf.api.generate_scene(0, 12, 30000)
    gf = np.array([0, 1000, 1000, 29999], np.uint32)
    host = wf.api.Scene(pos, idx, geometry_first=gf)
    devb = wf.api.Scene.from_device(T(pos, dev), T(idx.astype(np.int32), dev), geometry_first=gf)
    rays = scene_rays(host, 50000, 5)
    g = trace(wf, dev, devb, wf.BVH8_Q8, rays)
    assert np.array_equal(g, trace(wf, dev, host, wf.BVH8_Q8, rays))
    assert set(np.unique(g[g[:, 0] >= 0, 1]).tolist()) <= {0, 2, 3}
    torch.cuda.synchronize()


def test_device_build_rejects_bad_index(wf, dev):
    pos, _, idx = wf.api.generate_scene(0, 13, 100)
    bad = idx.copy()
    bad[7, 1] = pos.shape[0]
    with pytest.raises(wf.WfptError):
        wf.api.Scene.from_device(T(pos, dev), T(bad.astype(np.int32), dev))
    with pytest.raises(wf.WfptError):
        wf.api.Scene(pos, bad, device_build=True)
    assert wf.api.device_status() == 0


def test_device_build_one_triangle_and_city(wf, dev):
    pos, _, idx = wf.api.generate_scene(0, 14, 1)
    one = wf.api.Scene.from_device(T(pos, dev), T(idx.astype(np.int32), dev))
    assert one.info.num_triangles == 1
    pos, nrm, idx = wf.api.generate_scene(2, 1)  # city block, 3M triangles
    devb = wf.api.Scene(pos, idx, device_build=True)
    host = wf.api.Scene(pos, idx, bvh2=False)
    assert devb.info.build_ms > 0
    rays = scene_rays(devb, 200000, 9)
    g = trace(wf, dev, devb, wf.BVH8_Q8, rays)
    assert np.array_equal(g, trace(wf, dev, devb, wf.BVH2_FP32, rays))
    assert np.array_equal(g, trace(wf, dev, host, wf.BVH8_Q8, rays))
    assert wf.api.device_status() == 0
