"""wfpt_raygen_path_static (compaction over the library's fixed device
scratch, no allocation) against wfpt_raygen_path with caller scratch, through
the C ABI, on two calls in a row.  Collected last so that it also runs after
every other GPU test in one process; it passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from conftest import random_rays

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def N(t):
    return t.cpu().numpy()


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def scene(wf, orc):
    pos, nrm, idx = wf.api.generate_scene(0, 33, 20000)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, tris = sc.export_bvh2()
    return pos, nrm, idx, nodes, tris


def _inputs(orc, scene, n, seed):
    pos, nrm, idx, nodes, tris = scene
    rng = np.random.default_rng(seed)
    rays = random_rays(rng, n)
    res = orc.trace_bvh2(nodes, tris, rays)
    seeds = rng.integers(0, 2**32, n, dtype=np.uint32)
    i2p = rng.permutation(n).astype(np.int32)
    dec = rng.uniform(0.1, 1.0, (n, 4)).astype(np.float32)
    return rays, res, seeds, i2p, dec


def _run(wf, dev, fn, geom, inp, n):
    import torch
    rays, res, seeds, i2p, dec = inp
    d_seeds = T(seeds.view(np.int32), dev)
    d_dec = T(dec, dev)
    out = torch.zeros((n, 8), dtype=torch.float32, device=dev)
    o_i2p = torch.zeros(n, dtype=torch.int32, device=dev)
    cnt = torch.full((1,), 777, dtype=torch.int32, device=dev)
    fn(d_seeds, geom.table, T(rays, dev), out, T(i2p, dev), o_i2p, T(res, dev), d_dec, cnt, albedo=0.8)
    torch.cuda.synchronize()
    c = int(N(cnt)[0])
    return c, N(out)[:c], N(o_i2p)[:c], N(d_seeds), N(d_dec)


def test_static_scratch_matches_caller_scratch_twice(wf, orc, dev, scene):
    pos, nrm, idx, nodes, tris = scene
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    # Two calls in a row on one stream; the second covers more tiles than
    # the first, so state left over from the first call would show.
    for n, seed in ((40000, 1), (70001, 2)):
        inp = _inputs(orc, scene, n, seed)
        ref = _run(wf, dev, wf.api.raygen_path, geom, inp, n)
        l0 = wf._lib.load().wfpt_kernel_launch_count()
        got = _run(wf, dev, wf.api.raygen_path_static, geom, inp, n)
        assert wf._lib.load().wfpt_kernel_launch_count() - l0 == 1
        assert 0 < ref[0] < n
        assert got[0] == ref[0]
        assert np.array_equal(bits(got[1]), bits(ref[1]))
        assert np.array_equal(got[2], ref[2])
        assert np.array_equal(got[3], ref[3])
        assert np.array_equal(bits(got[4]), bits(ref[4]))
    assert wf.api.device_status() == 0


def test_static_scratch_rejects_oversized_n(wf):
    lib = wf._lib.load()
    buf = C.c_void_p(0x1000)
    n = wf.api.RAYGEN_PATH_STATIC_MAX_RAYS + 1
    assert lib.wfpt_raygen_path_static(buf, buf, buf, buf, buf, buf, buf, buf, buf, n, None, 0, 0.8, None) == 1
    assert b"WFPT_RAYGEN_PATH_STATIC_MAX_RAYS" in lib.wfpt_last_error_message()
