"""wfpt_raygen_path_static (compaction over the library's fixed device
scratch, no allocation) against wfpt_raygen_path with caller scratch, through
the C ABI, on two calls in a row, at n = 0 and at the array's maximum n.
Collected last so that it also runs after every other GPU test in one
process; it passes alone as well."""
import ctypes as C
import os
import subprocess
import sys
import textwrap
from pathlib import Path

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
        a0 = wf.api.tune_get("debug.alloc_count")
        got = _run(wf, dev, wf.api.raygen_path_static, geom, inp, n)
        assert wf._lib.load().wfpt_kernel_launch_count() - l0 == 1
        assert wf.api.tune_get("debug.alloc_count") == a0  # the library allocated nothing
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


def _synthetic_inputs(n, ntri, dev, seed):
    """Device-made inputs for sizes the CPU oracle cannot trace quickly:
    random rays, and hit records naming random triangles of the geometry
    (about a third of them misses) with random t and packed barycentrics."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    rays = torch.rand((n, 8), generator=g, device=dev)
    d = torch.randn((n, 3), generator=g, device=dev)
    rays[:, 4:7] = d / d.norm(dim=1, keepdim=True)
    prim = torch.randint(0, ntri, (n,), generator=g, device=dev, dtype=torch.int32)
    miss = torch.rand(n, generator=g, device=dev) < 0.35
    res = torch.zeros((n, 4), dtype=torch.int32, device=dev)
    res[:, 0] = torch.where(miss, torch.full_like(prim, -1), prim)
    res[:, 1] = torch.where(miss, torch.full_like(prim, -1), torch.zeros_like(prim))
    res[:, 2] = torch.where(miss, torch.full((n,), -1.0, device=dev),
                            torch.rand(n, generator=g, device=dev) * 4 + 0.01).view(torch.int32)
    u = torch.randint(0, 32768, (n,), generator=g, device=dev, dtype=torch.int32)
    v = torch.randint(0, 32768, (n,), generator=g, device=dev, dtype=torch.int32)
    res[:, 3] = u | (v << 16)
    seeds = torch.randint(-2**31, 2**31 - 1, (n,), generator=g, device=dev, dtype=torch.int32)
    i2p = torch.randperm(n, generator=g, device=dev).to(torch.int32)
    dec = torch.rand((n, 4), generator=g, device=dev) * 0.9 + 0.1
    return rays, res, seeds, i2p, dec


def _run_dev(fn, geom, inp, n):
    import torch
    rays, res, seeds, i2p, dec = inp
    d_seeds, d_dec = seeds.clone(), dec.clone()
    out = torch.zeros((max(n, 1), 8), dtype=torch.float32, device=rays.device)
    o_i2p = torch.zeros(max(n, 1), dtype=torch.int32, device=rays.device)
    cnt = torch.full((1,), 777, dtype=torch.int32, device=rays.device)
    fn(d_seeds, geom.table, rays, out, i2p, o_i2p, res, d_dec, cnt, n=n, albedo=0.8)
    torch.cuda.synchronize()
    c = int(cnt.item())
    return c, out[:c], o_i2p[:c], d_seeds, d_dec


def test_static_scratch_top_of_array_and_empty(wf, dev, scene):
    """n = WFPT_RAYGEN_PATH_STATIC_MAX_RAYS uses every tile state of the
    array (the last word included); n = 0 launches one idle block and must
    write a zero count.  Both are compared with the caller-scratch entry."""
    import torch
    pos, nrm, idx, nodes, tris = scene
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    ntri = idx.reshape(-1, 3).shape[0]
    n = wf.api.RAYGEN_PATH_STATIC_MAX_RAYS
    inp = _synthetic_inputs(n, ntri, dev, 7)
    ref = _run_dev(wf.api.raygen_path, geom, inp, n)
    a0 = wf.api.tune_get("debug.alloc_count")
    got = _run_dev(wf.api.raygen_path_static, geom, inp, n)
    assert wf.api.tune_get("debug.alloc_count") == a0
    assert 0 < ref[0] < n
    assert got[0] == ref[0]
    for a, b in zip(got[1:], ref[1:]):
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    del inp, ref, got
    empty = _synthetic_inputs(1, ntri, dev, 8)
    for fn in (wf.api.raygen_path, wf.api.raygen_path_static):
        assert _run_dev(fn, geom, empty, 0)[0] == 0
    assert wf.api.device_status() == 0


_CAPTURE_CHILD = textwrap.dedent("""
    import sys
    sys.path.insert(0, sys.argv[1])
    import torch
    import vulkanwavefrontpathtracer_gb300 as wf
    lib = wf._lib.load()
    dev = torch.device("cuda:0")
    n = 1000
    bufs = [torch.zeros(n * 8, dtype=torch.float32, device=dev) for _ in range(8)]
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    args = [b.data_ptr() for b in bufs]
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        st = lib.wfpt_raygen_path_static(*args, cnt.data_ptr(), n, None, 0, 0.8, s.cuda_stream)
    msg = lib.wfpt_last_error_message().decode()
    assert st == 1, st
    assert "capturing" in msg, msg
    # Outside the capture the same call runs (every ray misses: zero hits).
    res = torch.full((n, 4), -1, dtype=torch.int32, device=dev)
    st = lib.wfpt_raygen_path_static(args[0], args[1], args[2], args[3], args[4], args[5], res.data_ptr(),
                                     args[7], cnt.data_ptr(), n, None, 0, 0.8, None)
    torch.cuda.synchronize()
    assert st == 0, lib.wfpt_last_error_message()
    assert int(cnt.item()) == 0
    print("capture-check-ok")
""")


def test_static_scratch_first_call_under_capture_is_refused(wf):
    """In a fresh process (a CUDA context where the entry point was never
    called), a first call made while the stream is capturing launches nothing
    and returns WFPT_ERR_INVALID_ARGUMENT; the next call outside the capture
    works."""
    root = str(Path(__file__).resolve().parents[1])
    r = subprocess.run([sys.executable, "-c", _CAPTURE_CHILD, root], capture_output=True, text=True,
                       timeout=300, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "capture-check-ok" in r.stdout


def test_allocation_counter_sees_library_allocations(wf, dev, scene):
    """The counter the tests above rely on does count the library's own
    device allocations: a renderer sizing its buffers for a first frame
    raises it."""
    import torch
    pos, nrm, idx, nodes, tris = scene
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    r = wf.api.Renderer(ray_type=wf.PATH_RAYS, recursion_depth=1, bvh_kind=wf.BVH8_Q8)
    r.set_scene(sc, geom, (0.5, 1.6, 0.5), (0.5, 0.8, 0.9))
    px = torch.zeros((32 * 32, 4), dtype=torch.float32, device=dev)
    a0 = wf.api.tune_get("debug.alloc_count")
    r.render(wf.api.make_camera(position=(0.5, 0.5, 2.2)), 32, 32, px, px.clone())
    torch.cuda.synchronize()
    assert wf.api.tune_get("debug.alloc_count") > a0
    r.close()
    sc.close()
