"""Stage kernels through the C ABI against the CPU oracle, bit-exact.

Every float kernel evaluates the shader arithmetic with one IEEE rounding
per operation (no FMA contraction), like the oracle, so outputs must match
to the bit."""
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


def test_init_seeds(wf, orc, dev):
    import torch
    for n, frame in [(1, 1), (1000, 3), (65543, 12)]:
        s = torch.empty(n, dtype=torch.int32, device=dev)
        wf.api.init_seeds(s, frame)
        assert np.array_equal(N(s).view(np.uint32), orc.init_seeds(n, frame))


def test_raygen_primary(wf, orc, dev):
    import torch
    for (w, h), sample in [((37, 23), 0), ((256, 256), 5), ((64, 48), 1023)]:
        m = wf.api.camera_screen_to_world((0.5, 0.5, 2.5), (-10, 20, 5), 45.0, w / h, 0.001, 3.0)
        i2p, _ = wf.api.pixel_table(w, h)
        rays = torch.empty((w * h, 8), dtype=torch.float32, device=dev)
        wf.api.raygen_primary(m, T(i2p, dev), rays, (0.5, 0.5, 2.5), sample, w, h, 3.0)
        ref = orc.raygen_primary(m, i2p, (0.5, 0.5, 2.5), sample, w, h, 3.0)
        assert np.array_equal(bits(N(rays)), bits(ref))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_morton(wf, orc, dev, kind):
    import torch
    rng = np.random.default_rng(kind)
    rays = random_rays(rng, 50000, lo=-0.2, hi=1.2)
    smin, ssize = [0.0, -0.1, 0.05], [1.0, 1.3, 0.8]
    keys = torch.empty(50000, dtype=torch.int32 if kind == 0 else torch.int64, device=dev)
    idx = torch.empty(50000, dtype=torch.int32, device=dev)
    wf.api.morton(T(rays, dev), smin, ssize, kind, keys, idx)
    rk, ri = orc.morton(rays, smin, ssize, kind)
    got = N(keys).view(np.uint32 if kind == 0 else np.uint64)
    assert np.array_equal(got, rk)
    assert np.array_equal(N(idx).view(np.uint32), ri)


def test_morton_device_count(wf, orc, dev):
    import torch
    rays = random_rays(np.random.default_rng(9), 1000)
    keys = torch.full((1000,), -7, dtype=torch.int32, device=dev)
    idx = torch.full((1000,), -7, dtype=torch.int32, device=dev)
    cnt = torch.tensor([613], dtype=torch.int32, device=dev)
    wf.api.morton(T(rays, dev), [0, 0, 0], [1, 1, 1], 0, keys, idx, n_dev=cnt)
    rk, ri = orc.morton(rays[:613], [0, 0, 0], [1, 1, 1], 0)
    assert np.array_equal(N(keys)[:613].view(np.uint32), rk)
    assert np.all(N(keys)[613:] == -7) and np.all(N(idx)[613:] == -7)


def test_reorder(wf, orc, dev):
    import torch
    rng = np.random.default_rng(4)
    n = 70001
    rays = random_rays(rng, n)
    perm = rng.permutation(n).astype(np.uint32)
    s2i = rng.permutation(n).astype(np.int32)
    out = torch.empty((n, 8), dtype=torch.float32, device=dev)
    os2i = torch.empty(n, dtype=torch.int32, device=dev)
    oi2s = torch.empty(n, dtype=torch.int32, device=dev)
    wf.api.reorder(T(perm.view(np.int32), dev), T(rays, dev), out, T(s2i, dev), os2i, oi2s)
    r_out, r_s2i, r_i2s = orc.reorder(perm, rays, s2i)
    assert np.array_equal(bits(N(out)), bits(r_out))
    assert np.array_equal(N(os2i), r_s2i) and np.array_equal(N(oi2s), r_i2s)


@pytest.mark.parametrize("words,maps,counted", [(12, True, False), (12, False, True), (4, True, False),
                                                (8, True, True), (16, False, False)])
def test_reorder_records(wf, orc, dev, words, maps, counted):
    # 48-byte (12-word) wide records, and the 16/32/64-byte widths, with and
    # without slot maps; `counted` reads n from device memory.
    import torch
    rng = np.random.default_rng(words * 7 + maps)
    n = 50003
    recs = rng.integers(0, 2**32, size=(n, words), dtype=np.uint32).view(np.int32)
    perm = rng.permutation(n).astype(np.uint32)
    s2i = rng.permutation(n).astype(np.int32)
    out = torch.full((n, words), -7, dtype=torch.int32, device=dev)
    os2i = torch.empty(n, dtype=torch.int32, device=dev) if maps else None
    oi2s = torch.empty(n, dtype=torch.int32, device=dev) if maps else None
    m = n - 1000 if counted else n
    n_dev = torch.tensor([m], dtype=torch.int32, device=dev) if counted else None
    wf.api.reorder_records(T(perm.view(np.int32), dev), T(recs, dev), out, T(s2i, dev) if maps else None, os2i,
                           oi2s, n=n, n_dev=n_dev)
    if counted:
        # only the first m slots are written; the rest keep their fill
        ref = recs[perm[:m]]
        got = N(out)
        assert np.array_equal(got[:m], ref) and np.all(got[m:] == -7)
        return
    r_out, r_s2i, r_i2s = orc.reorder_records(perm, recs, s2i if maps else None)
    assert np.array_equal(N(out), r_out)
    if maps:
        assert np.array_equal(N(os2i), r_s2i) and np.array_equal(N(oi2s), r_i2s)


def _hits_for(rays, rng, miss_frac=0.3):
    n = rays.shape[0]
    res = np.zeros((n, 4), np.int32)
    t = rng.uniform(0.0, 2.0, n).astype(np.float32)
    res[:, 0] = rng.integers(0, 100, n)
    res[:, 2] = t.view(np.int32)
    miss = rng.random(n) < miss_frac
    res[miss, 0] = -1
    res[miss, 1] = -1
    res[miss, 2] = np.float32(-1.0).view(np.int32)
    return res


@pytest.mark.parametrize("S,bb", [(1, 0), (2, 17), (4, 0), (7, 100)])
def test_raygen_shadow(wf, orc, dev, S, bb):
    import torch
    rng = np.random.default_rng(S)
    n = 3000
    rays = random_rays(rng, n)
    res = _hits_for(rays, rng)
    seeds = rng.integers(0, 2**32, n, dtype=np.uint32)
    bs = n - bb
    out = torch.empty((bs * S, 8), dtype=torch.float32, device=dev)
    s2i = torch.empty(bs * S, dtype=torch.int32, device=dev)
    i2s = torch.empty(bs * S, dtype=torch.int32, device=dev)
    wf.api.raygen_shadow(T(seeds.view(np.int32), dev), T(rays, dev), T(res, dev), out, s2i, i2s, (0.3, 5.0, -1.0),
                         0.7, bb, bs, S)
    r_out, r_s2i, r_i2s = orc.raygen_shadow(seeds, rays, res, (0.3, 5.0, -1.0), 0.7, bb, bs, S)
    assert np.array_equal(bits(N(out)), bits(r_out))
    assert np.array_equal(N(s2i), r_s2i) and np.array_equal(N(i2s), r_i2s)


@pytest.fixture(scope="module")
def soup(wf, orc):
    pos, nrm, idx = wf.api.generate_scene(0, 21, 20000)
    sc = wf.api.Scene(pos, idx, host_only=True)
    nodes, tris = sc.export_bvh2()
    verts = wf.api.gltf_vertices(pos, nrm)
    return pos, nrm, idx, nodes, tris, verts


def test_raygen_path(wf, orc, dev, soup):
    import torch
    pos, nrm, idx, nodes, tris, verts = soup
    rng = np.random.default_rng(11)
    n = 40000
    rays = random_rays(rng, n)
    res = orc.trace_bvh2(nodes, tris, rays)
    assert 0.3 < np.mean(res[:, 0] >= 0) < 1.0
    seeds = rng.integers(0, 2**32, n, dtype=np.uint32)
    i2p = rng.permutation(n).astype(np.int32)
    dec = rng.uniform(0.1, 1.0, (n, 4)).astype(np.float32)
    hg = orc.HostGeometry(verts, idx)
    r_seeds, r_out, r_i2p, r_dec, r_cnt = orc.raygen_path(seeds, hg, rays, i2p, res, dec, albedo=0.8)
    g = wf.api.Geometry(pos, nrm, idx, device=dev)
    d_seeds = T(seeds.view(np.int32), dev)
    out = torch.zeros((n, 8), dtype=torch.float32, device=dev)
    o_i2p = torch.zeros(n, dtype=torch.int32, device=dev)
    d_dec = T(dec, dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    wf.api.raygen_path(d_seeds, g.table, T(rays, dev), out, T(i2p, dev), o_i2p, T(res, dev), d_dec, cnt, albedo=0.8)
    c = int(N(cnt)[0])
    assert c == r_cnt
    assert np.array_equal(bits(N(out)[:c]), bits(r_out))
    assert np.array_equal(N(o_i2p)[:c], r_i2p)
    assert np.array_equal(N(d_seeds).view(np.uint32), r_seeds)
    assert np.array_equal(bits(N(d_dec)), bits(r_dec))
    assert wf.api.device_status() == 0


def test_raygen_path_device_count_and_empty(wf, orc, dev, soup):
    import torch
    pos, nrm, idx, nodes, tris, verts = soup
    g = wf.api.Geometry(pos, nrm, idx, device=dev)
    n = 5000
    rng = np.random.default_rng(2)
    rays = random_rays(rng, n)
    res = orc.trace_bvh2(nodes, tris, rays)
    seeds = rng.integers(0, 2**32, n, dtype=np.uint32)
    i2p = np.arange(n, dtype=np.int32)
    dec = np.ones((n, 4), np.float32)
    for count in (0, 1, 257, 4999):
        out = torch.zeros((n, 8), dtype=torch.float32, device=dev)
        o_i2p = torch.zeros(n, dtype=torch.int32, device=dev)
        cnt = torch.full((1,), 12345, dtype=torch.int32, device=dev)
        ndev = torch.tensor([count], dtype=torch.int32, device=dev)
        wf.api.raygen_path(T(seeds.view(np.int32), dev), g.table, T(rays, dev), out, T(i2p, dev), o_i2p, T(res, dev),
                           T(dec, dev), cnt, n_dev=ndev)
        hg = orc.HostGeometry(verts, idx)
        _, r_out, _, _, r_cnt = orc.raygen_path(seeds[:count], hg, rays[:count], i2p[:count], res[:count],
                                                dec, albedo=0.8)
        assert int(N(cnt)[0]) == r_cnt
        assert np.array_equal(bits(N(out)[:r_cnt]), bits(r_out))


def test_reconstruct_smooth(wf, orc, dev, soup):
    pos, nrm, idx, nodes, tris, verts = soup
    rng = np.random.default_rng(5)
    n = 30000
    rays = random_rays(rng, n)
    res = orc.trace_bvh2(nodes, tris, rays)
    i2p = rng.permutation(n).astype(np.int32)
    px = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    dec = rng.uniform(0.1, 1.0, (n, 4)).astype(np.float32)
    g = wf.api.Geometry(pos, nrm, idx, device=dev)
    d_px = T(px, dev)
    for spp in (1, 3):
        d_px = T(px, dev)
        wf.api.reconstruct_smooth(T(rays, dev), T(res, dev), T(i2p, dev), d_px, T(dec, dev), g.table, (2, 3, -1),
                                  (0.2, 0.4, 0.9), spp)
        ref = orc.reconstruct_smooth(rays, res, i2p, px, dec, orc.HostGeometry(verts, idx), (2, 3, -1),
                                     (0.2, 0.4, 0.9), spp)
        assert np.array_equal(bits(N(d_px)), bits(ref))


@pytest.mark.parametrize("replace", [False, True])
def test_reconstruct_shadow(wf, orc, dev, replace):
    rng = np.random.default_rng(8)
    n, S, bb = 4000, 3, 250
    bs = n - bb
    res = np.zeros((bs * S, 4), np.int32)
    res[:, 0] = np.where(rng.random(bs * S) < 0.5, -1, 7)
    i2p = rng.permutation(n).astype(np.int32)
    i2s = rng.permutation(bs * S).astype(np.int32)
    inp = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    outp = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    d_out = T(outp, dev)
    wf.api.reconstruct_shadow(T(res, dev), T(i2p, dev), T(i2s, dev), T(inp, dev), d_out, bb, bs, S, replace=replace)
    ref = orc.reconstruct_shadow(res, i2p, i2s, inp, outp, bb, bs, S, replace=replace)
    assert np.array_equal(bits(N(d_out)), bits(ref))


def test_count_hits(wf, orc, dev):
    import torch
    rng = np.random.default_rng(3)
    for n in (1, 255, 256, 100003):
        res = np.zeros((n, 4), np.int32)
        res[:, 0] = np.where(rng.random(n) < 0.4, -1, rng.integers(0, 9, n))
        c = torch.zeros(1, dtype=torch.int32, device=dev)
        wf.api.count_hits(T(res, dev), c)
        assert int(N(c)[0]) == orc.count_hits(res)


@pytest.mark.parametrize("frame", [1, 2, 7])
def test_interpolate_colors(wf, orc, dev, frame):
    rng = np.random.default_rng(frame)
    n = 20000
    fp = rng.uniform(0, 3, (n, 4)).astype(np.float32)
    pp = rng.uniform(0, 3, (n, 4)).astype(np.float32)
    d_fp, d_pp = T(fp, dev), T(pp, dev)
    wf.api.interpolate_colors(d_fp, d_pp, frame, 0.6, 2.0)
    r_fp, r_pp = orc.interpolate_colors(fp, pp, frame, 0.6, 2.0)
    assert np.array_equal(bits(N(d_fp)), bits(r_fp)) and np.array_equal(bits(N(d_pp)), bits(r_pp))


def test_fill(wf, dev):
    import torch
    t = torch.zeros(1000003, dtype=torch.float32, device=dev)
    wf.api.fill_u32(t, int(np.float32(1.0).view(np.uint32)), t.numel())
    assert bool((t == 1.0).all())


def test_reorder_full_size_properties(wf, dev):
    """The reorder gather at the city's 8,294,400 rays: out[i] = in[idx[i]],
    the slot map follows the rays and index_to_slot inverts it."""
    import torch
    n = 3840 * 2160
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    rays = torch.rand((n, 8), generator=g, device=dev)
    idx = torch.randperm(n, generator=g, device=dev).to(torch.int32)
    s2i = torch.randperm(n, generator=g, device=dev).to(torch.int32)
    out = torch.empty_like(rays)
    os2i = torch.empty(n, dtype=torch.int32, device=dev)
    oi2s = torch.full((n,), -1, dtype=torch.int32, device=dev)
    wf.api.reorder(idx, rays, out, s2i, os2i, oi2s)
    torch.cuda.synchronize()
    assert wf.api.device_status() == 0
    li = idx.to(torch.int64)
    assert torch.equal(out, rays[li])
    assert torch.equal(os2i, s2i[li])
    slots = torch.arange(n, dtype=torch.int32, device=dev)
    assert torch.equal(oi2s[os2i.to(torch.int64)], slots)


@pytest.mark.parametrize("words,counted", [(12, False), (4, True), (16, False)])
def test_reorder_records_beyond_l2(wf, dev, words, counted):
    """Record gathers past the size from which the kernels stream the
    records with an L2 evict-first policy (4,194,304 rays): 48-, 16- and
    64-byte records by a random permutation, with slot maps; `counted`
    reads the ray count from device memory (the policy follows the host
    capacity)."""
    import torch
    n = (1 << 22) + 4099
    g = torch.Generator(device=dev)
    g.manual_seed(words)
    recs = torch.randint(-2**31, 2**31 - 1, (n, words), generator=g, device=dev, dtype=torch.int32)
    idx = torch.randperm(n, generator=g, device=dev).to(torch.int32)
    s2i = torch.randperm(n, generator=g, device=dev).to(torch.int32)
    out = torch.full((n, words), -7, dtype=torch.int32, device=dev)
    os2i = torch.full((n,), -7, dtype=torch.int32, device=dev)
    oi2s = torch.full((n,), -1, dtype=torch.int32, device=dev)
    m = n - 1000 if counted else n
    n_dev = torch.tensor([m], dtype=torch.int32, device=dev) if counted else None
    wf.api.reorder_records(idx, recs, out, s2i, os2i, oi2s, n=n, n_dev=n_dev)
    torch.cuda.synchronize()
    assert wf.api.device_status() == 0
    li = idx[:m].to(torch.int64)
    assert torch.equal(out[:m], recs[li]) and bool((out[m:] == -7).all())
    assert torch.equal(os2i[:m], s2i[li]) and bool((os2i[m:] == -7).all())
    written = os2i[:m].to(torch.int64)
    assert torch.equal(oi2s[written], torch.arange(m, dtype=torch.int32, device=dev))


def test_interpolate_colors_fp64_matches_oracle(wf, orc, dev):
    """The FP64 running mean over five frames, bit-exact against the
    oracle's double evaluation (pixels, tone-mapped frame and the double
    accumulator itself)."""
    import torch
    rng = np.random.default_rng(31)
    n = 30001
    pp = np.zeros((n, 4), np.float32)
    acc = np.zeros((n, 4), np.float64)
    d_pp = T(pp, dev)
    d_acc = torch.zeros((n, 4), dtype=torch.float64, device=dev)
    for frame in range(1, 6):
        fp = rng.uniform(0, 3, (n, 4)).astype(np.float32)
        fp[:5] = 0.0
        d_fp = T(fp, dev)
        wf.api.interpolate_colors_fp64(d_fp, d_pp, d_acc, frame, 0.6, 2.0)
        r_fp, pp, acc = orc.interpolate_colors_fp64(fp, pp, acc, frame, 0.6, 2.0)
        got_fp = N(d_fp)
        assert np.array_equal(np.isnan(got_fp), np.isnan(r_fp))
        assert np.array_equal(bits(np.nan_to_num(got_fp)), bits(np.nan_to_num(r_fp)))
        assert np.array_equal(bits(N(d_pp)), bits(pp))
        assert np.array_equal(N(d_acc).view(np.uint64), acc.view(np.uint64))


def test_fp64_accumulation_tracks_the_exact_mean(wf, dev):
    """Over 512 frames of random colours, the FP64 running mean stays within
    one float rounding of the exact mean of the frames, while the float
    running mean of interpolateColors.comp drifts much further."""
    import torch
    rng = np.random.default_rng(32)
    n, frames = 4096, 512
    d_pp32 = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    d_pp64 = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    d_acc = torch.zeros((n, 4), dtype=torch.float64, device=dev)
    total = np.zeros((n, 3), np.float64)
    for f in range(1, frames + 1):
        fp = rng.uniform(0, 1, (n, 4)).astype(np.float32)
        total += fp[:, :3]
        wf.api.interpolate_colors(T(fp, dev), d_pp32, f, 0.6, 2.0)
        wf.api.interpolate_colors_fp64(T(fp, dev), d_pp64, d_acc, f, 0.6, 2.0)
    exact = total / frames
    err32 = np.abs(N(d_pp32)[:, :3].astype(np.float64) - exact).max()
    err64 = np.abs(N(d_pp64)[:, :3].astype(np.float64) - exact).max()
    assert err64 <= 2.0**-24  # the mean is below 1: half an ulp of the float result
    assert err32 > 16 * err64
