"""Radix sort through the C ABI: bit-exact against a stable sort
(the oracle's, i.e. the order any stable LSD sort produces), across sizes
around tile boundaries, 32- and 64-bit keys, odd pass counts, partial key
widths, device-side counts and clustered Morton keys."""
import numpy as np
import pytest

from conftest import random_rays

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def N(t):
    return t.cpu().numpy()


def stable_ref(keys, key_bits):
    mask = (1 << key_bits) - 1 if key_bits < 64 else (1 << 64) - 1
    k = keys.astype(np.uint64) & np.uint64(mask)
    order = np.argsort(k, kind="stable")
    return keys[order], order.astype(np.uint32)


def run_sort(wf, dev, keys, key_bits, n_dev=None):
    import torch
    is64 = key_bits > 32
    dk = T(keys.view(np.int64 if is64 else np.int32), dev)
    dv = torch.arange(keys.shape[0], dtype=torch.int32, device=dev)
    wf.api.sort_pairs(dk, dv, key_bits, n_dev=None if n_dev is None else torch.tensor([n_dev], dtype=torch.int32,
                                                                                       device=dev))
    got_k = N(dk).view(np.uint64 if is64 else np.uint32)
    got_v = N(dv).view(np.uint32)
    return got_k, got_v


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 255, 4095, 4096, 4097, 65536, 123457, (1 << 20) + 3])
def test_sort_u32_sizes(wf, dev, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2**32, n, dtype=np.uint32)
    k, v = run_sort(wf, dev, keys, 32)
    rk, rv = stable_ref(keys, 32)
    assert np.array_equal(k, rk) and np.array_equal(v, rv)
    assert wf.api.device_status() == 0


def test_sort_matches_oracle_with_duplicates(wf, orc, dev):
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 64, 100000, dtype=np.uint32)  # heavy duplicates: stability matters
    k, v = run_sort(wf, dev, keys, 32)
    ok, ov = orc.sort_pairs(keys, np.arange(100000, dtype=np.uint32), 32)
    assert np.array_equal(k, ok) and np.array_equal(v, ov)


@pytest.mark.parametrize("key_bits", [63, 64, 48, 40, 33])
def test_sort_u64(wf, dev, key_bits):
    rng = np.random.default_rng(key_bits)
    n = 300001
    keys = rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    keys[::7] = keys[3]  # duplicates
    k, v = run_sort(wf, dev, keys, key_bits)
    rk, rv = stable_ref(keys, key_bits)
    assert np.array_equal(v, rv)
    assert np.array_equal(k, rk)


@pytest.mark.parametrize("key_bits", [8, 12, 24])
def test_sort_partial_key_bits(wf, dev, key_bits):
    rng = np.random.default_rng(key_bits)
    keys = rng.integers(0, 2**32, 50000, dtype=np.uint32)
    k, v = run_sort(wf, dev, keys, key_bits)
    _, rv = stable_ref(keys, key_bits)
    assert np.array_equal(v, rv)


def test_sort_device_count(wf, dev):
    rng = np.random.default_rng(7)
    n, c = 200000, 123456
    for bits in (32, 40):
        keys = rng.integers(0, 2**32 if bits == 32 else 2**40, n, dtype=np.uint64)
        keys = keys.astype(np.uint32) if bits == 32 else keys
        k, v = run_sort(wf, dev, keys, bits, n_dev=c)
        rk, rv = stable_ref(keys[:c], bits)
        assert np.array_equal(v[:c], rv) and np.array_equal(k[:c], rk)
        # elements past the device count are left untouched
        assert np.array_equal(k[c:], keys[c:]) and np.array_equal(v[c:], np.arange(c, n, dtype=np.uint32))


@pytest.mark.parametrize("kind,bits", [(0, 32), (1, 48), (2, 63)])
def test_sort_clustered_morton_keys(wf, orc, dev, kind, bits):
    """Morton keys of clustered 6-D Gaussian ray origins/directions."""
    import torch
    rng = np.random.default_rng(kind + 10)
    n = 1 << 18
    centers = rng.uniform(0.2, 0.8, (16, 3))
    o = centers[rng.integers(0, 16, n)] + rng.normal(0, 0.02, (n, 3))
    d = rng.normal(0, 1, (n, 3)) * 0.1 + np.array([0.3, -1.0, 0.2])
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = o
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    keys = torch.empty(n, dtype=torch.int32 if kind == 0 else torch.int64, device=dev)
    idx = torch.empty(n, dtype=torch.int32, device=dev)
    wf.api.morton(T(rays, dev), [0, 0, 0], [1, 1, 1], kind, keys, idx)
    wf.api.sort_pairs(keys, idx, bits)
    rk, ri = orc.morton(rays, [0, 0, 0], [1, 1, 1], kind)
    sk, si = orc.sort_pairs(rk, ri, bits)
    assert np.array_equal(N(idx).view(np.uint32), si)
    assert np.array_equal(N(keys).view(sk.dtype), sk)


def test_sort_scratch_too_small(wf, dev):
    import torch
    k = torch.zeros(5000, dtype=torch.int32, device=dev)
    v = torch.zeros(5000, dtype=torch.int32, device=dev)
    small = torch.empty(64, dtype=torch.uint8, device=dev)
    with pytest.raises(wf.WfptError):
        wf.api.sort_pairs(k, v, 32, scratch=small)


@pytest.mark.parametrize("digit_bits", [8, 4])
@pytest.mark.parametrize("tiles", [1, 2, 3])
@pytest.mark.parametrize("n,key_bits", [(1, 32), (2047, 32), (2049, 32), (4095, 32), (4097, 32), (8191, 32),
                                        (8193, 32), (10239, 32), (10241, 32), (123457, 32), (9000, 12),
                                        (70001, 33), (1535, 63), (1537, 64), (3073, 63), (7167, 63), (7169, 63),
                                        (14337, 64), (7679, 63), (7681, 63), (15361, 64), (300001, 48), (65537, 62), (2073600, 63)])
def test_sort_tile_variants(wf, dev, tiles, n, key_bits, digit_bits):
    """Every tile size and both digit widths give the stable order, at sizes
    around the tile boundaries, odd and even pass counts, key widths that
    are not multiples of the digit width, and the frame's wavefront size."""
    rng = np.random.default_rng(n + key_bits)
    if key_bits > 32:
        keys = rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    else:
        keys = rng.integers(0, 2**32, n, dtype=np.uint32)
    keys[::5] = keys[len(keys) // 2]  # duplicates: stability matters
    if key_bits < 32:
        keys &= np.uint32((1 << key_bits) - 1) | np.uint32(0xF0000000)  # high bits outside key_bits are ignored
    old = wf.api.tune_get("sort.tiles"), wf.api.tune_get("sort.digit_bits")
    try:
        wf.api.tune_set("sort.tiles", tiles)
        wf.api.tune_set("sort.digit_bits", digit_bits)
        k, v = run_sort(wf, dev, keys, key_bits)
    finally:
        wf.api.tune_set("sort.tiles", old[0])
        wf.api.tune_set("sort.digit_bits", old[1])
    rk, rv = stable_ref(keys, key_bits)
    assert np.array_equal(v, rv) and np.array_equal(k, rk)
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("key_bits,n", [(63, 2073600), (63, 5000000), (32, 3000001)])
def test_sort_captured_graph_replays(wf, dev, key_bits, n):
    """The sort captured into a CUDA graph (its passes are launched as
    programmatic dependents of the kernel before them, which capture turns
    into programmatic edges) and replayed on new keys copied into the
    captured buffers: every replay gives the stable order.  Sizes of one
    wave of tiles and of several."""
    import torch
    is64 = key_bits > 32
    kt = torch.int64 if is64 else torch.int32
    keys = torch.zeros(n, dtype=kt, device=dev)
    vals = torch.zeros(n, dtype=torch.int32, device=dev)
    scratch = torch.empty(wf.api.sort_scratch_bytes(n, key_bits), dtype=torch.uint8, device=dev)
    iota = torch.arange(n, dtype=torch.int32, device=dev)
    wf.api.sort_pairs(keys, vals, key_bits, scratch=scratch)  # prepares the kernels outside the capture
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        wf.api.sort_pairs(keys, vals, key_bits, scratch=scratch, stream=s)
    rng = np.random.default_rng(key_bits + n)
    for rep in range(3):
        if is64:
            src = rng.integers(0, 2**63, n, dtype=np.uint64)
        else:
            src = rng.integers(0, 2**32, n, dtype=np.uint32)
        src[:: 4 + rep] = src[7]  # duplicates: stability matters
        keys.copy_(T(src.view(np.int64 if is64 else np.int32), dev))
        vals.copy_(iota)
        g.replay()
        torch.cuda.synchronize()
        rk, rv = stable_ref(src, key_bits)
        assert np.array_equal(N(vals).view(np.uint32), rv), rep
        assert np.array_equal(N(keys).view(np.uint64 if is64 else np.uint32), rk), rep
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("key_bits", [63, 32])
def test_sort_unaligned_buffers(wf, dev, key_bits):
    """Caller buffers one element past a 16-byte boundary: the passes that
    read them skip the L2 bulk prefetch of later tiles (it needs 16-byte
    aligned arrays), the passes that read the aligned scratch copy keep it,
    and the order is the stable one either way.  4M pairs: several waves of
    tiles, so tiles are prefetched ahead in the aligned passes."""
    import torch
    n = 1 << 22
    rng = np.random.default_rng(key_bits + 100)
    if key_bits > 32:
        keys = rng.integers(0, 2**63, n, dtype=np.uint64)
    else:
        keys = rng.integers(0, 2**32, n, dtype=np.uint32)
    keys[::3] = keys[11]
    is64 = key_bits > 32
    kbuf = torch.zeros(n + 1, dtype=torch.int64 if is64 else torch.int32, device=dev)
    vbuf = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    dk, dv = kbuf[1:], vbuf[1:]
    assert dk.data_ptr() % 16 != 0 and dv.data_ptr() % 16 != 0
    dk.copy_(T(keys.view(np.int64 if is64 else np.int32), dev))
    dv.copy_(torch.arange(n, dtype=torch.int32, device=dev))
    wf.api.sort_pairs(dk, dv, key_bits)
    rk, rv = stable_ref(keys, key_bits)
    assert np.array_equal(N(dv).view(np.uint32), rv)
    assert np.array_equal(N(dk).view(np.uint64 if is64 else np.uint32), rk)
    assert int(kbuf[0]) == 0 and int(vbuf[0]) == 0
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("key_bits,n,counted", [(44, (1 << 24) + 4097, False), (64, (1 << 24) + 1, False),
                                                (63, (1 << 24) + 77, True), (32, (1 << 24) + 3, False)])
def test_sort_large_histogram_bit_exact(wf, dev, key_bits, n, counted):
    """Sorts of 2^24 pairs and more with five passes or more build their
    digit histograms in lane-private 16-bit counter columns: the stable
    order, bit for bit, for a key width that is not a multiple of 8 (44
    bits: 6 passes, the top one on 4 bits), full 64-bit keys, a count read
    from device memory (the histogram's grid follows the host capacity, the
    count the device value), and 32-bit keys (four passes: the plain
    histogram kernel) at the same size."""
    rng = np.random.default_rng(n + key_bits)
    if key_bits > 32:
        keys = rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    else:
        keys = rng.integers(0, 2**32, n, dtype=np.uint32)
    keys[::3] = keys[7]  # a third of the keys equal: one digit bin holds them in every pass
    m = n - 5000 if counted else n
    k, v = run_sort(wf, dev, keys, key_bits, n_dev=m if counted else None)
    rk, rv = stable_ref(keys[:m], key_bits)
    assert np.array_equal(v[:m], rv) and np.array_equal(k[:m], rk)
    if counted:
        assert np.array_equal(k[m:], keys[m:]) and np.array_equal(v[m:], np.arange(m, n, dtype=np.uint32))
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("key_bits", [63, 32])
def test_sort_full_size_properties(wf, dev, key_bits):
    """2^26 pairs, the microbenchmark's largest size (beyond what a CPU
    stable sort checks quickly): keys non-decreasing, values a permutation,
    each output key the input key its value points at, and equal keys in
    input order (values are the input positions, so they increase within
    a run of equal keys).  Keys are drawn from a quarter of n values, so
    most keys repeat."""
    import torch
    n = 1 << 26
    g = torch.Generator(device=dev)
    g.manual_seed(key_bits)
    hi = (1 << 62) if key_bits > 32 else (1 << 31)
    pool = torch.randint(0, hi, (n // 4,), generator=g, device=dev, dtype=torch.int64)
    src = pool[torch.randint(0, n // 4, (n,), generator=g, device=dev)]
    if key_bits <= 32:
        src = src.to(torch.int32)
    keys = src.clone()
    vals = torch.arange(n, dtype=torch.int32, device=dev)
    wf.api.sort_pairs(keys, vals, key_bits)
    torch.cuda.synchronize()
    assert wf.api.device_status() == 0
    k = keys.to(torch.int64)
    if key_bits <= 32:
        k = k & 0xFFFFFFFF  # compare as unsigned 32-bit
    assert bool((k[1:] >= k[:-1]).all())
    v = vals.to(torch.int64)
    assert bool((torch.bincount(v, minlength=n) == 1).all())
    assert bool((keys == src[v]).all())
    same = k[1:] == k[:-1]
    assert bool((v[1:][same] > v[:-1][same]).all())
    assert int(same.sum()) > n // 2
