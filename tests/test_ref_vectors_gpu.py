"""The CUDA stage kernels, through the C ABI, against outputs of the
reference's own shader and host sources compiled for the CPU
(tests/golden/ref_vectors.npz; see tests/refvectors.py for the bars): the
same check the oracle passes on the CPU, made on the device without the
oracle in between."""
import numpy as np
import pytest

import refvectors as rv

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def N(t):
    return t.cpu().numpy()


def gpu_impl(wf, dev):
    import torch
    api = wf.api

    def init_seeds(n, frame):
        s = torch.empty(n, dtype=torch.int32, device=dev)
        api.init_seeds(s, frame)
        return N(s).view(np.uint32)

    def raygen_primary(m, i2p, origin, sample, w, h, max_dist):
        rays = torch.empty((w * h, 8), dtype=torch.float32, device=dev)
        api.raygen_primary(m, T(i2p, dev), rays, origin, sample, w, h, max_dist)
        return N(rays)

    def morton(rays, smin, ssize):
        n = rays.shape[0]
        keys = torch.empty(n, dtype=torch.int32, device=dev)
        idx = torch.empty(n, dtype=torch.int32, device=dev)
        api.morton(T(rays, dev), smin, ssize, 0, keys, idx)
        return N(keys).view(np.uint32), N(idx).view(np.uint32)

    def reorder(idx, rays, s2i):
        n = idx.shape[0]
        out = torch.empty((n, 8), dtype=torch.float32, device=dev)
        os2i = torch.empty(n, dtype=torch.int32, device=dev)
        oi2s = torch.full((n,), -1, dtype=torch.int32, device=dev)
        api.reorder(T(idx.view(np.int32), dev), T(rays, dev), out, T(s2i, dev), os2i, oi2s)
        return N(out), N(os2i), N(oi2s)

    def raygen_shadow(seeds, rays, res, light, radius, bb, bs, S):
        out = torch.empty((bs * S, 8), dtype=torch.float32, device=dev)
        s2i = torch.empty(bs * S, dtype=torch.int32, device=dev)
        i2s = torch.empty(bs * S, dtype=torch.int32, device=dev)
        api.raygen_shadow(T(seeds.view(np.int32), dev), T(rays, dev), T(res, dev), out, s2i, i2s, light, radius, bb,
                          bs, S)
        return N(out), N(s2i), N(i2s)

    def raygen_path(pos, nrm, idx, seeds, rays, i2p, res, dec):
        n = rays.shape[0]
        g = api.Geometry(pos, nrm, idx, device=dev)
        d_seeds, d_dec = T(seeds.view(np.int32), dev), T(dec, dev)
        out = torch.zeros((n, 8), dtype=torch.float32, device=dev)
        o_i2p = torch.zeros(n, dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int32, device=dev)
        api.raygen_path(d_seeds, g.table, T(rays, dev), out, T(i2p, dev), o_i2p, T(res, dev), d_dec, cnt, albedo=0.8)
        c = int(N(cnt)[0])
        return N(d_seeds).view(np.uint32), N(out)[:c], N(o_i2p)[:c], N(d_dec), c

    def reconstruct_smooth(pos, nrm, idx, rays, res, i2p, px, dec, light, bg, spp):
        g = api.Geometry(pos, nrm, idx, device=dev)
        d_px = T(px, dev)
        api.reconstruct_smooth(T(rays, dev), T(res, dev), T(i2p, dev), d_px, T(dec, dev), g.table, light, bg, spp)
        return N(d_px)

    def reconstruct_shadow(res, i2p, i2s, inp, prev, bb, bs, S):
        d_out = T(prev, dev)
        api.reconstruct_shadow(T(res, dev), T(i2p, dev), T(i2s, dev), T(inp, dev), d_out, bb, bs, S)
        return N(d_out)

    def count_hits(res):
        c = torch.zeros(1, dtype=torch.int32, device=dev)
        api.count_hits(T(res, dev), c)
        return int(N(c)[0])

    def interpolate_colors(fp, pp, frame, key, white):
        d_fp, d_pp = T(fp, dev), T(pp, dev)
        api.interpolate_colors(d_fp, d_pp, frame, key, white)
        return N(d_fp), N(d_pp)

    return {
        "init_seeds": init_seeds,
        "pixel_table": api.pixel_table,
        "camera": api.camera_screen_to_world,
        "raygen_primary": raygen_primary,
        "morton_aila32": morton,
        "reorder": reorder,
        "raygen_shadow": raygen_shadow,
        "raygen_path": raygen_path,
        "reconstruct_smooth": reconstruct_smooth,
        "reconstruct_shadow": reconstruct_shadow,
        "count_hits": count_hits,
        "interpolate_colors": interpolate_colors,
    }


def test_kernels_match_reference_vectors(wf, dev):
    assert rv.check_all(gpu_impl(wf, dev)) == rv.ALL_STAGES
    assert wf.api.device_status() == 0
