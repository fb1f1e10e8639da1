"""The stage chain of one shadow pass and one path bounce driven stage by
stage through the C ABI, each stage compared with the oracle on the same
inputs: primary rays -> closest hit -> shading -> shadow rays -> any hit ->
visibility -> path rays -> closest hit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def N(t):
    return t.cpu().numpy()


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def diff_report(name, got, ref):
    g, r = bits(got).reshape(len(got), -1), bits(ref).reshape(len(ref), -1)
    bad = np.nonzero((g != r).any(axis=1))[0]
    if bad.size == 0:
        return None
    i = bad[0]
    return f"{name}: {bad.size} of {len(g)} rows differ; first row {i}: got {got[i]} ref {ref[i]}"


def test_shadow_and_path_chain(wf, orc, dev):
    import torch
    api = wf.api
    pos, nrm, idx = api.generate_scene(0, 1, 65536)
    sc = api.Scene(pos, idx)
    nodes, tris = sc.export_bvh2()
    geom = api.Geometry(pos, nrm, idx, device=dev)
    hg = orc.HostGeometry(api.gltf_vertices(pos, nrm), idx)
    w, h, S = 96, 64, 2
    n = w * h
    light, bg = (0.5, 1.6, 0.5), (0.53, 0.81, 0.98)
    eye = (0.5, 0.5, 2.2)
    m = api.camera_screen_to_world(eye, (0, 0, 0), 45.0, w / h, 0.001, 10.0)
    i2p, _ = api.pixel_table(w, h)
    problems = []

    rays = torch.empty((n, 8), dtype=torch.float32, device=dev)
    api.raygen_primary(m, T(i2p, dev), rays, eye, 0, w, h, 10.0)
    o_rays = orc.raygen_primary(m, i2p, eye, 0, w, h, 10.0)
    problems.append(diff_report("primary rays", N(rays), o_rays))

    hits = torch.empty((n, 4), dtype=torch.int32, device=dev)
    api.trace(sc, wf.BVH2_FP32, rays, hits)
    o_hits = orc.trace_bvh2(nodes, tris, o_rays)
    problems.append(diff_report("primary hits", N(hits), o_hits))

    seeds = torch.empty(n, dtype=torch.int32, device=dev)
    api.init_seeds(seeds, 1)
    o_seeds = orc.init_seeds(n, 1)
    dec = torch.ones((n, 4), dtype=torch.float32, device=dev)
    aux = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    api.reconstruct_smooth(rays, hits, T(i2p, dev), aux, dec, geom.table, light, bg, 1)
    o_aux = orc.reconstruct_smooth(o_rays, o_hits, i2p, np.zeros((n, 4), np.float32), np.ones((n, 4), np.float32), hg,
                                   light, bg, 1)
    problems.append(diff_report("primary shading", N(aux), o_aux))

    srays = torch.empty((n * S, 8), dtype=torch.float32, device=dev)
    s2i = torch.empty(n * S, dtype=torch.int32, device=dev)
    i2s = torch.empty(n * S, dtype=torch.int32, device=dev)
    api.raygen_shadow(seeds, rays, hits, srays, s2i, i2s, light, 0.1, 0, n, S)
    o_srays, o_s2i, o_i2s = orc.raygen_shadow(o_seeds, o_rays, o_hits, light, 0.1, 0, n, S)
    problems.append(diff_report("shadow rays", N(srays), o_srays))

    shits = torch.empty((n * S, 4), dtype=torch.int32, device=dev)
    api.trace(sc, wf.BVH2_FP32, srays, shits, closest_hit=False)
    o_shits = orc.trace_bvh2(nodes, tris, o_srays, closest=False)
    problems.append(diff_report("shadow hits", N(shits), o_shits))

    fp = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    api.reconstruct_shadow(shits, T(i2p, dev), i2s, aux, fp, 0, n, S)
    o_fp = orc.reconstruct_shadow(o_shits, i2p, o_i2s, o_aux, np.zeros((n, 4), np.float32), 0, n, S)
    problems.append(diff_report("visibility", N(fp), o_fp))

    out = torch.zeros((n, 8), dtype=torch.float32, device=dev)
    o_i2p_t = torch.zeros(n, dtype=torch.int32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    api.raygen_path(seeds, geom.table, rays, out, T(i2p, dev), o_i2p_t, hits, dec, cnt)
    o_seeds2, o_out, o_pi2p, o_dec, o_cnt = orc.raygen_path(o_seeds, hg, o_rays, i2p, o_hits,
                                                            np.ones((n, 4), np.float32))
    c = int(N(cnt)[0])
    problems.append(None if c == o_cnt else f"path count {c} vs {o_cnt}")
    problems.append(diff_report("path rays", N(out)[:c], o_out))
    phits = torch.empty((c, 4), dtype=torch.int32, device=dev)
    api.trace(sc, wf.BVH2_FP32, out[:c].contiguous(), phits)
    problems.append(diff_report("path hits", N(phits), orc.trace_bvh2(nodes, tris, o_out)))
    problems = [p for p in problems if p]
    assert not problems, "\n".join(problems)
