"""Test infrastructure: ctypes binding of the CPU oracle (liboracle.so).

Only the tests, the smoke check and the bench's CPU-baseline leg use this
module.  It restates the reference shaders on the CPU (see oracle.cpp); the
product path never calls it.  Arrays are numpy: rays float32 [n, 8], hits
int32 [n, 4] (t as float bits), pixels float32 [n, 4].
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None
_P = C.c_void_p


class FrameCfg(C.Structure):
    _fields_ = [("ray_type", C.c_int), ("spp", C.c_int), ("S", C.c_int), ("depth", C.c_int),
                ("radius", C.c_float), ("key", C.c_float), ("white", C.c_float), ("albedo", C.c_float),
                ("sort_shadow", C.c_int), ("reorder_shadow", C.c_int), ("sort_path", C.c_int),
                ("reorder_path", C.c_int), ("morton_kind", C.c_int), ("frame_index", C.c_int),
                ("path_sort_skip", C.c_int), ("accumulate_fp64", C.c_int), ("pixel_stride", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("primary", C.c_uint64), ("shadow", C.c_uint64), ("path", C.c_uint64),
                ("path_per_bounce", C.c_uint32 * 8), ("hits_per_pass", C.c_uint32 * 9)]


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = C.CDLL(str(path))
        lib.orc_count_hits.restype = C.c_uint32
        lib.orc_raygen_path.restype = C.c_uint32
        lib.orc_fp64_scene_create.restype = C.c_void_p
        lib.orc_num_threads.restype = C.c_int
        _lib = lib
    return _lib


def _f(v, n):
    a = np.ascontiguousarray(np.asarray(v, np.float32).ravel())
    assert a.size == n
    return a


_KEEP: list = []


def ptr(a: np.ndarray):
    """Pointer to a numpy array; the array is kept alive until the next
    oracle call returns (temporaries passed inline would otherwise be freed
    before the C function runs)."""
    if a is None:
        return None
    _KEEP.append(a)
    return C.c_void_p(a.ctypes.data)


def _call(fn, *args):
    try:
        return fn(*args)
    finally:
        _KEEP.clear()


def num_threads() -> int:
    return _call(load().orc_num_threads, )


def init_seeds(n, frame_index):
    s = np.empty(n, np.uint32)
    _call(load().orc_init_seeds, ptr(s), C.c_uint32(n), C.c_int(frame_index))
    return s


def pixel_table(w, h):
    a = np.empty(w * h, np.int32)
    b = np.empty(w * h, np.int32)
    _call(load().orc_pixel_table, C.c_int(w), C.c_int(h), ptr(a), ptr(b))
    return a, b


def camera_screen_to_world(pos, rot, fov, aspect, zn, zf):
    out = np.empty(16, np.float32)
    p, r = _f(pos, 3), _f(rot, 3)
    _call(load().orc_camera_screen_to_world, ptr(p), ptr(r), C.c_float(fov), C.c_float(aspect), C.c_float(zn),
                                      C.c_float(zf), ptr(out))
    return out


def raygen_primary(m, i2p, origin, sample_index, w, h, max_dist):
    rays = np.empty((w * h, 8), np.float32)
    m, o = _f(m, 16), _f(origin, 3)
    i2p = np.ascontiguousarray(i2p, np.int32)
    _call(load().orc_raygen_primary, ptr(m), ptr(i2p), ptr(rays), ptr(o), C.c_int(sample_index), C.c_int(w), C.c_int(h),
                              C.c_float(max_dist))
    return rays


def morton(rays, smin, ssize, kind):
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    keys = np.empty(n, np.uint32 if kind == 0 else np.uint64)
    idx = np.empty(n, np.uint32)
    a, b = _f(smin, 3), _f(ssize, 3)
    _call(load().orc_morton, ptr(rays), C.c_uint32(n), ptr(a), ptr(b), C.c_int(kind), ptr(keys), ptr(idx))
    return keys, idx


def sort_pairs(keys, vals, key_bits):
    keys = np.ascontiguousarray(keys).copy()
    vals = np.ascontiguousarray(vals, np.uint32).copy()
    _call(load().orc_sort_pairs, ptr(keys), ptr(vals), C.c_uint32(keys.shape[0]), C.c_int(key_bits))
    return keys, vals


def sort_pairs_mt(keys, vals, key_bits):
    """The same order as sort_pairs, by the multi-threaded LSD radix sort."""
    keys = np.ascontiguousarray(keys).copy()
    vals = np.ascontiguousarray(vals, np.uint32).copy()
    _call(load().orc_sort_pairs_mt, ptr(keys), ptr(vals), C.c_uint32(keys.shape[0]), C.c_int(key_bits))
    return keys, vals


def bvh2_build(positions, indices):
    """The oracle's own binned-SAH BVH2 (traversal format of trace_bvh2):
    (nodes uint8 [m, 64], triangle records uint8 [t, 48])."""
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32)
    nt = idx.size // 3
    nodes = np.zeros((2 * max(nt, 1), 64), np.uint8)
    tris = np.zeros((nt, 48), np.uint8)
    load().orc_bvh2_build.restype = C.c_uint32
    m = _call(load().orc_bvh2_build, ptr(pos), ptr(idx), C.c_uint32(nt), ptr(nodes), ptr(tris))
    return nodes[:m].copy(), tris


def generate_scene(kind, seed, num_triangles=0):
    """The benchmark workloads' seeded scenes (positions, normals, indices),
    from the generator the product uses, without loading the product."""
    nv, nt = C.c_uint32(0), C.c_uint32(0)
    lib = load()
    if not lib.orc_generate_scene(C.c_int(kind), C.c_uint64(seed), C.c_uint32(num_triangles), None, None,
                                  C.byref(nv), None, C.byref(nt)):
        raise ValueError("unknown scene kind")
    pos = np.empty((nv.value, 3), np.float32)
    nrm = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.uint32)
    _call(lib.orc_generate_scene, C.c_int(kind), C.c_uint64(seed), C.c_uint32(num_triangles), ptr(pos), ptr(nrm),
          C.byref(nv), ptr(idx), C.byref(nt))
    return pos, nrm, idx


def gltf_vertices(positions, normals):
    """96-byte vkglTF::Vertex records (pos.xyz, normal.xyz, then zeros)."""
    v = np.zeros((positions.shape[0], 24), np.float32)
    v[:, 0:3] = positions
    v[:, 3:6] = normals
    return v


def reorder(idx, in_rays, in_s2i, index_space=None):
    n = idx.shape[0]
    out = np.empty((n, 8), np.float32)
    s2i = np.empty(n, np.int32)
    i2s = np.full(index_space or n, -1, np.int32)
    _call(load().orc_reorder, ptr(np.ascontiguousarray(idx, np.uint32)), ptr(np.ascontiguousarray(in_rays, np.float32)),
                       ptr(out), ptr(np.ascontiguousarray(in_s2i, np.int32)), ptr(s2i), ptr(i2s), C.c_uint32(n))
    return out, s2i, i2s


def reorder_records(idx, in_records, in_s2i=None, index_space=None):
    """Gather of fixed-width records (rows of `in_records`, any dtype) by
    `idx`; slot maps as in reorder() when in_s2i is given."""
    n = idx.shape[0]
    src = np.ascontiguousarray(in_records)
    rb = src.shape[1] * src.itemsize
    out = np.empty((n,) + src.shape[1:], src.dtype)
    s2i = np.empty(n, np.int32) if in_s2i is not None else None
    i2s = np.full(index_space or n, -1, np.int32) if in_s2i is not None else None
    _call(load().orc_reorder_records, ptr(np.ascontiguousarray(idx, np.uint32)), ptr(src), ptr(out), C.c_uint32(rb),
          ptr(np.ascontiguousarray(in_s2i, np.int32)) if in_s2i is not None else None, ptr(s2i) if s2i is not None
          else None, ptr(i2s) if i2s is not None else None, C.c_uint32(n))
    return out, s2i, i2s


def sobol2d(i):
    x, y = C.c_float(), C.c_float()
    _call(load().orc_sobol2d, C.c_uint32(i), C.byref(x), C.byref(y))
    return x.value, y.value


def sincos_2pi(r):
    s, c = C.c_float(), C.c_float()
    _call(load().orc_sincos_2pi, C.c_float(r), C.byref(s), C.byref(c))
    return s.value, c.value


def raygen_shadow(seeds, in_rays, in_res, light, radius, bb, bs, S):
    ns = bs * S
    out = np.empty((ns, 8), np.float32)
    s2i = np.empty(ns, np.int32)
    i2s = np.empty(ns, np.int32)
    _call(load().orc_raygen_shadow, ptr(np.ascontiguousarray(seeds, np.uint32)), ptr(np.ascontiguousarray(in_rays, np.float32)),
                             ptr(np.ascontiguousarray(in_res, np.int32)), ptr(out), ptr(s2i), ptr(i2s),
                             ptr(_f(light, 3)), C.c_float(radius), C.c_int(bb), C.c_int(bs), C.c_int(S))
    return out, s2i, i2s


class HostGeometry:
    """Geometry table pointing at host arrays (96-byte vertices, uint32 indices)."""

    def __init__(self, vertices: np.ndarray, indices: np.ndarray):
        self.vertices = np.ascontiguousarray(vertices, np.float32)
        self.indices = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        self.table = np.array([[self.vertices.ctypes.data, self.indices.ctypes.data]], np.uint64)


def raygen_path(seeds, geom: HostGeometry, in_rays, in_i2p, in_res, decreases, albedo=0.8):
    n = in_rays.shape[0]
    seeds = np.ascontiguousarray(seeds, np.uint32).copy()
    dec = np.ascontiguousarray(decreases, np.float32).copy()
    out = np.zeros((n, 8), np.float32)
    out_i2p = np.zeros(n, np.int32)
    cnt = _call(load().orc_raygen_path, ptr(seeds), ptr(geom.table), ptr(np.ascontiguousarray(in_rays, np.float32)),
                                 ptr(out), ptr(np.ascontiguousarray(in_i2p, np.int32)), ptr(out_i2p),
                                 ptr(np.ascontiguousarray(in_res, np.int32)), ptr(dec), C.c_uint32(n),
                                 C.c_float(albedo))
    return seeds, out[:cnt], out_i2p[:cnt], dec, cnt


def reconstruct_smooth(rays, res, i2p, pixels, decreases, geom: HostGeometry, light, bg, spp):
    px = np.ascontiguousarray(pixels, np.float32).copy()
    n = rays.shape[0]
    _call(load().orc_reconstruct_smooth, ptr(np.ascontiguousarray(rays, np.float32)), ptr(np.ascontiguousarray(res, np.int32)),
                                  ptr(np.ascontiguousarray(i2p, np.int32)), ptr(px),
                                  ptr(np.ascontiguousarray(decreases, np.float32)), ptr(geom.table), ptr(_f(light, 3)),
                                  ptr(_f(bg, 3)), C.c_uint32(n), C.c_int(spp))
    return px


def reconstruct_shadow(res, i2p, i2s, in_pixels, out_pixels, bb, bs, S, replace=False):
    out = np.ascontiguousarray(out_pixels, np.float32).copy()
    _call(load().orc_reconstruct_shadow, ptr(np.ascontiguousarray(res, np.int32)), ptr(np.ascontiguousarray(i2p, np.int32)),
                                  ptr(np.ascontiguousarray(i2s, np.int32)),
                                  ptr(np.ascontiguousarray(in_pixels, np.float32)), ptr(out), C.c_int(bb),
                                  C.c_int(bs), C.c_int(S), C.c_int(1 if replace else 0))
    return out


def count_hits(res):
    res = np.ascontiguousarray(res, np.int32)
    return int(_call(load().orc_count_hits, ptr(res), C.c_uint32(res.shape[0])))


def interpolate_colors(frame_pixels, pixels, frame_index, key, white):
    fp = np.ascontiguousarray(frame_pixels, np.float32).copy()
    pp = np.ascontiguousarray(pixels, np.float32).copy()
    _call(load().orc_interpolate_colors, ptr(fp), ptr(pp), C.c_uint32(fp.shape[0]), C.c_int(frame_index), C.c_float(key),
                                  C.c_float(white))
    return fp, pp


def trace_bvh2(nodes: np.ndarray, tris: np.ndarray, rays, closest=True, ray_index=None):
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    res = np.empty((n, 4), np.int32)
    ri = None if ray_index is None else np.ascontiguousarray(ray_index, np.uint32)
    _call(load().orc_trace_bvh2, ptr(nodes), ptr(tris), ptr(rays), ptr(res), ptr(ri), C.c_uint32(n),
                          C.c_int(1 if closest else 0))
    return res


def trace_brute(tris: np.ndarray, rays, closest=True):
    """Closest hit over every triangle record (no BVH), same test and tie
    rule as trace_bvh2."""
    rays = np.ascontiguousarray(rays, np.float32)
    t = np.ascontiguousarray(tris)
    nt = t.nbytes // 48
    res = np.empty((rays.shape[0], 4), np.int32)
    _call(load().orc_trace_brute, ptr(t), C.c_uint32(nt), ptr(rays), ptr(res), C.c_uint32(rays.shape[0]),
          C.c_int(1 if closest else 0))
    return res


class Fp64Scene:
    """FP64 closest/any-hit oracle over its own BVH."""

    def __init__(self, positions, indices, geometry_first=None):
        self._pos = np.ascontiguousarray(positions, np.float32)
        self._idx = np.ascontiguousarray(indices, np.uint32)
        gf = None if geometry_first is None else np.ascontiguousarray(geometry_first, np.uint32)
        self.h = _call(load().orc_fp64_scene_create, ptr(self._pos), ptr(self._idx), C.c_uint32(self._idx.shape[0]),
                                              ptr(gf), C.c_uint32(0 if gf is None else gf.shape[0]))

    def trace(self, rays, closest=True):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.empty(n, np.float64)
        tri = np.empty(n, np.int64)
        _call(load().orc_fp64_trace, C.c_void_p(self.h), ptr(rays), C.c_uint32(n), C.c_int(1 if closest else 0), ptr(t),
                              ptr(tri))
        return t, tri

    def __del__(self):
        try:
            _call(load().orc_fp64_scene_destroy, C.c_void_p(self.h))
        except Exception:
            pass


def render_frame(nodes, tris, geom: HostGeometry, smin, smax, light, bg, s2w, eye, zfar, w, h, cfg: FrameCfg,
                 pixels=None, accum=None):
    """One frame of Renderer::render.  With cfg.accumulate_fp64 the running
    mean lives in `accum` (float64 [w*h, 4], updated in place; allocated
    when None and returned as a fourth value)."""
    n = w * h
    px = np.zeros((n, 4), np.float32) if pixels is None else np.ascontiguousarray(pixels, np.float32).copy()
    fp = np.zeros((n, 4), np.float32)
    st = Stats()
    if cfg.accumulate_fp64 and accum is None:
        accum = np.zeros((n, 4), np.float64)
    _call(load().orc_render_frame, ptr(nodes), ptr(tris), ptr(geom.table), ptr(_f(smin, 3)), ptr(_f(smax, 3)),
                            ptr(_f(light, 3)), ptr(_f(bg, 3)), ptr(_f(s2w, 16)), ptr(_f(eye, 3)), C.c_float(zfar),
                            C.c_int(w), C.c_int(h), C.byref(cfg), ptr(px), ptr(fp), C.byref(st),
                            ptr(accum) if cfg.accumulate_fp64 else None)
    if cfg.accumulate_fp64:
        return px, fp, st, accum
    return px, fp, st


def interpolate_colors_fp64(frame_pixels, pixels, accum, frame_index, key, white):
    """Returns (frame_pixels, pixels, accum) after one FP64 running-mean step."""
    fp = np.ascontiguousarray(frame_pixels, np.float32).copy()
    pp = np.ascontiguousarray(pixels, np.float32).copy()
    acc = np.ascontiguousarray(accum, np.float64).copy()
    _call(load().orc_interpolate_colors_fp64, ptr(fp), ptr(pp), ptr(acc), C.c_uint32(fp.shape[0]),
          C.c_int(frame_index), C.c_float(key), C.c_float(white))
    return fp, pp, acc
