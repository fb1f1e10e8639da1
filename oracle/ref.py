"""Test infrastructure: ctypes binding of oracle/_ref/libref.so, the
reference's own shader and host sources compiled for the CPU by
oracle/ref_build.py.  The tests use it to pin the restatement in oracle.cpp
(and, through fixtures written by tests/golden/make_ref_golden.py, the GPU
kernels).  Building it needs the reference checkout; available() says
whether it could be built here.  Array conventions follow oracle/__init__.py:
rays float32 [n, 8], hits int32 [n, 4], pixels float32 [n, 4].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ref_build as _build

_lib = None
_err = None


def available() -> bool:
    global _err
    try:
        load()
        return True
    except FileNotFoundError as e:
        _err = str(e)
        return False


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        lib.ref_raygen_path.restype = C.c_uint32
        lib.ref_count_hits.restype = C.c_uint32
        _lib = lib
    return _lib


_KEEP: list = []


def _p(a):
    """Pointer to a numpy array, which is kept alive until the current entry
    point returns (a temporary passed inline would otherwise be freed before
    the C function reads it)."""
    if a is None:
        return None
    _KEEP.append(a)
    return C.c_void_p(a.ctypes.data)


def _call(name, *args):
    try:
        return getattr(load(), name)(*args)
    finally:
        _KEEP.clear()


def _c(a, dt):
    return np.ascontiguousarray(a, dt)


def _v3(v):
    return _c(np.asarray(v, np.float32).reshape(3), np.float32)


def init_seeds(n, frame_index):
    s = np.empty(n, np.uint32)
    _call("ref_init_seeds", _p(s), C.c_int(n), C.c_int(frame_index))
    return s


def pixel_table(w, h):
    a = np.empty(w * h, np.int32)
    b = np.empty(w * h, np.int32)
    _call("ref_pixel_table", C.c_int(w), C.c_int(h), _p(a), _p(b))
    return a, b


def camera_screen_to_world(pos, rot, fov, aspect, zn, zf):
    """Returns (screenToWorld, view, perspective), each 16 floats column-major."""
    out = np.empty(16, np.float32)
    view = np.empty(16, np.float32)
    proj = np.empty(16, np.float32)
    _call("ref_camera_screen_to_world", _p(_v3(pos)), _p(_v3(rot)), C.c_float(fov), C.c_float(aspect), C.c_float(zn),
                                      C.c_float(zf), _p(out), _p(view), _p(proj))
    return out, view, proj


def raygen_primary(m, i2p, origin, sample_index, w, h, max_dist):
    rays = np.empty((w * h, 8), np.float32)
    m = _c(np.asarray(m, np.float32).reshape(16), np.float32)
    i2p = _c(i2p, np.int32)
    o = _v3(origin)
    _call("ref_raygen_primary", _p(m), _p(i2p), _p(rays), _p(o), C.c_int(sample_index), C.c_int(w), C.c_int(h),
                              C.c_float(max_dist))
    return rays


def morton_aila32(rays, smin, ssize):
    rays = _c(rays, np.float32)
    n = rays.shape[0]
    keys = np.empty(n, np.uint32)
    idx = np.empty(n, np.uint32)
    a, b = _v3(smin), _v3(ssize)
    _call("ref_morton_aila32", _p(rays), C.c_uint32(n), _p(a), _p(b), _p(keys), _p(idx))
    return keys, idx


def reorder(idx, in_rays, in_s2i, index_space=None):
    idx = _c(idx, np.uint32)
    in_rays = _c(in_rays, np.float32)
    in_s2i = _c(in_s2i, np.int32)
    n = idx.shape[0]
    out = np.empty((n, 8), np.float32)
    s2i = np.empty(n, np.int32)
    i2s = np.full(index_space or n, -1, np.int32)
    _call("ref_reorder", _p(idx), _p(in_rays), _p(out), _p(in_s2i), _p(s2i), _p(i2s), C.c_int(n))
    return out, s2i, i2s


def raygen_shadow(seeds, in_rays, in_res, light, radius, bb, bs, S):
    seeds, in_rays, in_res = _c(seeds, np.uint32), _c(in_rays, np.float32), _c(in_res, np.int32)
    out = np.empty((bs * S, 8), np.float32)
    s2i = np.empty(bs * S, np.int32)
    i2s = np.empty(bs * S, np.int32)
    _call("ref_raygen_shadow", _p(seeds), _p(in_rays), _p(in_res), _p(out), _p(s2i), _p(i2s), _p(_v3(light)),
                             C.c_float(radius), C.c_int(bb), C.c_int(bs), C.c_int(S))
    return out, s2i, i2s


def raygen_path(seeds, table, in_rays, in_i2p, in_res, decreases):
    """table: uint64 [g, 2] of {vertexAddr, indexAddr} host addresses (the
    arrays must stay alive).  Returns seeds, out rays, out i2p, decreases,
    count, as oracle.raygen_path does."""
    n = in_rays.shape[0]
    seeds = _c(seeds, np.uint32).copy()
    dec = _c(decreases, np.float32).copy()
    out = np.zeros((n, 8), np.float32)
    out_i2p = np.zeros(n, np.int32)
    cnt = np.zeros(1, np.uint32)
    t, r, i, h = _c(table, np.uint64), _c(in_rays, np.float32), _c(in_i2p, np.int32), _c(in_res, np.int32)
    c = _call("ref_raygen_path", _p(seeds), _p(t), _p(r), _p(out), _p(i), _p(out_i2p), _p(h), _p(dec), _p(cnt),
                               C.c_int(n))
    return seeds, out[:c], out_i2p[:c], dec, int(c)


def reconstruct_smooth(rays, res, i2p, pixels, decreases, table, light, bg, spp):
    px = _c(pixels, np.float32).copy()
    r, h, i, d, t = (_c(rays, np.float32), _c(res, np.int32), _c(i2p, np.int32), _c(decreases, np.float32),
                     _c(table, np.uint64))
    _call("ref_reconstruct_smooth", _p(r), _p(h), _p(i), _p(px), _p(d), _p(t), _p(_v3(light)), _p(_v3(bg)),
                                  C.c_int(r.shape[0]), C.c_int(spp))
    return px


def reconstruct_shadow(res, i2p, i2s, in_pixels, out_pixels, bb, bs, S, replace=False):
    out = _c(out_pixels, np.float32).copy()
    h, a, b, ip = _c(res, np.int32), _c(i2p, np.int32), _c(i2s, np.int32), _c(in_pixels, np.float32)
    _call("ref_reconstruct_shadow", _p(h), _p(a), _p(b), _p(ip), _p(out), C.c_int(bb), C.c_int(bs), C.c_int(S),
                                  C.c_int(1 if replace else 0))
    return out


def count_hits(res):
    res = _c(res, np.int32)
    return int(_call("ref_count_hits", _p(res), C.c_int(res.shape[0])))


def interpolate_colors(frame_pixels, pixels, frame_index, key, white):
    fp = _c(frame_pixels, np.float32).copy()
    pp = _c(pixels, np.float32).copy()
    _call("ref_interpolate_colors", _p(fp), _p(pp), C.c_int(fp.shape[0]), C.c_int(frame_index), C.c_float(key),
                                  C.c_float(white))
    return fp, pp
