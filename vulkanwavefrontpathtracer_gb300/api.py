"""Python host interface over the C ABI, mirroring the reference's stage
interface (RayGen, Tracer, Renderer) with torch CUDA tensors as buffers.

Buffer layouts (all torch tensors on one CUDA device):
  rays      float32 [n, 8]   origin.xyz, tmin, direction.xyz, tmax  (Ray, Ray.h:32-37)
  hits      int32   [n, 4]   primitiveId, geometryId, t (float bits), packedBary (RayResult)
  pixels    float32 [n, 4]   RGBA per pixel
  slot maps int32   [n]
  keys      int32/int64 [n]  Morton keys (32-bit or 64-bit patterns)
Every call is asynchronous on the current torch stream (or `stream`).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib as L

try:
    import torch
except ImportError:  # pragma: no cover - torch is a hard dependency of the GPU path
    torch = None


def _p(t) -> Optional[C.c_void_p]:
    return None if t is None else C.c_void_p(t.data_ptr())


def _s(stream=None) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream.cuda_stream)


def _n(t, n):
    return int(t.shape[0]) if n is None else int(n)


def lib():
    return L.load()


def device_status() -> int:
    """Synchronises and returns the device status bits; raises on a timeout
    or bounds flag."""
    flags = C.c_uint32(0)
    st = lib().wfpt_device_status(C.byref(flags))
    L.check(st)
    return flags.value


def tune_set(key: str, value: int) -> None:
    """Sets a process-wide tuning knob (see wfpt_tune_set in include/wfpt.h)."""
    L.check(lib().wfpt_tune_set(key.encode(), int(value)))


def selftest_wait_timeout(which: int) -> int:
    """Runs one bounded device wait that cannot succeed (0: radix sort
    look-back, 1: path compaction look-back) and returns the wfpt_status
    that wfpt_device_status reports afterwards (WFPT_ERR_TIMEOUT = 4 when
    the wait gave up as designed)."""
    return int(lib().wfpt_selftest_wait_timeout(int(which)))


def tune_get(key: str) -> int:
    v = C.c_int64(0)
    L.check(lib().wfpt_tune_get(key.encode(), C.byref(v)))
    return v.value


def trace_counters(reset: bool = True) -> dict:
    """Counters of the counting traversal kernels (enable with
    tune_set("trace.count", 1))."""
    out = (C.c_uint64 * 4)()
    L.check(lib().wfpt_trace_counters(out, 1 if reset else 0))
    return {"nodes": out[0], "tris": out[1], "rays": out[2], "warp_iters": out[3]}


# ------------------------------------------------------------ host helpers
def pixel_table(width: int, height: int):
    i2p = np.empty(width * height, np.int32)
    p2i = np.empty(width * height, np.int32)
    L.check(lib().wfpt_pixel_table(width, height, i2p.ctypes.data, p2i.ctypes.data))
    return i2p, p2i


def camera_screen_to_world(position, rotation_deg, fov_deg, aspect, znear, zfar) -> np.ndarray:
    out = (C.c_float * 16)()
    L.check(lib().wfpt_camera_screen_to_world(L.fvec(position, 3), L.fvec(rotation_deg, 3), fov_deg, aspect, znear,
                                              zfar, out))
    return np.array(out, dtype=np.float32)


# ------------------------------------------------------------ stage kernels
def init_seeds(seeds, frame_index: int, n=None, stream=None):
    L.check(lib().wfpt_init_seeds(_p(seeds), _n(seeds, n), frame_index, _s(stream)))


def raygen_primary(screen_to_world, index_to_pixel, rays, origin, sample_index, width, height, max_dist, stream=None):
    L.check(lib().wfpt_raygen_primary(L.fvec(np.asarray(screen_to_world, np.float32).ravel(), 16),
                                      _p(index_to_pixel), _p(rays), L.fvec(origin, 3), sample_index, width, height,
                                      max_dist, _s(stream)))


def morton(rays, scene_min, scene_size, kind, keys, indices, n=None, n_dev=None, stream=None):
    L.check(lib().wfpt_morton(_p(rays), _n(rays, n), _p(n_dev), L.fvec(scene_min, 3), L.fvec(scene_size, 3), kind,
                              _p(keys), _p(indices), _s(stream)))


def sort_scratch_bytes(n: int, key_bits: int) -> int:
    return int(lib().wfpt_sort_scratch_bytes(n, key_bits))


def sort_pairs(keys, values, key_bits, scratch=None, n=None, n_dev=None, stream=None):
    n = _n(keys, n)
    need = sort_scratch_bytes(n, key_bits)
    if scratch is None:
        scratch = torch.empty(max(need, 1), dtype=torch.uint8, device=keys.device)
    L.check(lib().wfpt_sort_pairs(_p(keys), _p(values), n, _p(n_dev), key_bits, _p(scratch), scratch.numel(),
                                  _s(stream)))
    return scratch


def reorder(ray_index, in_rays, out_rays, in_slot_to_index, out_slot_to_index, out_index_to_slot, n=None,
            n_dev=None, stream=None):
    L.check(lib().wfpt_reorder(_p(ray_index), _p(in_rays), _p(out_rays), _p(in_slot_to_index), _p(out_slot_to_index),
                               _p(out_index_to_slot), _n(ray_index, n), _p(n_dev), _s(stream)))


def reorder_records(ray_index, in_records, out_records, in_slot_to_index=None, out_slot_to_index=None,
                    out_index_to_slot=None, n=None, n_dev=None, stream=None):
    """Reorder gather of fixed-width records (rows of 16, 32, 48 or 64
    bytes); the slot maps are optional, as in wfpt_reorder_records."""
    if in_records.dim() != 2 or not in_records.is_contiguous() or not out_records.is_contiguous():
        raise ValueError("records are the rows of a contiguous 2-D tensor")
    rb = in_records.stride(0) * in_records.element_size()
    if out_records.dim() != 2 or out_records.stride(0) * out_records.element_size() != rb:
        raise ValueError("in_records and out_records rows differ in width")
    L.check(lib().wfpt_reorder_records(_p(ray_index), _p(in_records), _p(out_records), rb, _p(in_slot_to_index),
                                       _p(out_slot_to_index), _p(out_index_to_slot), _n(ray_index, n), _p(n_dev),
                                       _s(stream)))


def trace(scene: "Scene", bvh_kind, rays, results, ray_index=None, closest_hit=True, n=None, n_dev=None,
          stream=None):
    L.check(lib().wfpt_trace(scene.handle, bvh_kind, _p(rays), _p(results), _p(ray_index), _n(rays, n), _p(n_dev),
                             1 if closest_hit else 0, _s(stream)))


def trace_sort(scene: "Scene", bvh_kind, rays, results, scene_min, scene_max, morton_kind, reorder, keys, indices,
               rays_out=None, slot_to_index=None, slot_to_index_out=None, index_to_slot_out=None, closest_hit=True,
               scratch=None, n=None, n_dev=None, stream=None):
    """Tracer::traceSort: Morton -> sort -> reorder (or indirect) -> trace."""
    n = _n(rays, n)
    if scratch is None:
        scratch = torch.empty(max(sort_scratch_bytes(n, 64), 1), dtype=torch.uint8, device=rays.device)
    L.check(lib().wfpt_trace_sort(scene.handle, bvh_kind, _p(rays), _p(results), n, _p(n_dev),
                                  L.fvec(scene_min, 3), L.fvec(scene_max, 3), morton_kind, 1 if reorder else 0,
                                  _p(rays_out), _p(slot_to_index), _p(slot_to_index_out), _p(index_to_slot_out),
                                  _p(keys), _p(indices), 1 if closest_hit else 0, _p(scratch), scratch.numel(),
                                  _s(stream)))
    return scratch


def raygen_shadow(seeds, in_rays, in_results, out_rays, out_slot_to_index, out_index_to_slot, light, light_radius,
                  batch_begin, batch_size, num_samples, n_in_dev=None, stream=None):
    L.check(lib().wfpt_raygen_shadow(_p(seeds), _p(in_rays), _p(in_results), _p(out_rays), _p(out_slot_to_index),
                                     _p(out_index_to_slot), L.fvec(light, 3), light_radius, batch_begin, batch_size,
                                     _p(n_in_dev), num_samples, _s(stream)))


def raygen_path_scratch_bytes(n: int) -> int:
    return int(lib().wfpt_raygen_path_scratch_bytes(n))


def raygen_path(seeds, geometries, in_rays, out_rays, in_index_to_pixel, out_index_to_pixel, in_results, decreases,
                out_count, n=None, n_dev=None, albedo=0.8, russian_roulette=False, scratch=None, stream=None):
    n = _n(in_rays, n)
    if scratch is None:
        scratch = torch.empty(raygen_path_scratch_bytes(n), dtype=torch.uint8, device=in_rays.device)
    L.check(lib().wfpt_raygen_path(_p(seeds), _p(geometries), _p(in_rays), _p(out_rays), _p(in_index_to_pixel),
                                   _p(out_index_to_pixel), _p(in_results), _p(decreases), _p(out_count), n, _p(n_dev),
                                   1 if russian_roulette else 0, albedo, _p(scratch), scratch.numel(), _s(stream)))
    return scratch


RAYGEN_PATH_STATIC_MAX_RAYS = 16777216


def raygen_path_static(seeds, geometries, in_rays, out_rays, in_index_to_pixel, out_index_to_pixel, in_results,
                       decreases, out_count, n=None, n_dev=None, albedo=0.8, russian_roulette=False, stream=None):
    """raygen_path over the library's own fixed scratch: allocates nothing.
    n at most RAYGEN_PATH_STATIC_MAX_RAYS; calls on one device must not
    overlap in time (they share the scratch)."""
    L.check(lib().wfpt_raygen_path_static(_p(seeds), _p(geometries), _p(in_rays), _p(out_rays),
                                          _p(in_index_to_pixel), _p(out_index_to_pixel), _p(in_results),
                                          _p(decreases), _p(out_count), _n(in_rays, n), _p(n_dev),
                                          1 if russian_roulette else 0, albedo, _s(stream)))


def reconstruct_smooth(rays, results, index_to_pixel, pixels, decreases, geometries, light, background,
                       num_samples, n=None, n_dev=None, stream=None):
    L.check(lib().wfpt_reconstruct_smooth(_p(rays), _p(results), _p(index_to_pixel), _p(pixels), _p(decreases),
                                          _p(geometries), L.fvec(light, 3), L.fvec(background, 3), _n(rays, n),
                                          _p(n_dev), num_samples, _s(stream)))


def reconstruct_shadow(shadow_results, index_to_pixel, index_to_slot, in_pixels, out_pixels, batch_begin, batch_size,
                       num_samples, replace=False, n_in_dev=None, stream=None):
    L.check(lib().wfpt_reconstruct_shadow(_p(shadow_results), _p(index_to_pixel), _p(index_to_slot), _p(in_pixels),
                                          _p(out_pixels), batch_begin, batch_size, _p(n_in_dev), num_samples,
                                          1 if replace else 0, _s(stream)))


def count_hits(results, count, n=None, n_dev=None, stream=None):
    L.check(lib().wfpt_count_hits(_p(results), _n(results, n), _p(n_dev), _p(count), _s(stream)))


def interpolate_colors(frame_pixels, pixels, frame_index, key_value, white_point, n=None, stream=None):
    L.check(lib().wfpt_interpolate_colors(_p(frame_pixels), _p(pixels), _n(pixels, n), frame_index, key_value,
                                          white_point, _s(stream)))


def interpolate_colors_fp64(frame_pixels, pixels, accum, frame_index, key_value, white_point, n=None, stream=None):
    """interpolate_colors with the running mean in double: accum is a
    float64 tensor of 4 values per pixel (xyz the mean), kept across frames."""
    if accum.dtype != torch.float64 or accum.numel() < 4 * _n(pixels, n):
        raise ValueError("accum must be a float64 tensor of 4 values per pixel")
    L.check(lib().wfpt_interpolate_colors_fp64(_p(frame_pixels), _p(pixels), _p(accum), _n(pixels, n), frame_index,
                                               key_value, white_point, _s(stream)))


def fill_u32(dst, pattern: int, count: int, stream=None):
    L.check(lib().wfpt_fill_u32(_p(dst), pattern & 0xFFFFFFFF, count, _s(stream)))


# ------------------------------------------------------------------ scenes
def generate_scene(kind: int, seed: int, num_triangles: int = 0):
    """Seeded synthetic scene: (positions [V,3] f32, normals [V,3] f32,
    indices [T,3] u32).  kind 0 soup, 1 courtyard, 2 city (3M), 3 city ~N."""
    nv = C.c_uint32(0)
    nt = C.c_uint32(0)
    L.check(lib().wfpt_generate_scene(kind, seed, num_triangles, None, None, C.byref(nv), None, C.byref(nt)))
    pos = np.empty((nv.value, 3), np.float32)
    nrm = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.uint32)
    L.check(lib().wfpt_generate_scene(kind, seed, num_triangles, pos.ctypes.data, nrm.ctypes.data, C.byref(nv),
                                      idx.ctypes.data, C.byref(nt)))
    return pos, nrm, idx


def gltf_vertices(positions: np.ndarray, normals: np.ndarray) -> np.ndarray:
    """Packs vertices in the 96-byte vkglTF::Vertex layout
    (base/VulkanglTFModel.h:221-228): pos.xyz, normal.xyz, uv.xy, then
    joint0, weight0, color, tangent (zero here)."""
    v = np.zeros((positions.shape[0], 24), np.float32)
    v[:, 0:3] = positions
    v[:, 3:6] = normals
    return v


class Geometry:
    """Device-side shading geometry: vertex buffer, index buffer and the
    geometry table {vertexAddr, indexAddr} (geometrytypes.glsl:9-12), one
    entry per geometry; geometry_first[g] (nullable: one geometry) is its
    first triangle, and its index address is pre-offset to it, as the
    reference offsets by firstIndex (WaveFrontPathTracer.cpp:268-271)."""

    def __init__(self, positions, normals, indices, device="cuda", geometry_first=None):
        self.vertices = torch.from_numpy(gltf_vertices(positions, normals)).to(device)
        self.indices = torch.from_numpy(np.ascontiguousarray(indices).view(np.int32).reshape(-1)).to(device)
        first = [0] if geometry_first is None else [int(x) for x in geometry_first]
        table = np.array([[self.vertices.data_ptr(), self.indices.data_ptr() + 12 * f] for f in first],
                         dtype=np.uint64)
        self.table = torch.from_numpy(table.view(np.int64)).to(device)
        self.host_vertices = gltf_vertices(positions, normals)
        self.host_indices = np.ascontiguousarray(indices, np.uint32)


class Scene:
    """Acceleration structures of one triangle mesh (replaces the BLAS/TLAS)."""

    HOST_ONLY = 0x100
    DEVICE_BUILD = 0x200

    def __init__(self, positions, indices, geometry_first=None, bvh2=True, bvh8=True, host_only=False,
                 device_build=False, _handle=None):
        if _handle is not None:
            h = _handle
        else:
            positions = np.ascontiguousarray(positions, np.float32)
            indices = np.ascontiguousarray(indices, np.uint32)
            gf = None if geometry_first is None else np.ascontiguousarray(geometry_first, np.uint32)
            mask = ((1 if bvh2 else 0) | (2 if bvh8 else 0) | (self.HOST_ONLY if host_only else 0)
                    | (self.DEVICE_BUILD if device_build else 0))
            h = C.c_void_p()
            L.check(lib().wfpt_scene_create(positions.ctypes.data, positions.shape[0], indices.ctypes.data,
                                            indices.shape[0], None if gf is None else gf.ctypes.data,
                                            0 if gf is None else gf.shape[0], mask, C.byref(h)))
        self._init_from_handle(h)

    @classmethod
    def from_device(cls, positions, indices, geometry_first=None, bvh2=True, bvh8=True, stream=None):
        """Builds the BVHs on the GPU from device tensors: positions float32
        (V, 3), indices int32/uint32 (T, 3); geometry_first a host array."""
        if not (positions.is_cuda and indices.is_cuda):
            raise ValueError("positions and indices must be device tensors")
        positions = positions.contiguous()
        indices = indices.contiguous()
        gf = None if geometry_first is None else np.ascontiguousarray(geometry_first, np.uint32)
        mask = (1 if bvh2 else 0) | (2 if bvh8 else 0)
        h = C.c_void_p()
        L.check(lib().wfpt_scene_create_device(_p(positions), positions.shape[0], _p(indices), indices.shape[0],
                                               None if gf is None else gf.ctypes.data,
                                               0 if gf is None else gf.shape[0], mask, _s(stream), C.byref(h)))
        return cls(None, None, _handle=h)

    def _init_from_handle(self, h):
        self.handle = h
        info = L.SceneInfo()
        L.check(lib().wfpt_scene_get_info(h, C.byref(info)))
        self.info = info
        self.bounds_min = np.array(info.bounds_min, np.float32)
        self.bounds_max = np.array(info.bounds_max, np.float32)

    def _export(self, fn):
        nb = C.c_size_t(0)
        tb = C.c_size_t(0)
        L.check(fn(self.handle, None, C.byref(nb), None, C.byref(tb)))
        nodes = np.empty(nb.value, np.uint8)
        tris = np.empty(tb.value, np.uint8)
        L.check(fn(self.handle, nodes.ctypes.data, C.byref(nb), tris.ctypes.data, C.byref(tb)))
        return nodes, tris

    def export_bvh2(self):
        """(nodes uint8[64*N], triangles uint8[48*T]) of the binary BVH."""
        return self._export(lib().wfpt_scene_export_bvh2)

    def export_bvh8(self):
        """(nodes uint8[80*N], triangles uint8[48*T]) of the 8-wide BVH."""
        return self._export(lib().wfpt_scene_export_bvh8)

    def close(self):
        if self.handle:
            lib().wfpt_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- renderer
def default_config(**overrides) -> L.RendererConfig:
    cfg = L.RendererConfig()
    lib().wfpt_renderer_config_default(C.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


def make_camera(position, rotation_deg=(0.0, 0.0, 0.0), fov_deg=45.0, znear=0.001, zfar=3.0) -> L.Camera:
    cam = L.Camera()
    cam.position[:] = [float(x) for x in position]
    cam.rotation_deg[:] = [float(x) for x in rotation_deg]
    cam.fov_deg = fov_deg
    cam.znear = znear
    cam.zfar = zfar
    return cam


class Renderer:
    """Renderer::render (Renderer.cpp:552-654) behind the C ABI."""

    def __init__(self, config: Optional[L.RendererConfig] = None, **overrides):
        cfg = config if config is not None else default_config(**overrides)
        h = C.c_void_p()
        L.check(lib().wfpt_renderer_create(C.byref(cfg), C.byref(h)))
        self.handle = h
        self.config = cfg

    def set_config(self, cfg: L.RendererConfig):
        L.check(lib().wfpt_renderer_set_config(self.handle, C.byref(cfg)))
        self.config = cfg

    def set_scene(self, scene: Scene, geometry: Geometry, light: Sequence[float], background: Sequence[float],
                  scene_min=None, scene_max=None):
        self._keep = (scene, geometry)
        L.check(lib().wfpt_renderer_set_scene(self.handle, scene.handle, _p(geometry.table),
                                              None if scene_min is None else L.fvec(scene_min, 3),
                                              None if scene_max is None else L.fvec(scene_max, 3),
                                              L.fvec(light, 3), L.fvec(background, 3)))

    def reset_frame_index(self):
        lib().wfpt_renderer_reset_frame_index(self.handle)

    def render(self, camera: L.Camera, width: int, height: int, pixels, frame_pixels, stream=None):
        L.check(lib().wfpt_renderer_render(self.handle, C.byref(camera), width, height, _p(pixels), _p(frame_pixels),
                                           _s(stream)))

    def stats(self) -> L.RenderStats:
        st = L.RenderStats()
        L.check(lib().wfpt_renderer_get_stats(self.handle, C.byref(st)))
        return st

    def close(self):
        if self.handle:
            lib().wfpt_renderer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Batched render requests behind the C ABI (wfpt_batch_*): every
    request's frame recorded once into one CUDA graph over `streams`
    branches and replayed per render() call.  Each request is a dict with
    scene (Scene), geometry (Geometry), light, background, camera (Camera),
    width, height, config (RendererConfig), pixels and frame_pixels (device
    float tensors of width*height*4)."""

    def __init__(self, requests, streams: int = 4):
        arr = (L.Request * len(requests))()
        self._keep = []
        for i, q in enumerate(requests):
            r = arr[i]
            r.scene = q["scene"].handle
            r.geometries = q["geometry"].table.data_ptr()
            r.light[:] = [float(x) for x in q["light"]]
            r.background[:] = [float(x) for x in q["background"]]
            r.camera = q["camera"]
            r.width, r.height = int(q["width"]), int(q["height"])
            r.config = q["config"]
            r.pixels = q["pixels"].data_ptr()
            r.frame_pixels = q["frame_pixels"].data_ptr()
            self._keep.append((q["scene"], q["geometry"], q["pixels"], q["frame_pixels"]))
        self.count = len(requests)
        h = C.c_void_p()
        L.check(lib().wfpt_batch_create(arr, self.count, streams, C.byref(h)))
        self.handle = h

    def render(self, cameras=None, stream=None):
        cams = None
        if cameras is not None:
            cams = (L.Camera * self.count)(*cameras)
        L.check(lib().wfpt_batch_render(self.handle, cams, _s(stream)))

    def stats(self, i: int) -> L.RenderStats:
        st = L.RenderStats()
        L.check(lib().wfpt_batch_get_stats(self.handle, i, C.byref(st)))
        return st

    def kernels(self) -> int:
        return int(lib().wfpt_batch_kernels(self.handle))

    def reset_frame_index(self):
        lib().wfpt_batch_reset_frame_index(self.handle)

    def close(self):
        if self.handle:
            lib().wfpt_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
