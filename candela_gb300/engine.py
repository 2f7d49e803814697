"""Python host side of the ray-query engine, over the C ABI (include/rq.h).

`RayIntersector` mirrors the reference's host wrapper `Candela::RayIntersector<T>`
(Source/Core/BVH/Intersector.h:60-451): objects are added one at a time (AddObject builds the
object's BVH and appends its nodes / triangles / vertices to global buffers, rebasing vertex
indices, :169-198), entities instance objects with a model matrix (PushEntity, :200-216),
BufferEntities / BufferData upload (:226-351), and queries run on the device.  Queries accept
device tensors (torch, resident in HBM) or host numpy arrays (copied inside the call).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import (ENTITY_DTYPE, HIT_DTYPE, RAY_DTYPE, STACK_NODE_DTYPE, STACKLESS_NODE_DTYPE,
                   TRI_DTYPE, VERTEX_DTYPE, check, lib, ptr)

STACK, STACKLESS, BVH8Q = L.LAYOUT_STACK, L.LAYOUT_STACKLESS, L.LAYOUT_BVH8Q


@dataclass
class BVH:
    """Host buffers of one object's BVH, in the reference's byte layout."""
    layout: int
    nodes: np.ndarray       # STACK_NODE_DTYPE or STACKLESS_NODE_DTYPE
    tris: np.ndarray        # TRI_DTYPE
    n_nodes_used: int
    leaf_count: int
    split_fails: int
    build_ms: float


def build_bvh(vertices: np.ndarray, indices: np.ndarray, mesh_ids=None, tri_offset: int = 0,
              layout: int = STACK, leaf_size: int = 2, swap_children: bool = False,
              swap_seed: int = 0, n_threads: int = 0, ctx=None) -> BVH:
    """BVH::BuildBVH for one object (BVHConstructor.cpp:951-1108) via rq_build_bvh, or via
    rq_build_bvh_gpu on the context's GPU when `ctx` is given (same buffers)."""
    v = np.ascontiguousarray(vertices, dtype=VERTEX_DTYPE)
    idx = np.ascontiguousarray(indices, dtype=np.uint32).ravel()
    mid = None if mesh_ids is None else np.ascontiguousarray(mesh_ids, dtype=np.int32)
    opts = L.RqBuildOpts(leaf_size, int(swap_children), swap_seed & 0xFFFFFFFF, n_threads)
    h = C.c_void_p()
    if ctx is None:
        check(lib().rq_build_bvh(ptr(v), v.shape[0], ptr(idx), idx.size, ptr(mid), tri_offset, layout,
                                 C.byref(opts), C.byref(h)))
    else:
        check(lib().rq_build_bvh_gpu(ctx.handle, ptr(v), v.shape[0], ptr(idx), idx.size, ptr(mid), tri_offset,
                                     layout, C.byref(opts), C.byref(h)), ctx.handle)
    try:
        info = L.RqBvhInfo()
        check(lib().rq_bvh_info_get(h, C.byref(info)))
        np_ = C.c_void_p()
        nn = C.c_int64()
        check(lib().rq_bvh_nodes(h, C.byref(np_), C.byref(nn)))
        dt = STACK_NODE_DTYPE if layout == STACK else STACKLESS_NODE_DTYPE
        nodes = np.frombuffer(C.string_at(np_.value, nn.value * dt.itemsize), dtype=np.float32)
        nodes = nodes.reshape(nn.value, dt.itemsize // 4).copy()
        tp = C.c_void_p()
        nt = C.c_int64()
        check(lib().rq_bvh_triangles(h, C.byref(tp), C.byref(nt)))
        tris = np.frombuffer(C.string_at(tp.value, nt.value * 16), dtype=np.int32).reshape(-1, 4).copy()
        return BVH(layout, nodes, tris, info.n_nodes_used, info.leaf_count, info.split_fails,
                   info.build_ms)
    finally:
        lib().rq_bvh_free(h)


def build_bvh8_host(layout, nodes, tris, vertices, node_offset=0, node_count=None):
    """rq_build_bvh8: host-side BVH8 of one object.  Returns (nodes uint32 (N, 20),
    triangle records float32 (M, 16))."""
    n = np.ascontiguousarray(nodes, dtype=np.float32)
    t = np.ascontiguousarray(tris, dtype=np.int32)
    v = np.ascontiguousarray(vertices)
    node_count = n.shape[0] - node_offset if node_count is None else node_count
    h = C.c_void_p()
    check(lib().rq_build_bvh8(layout, ptr(n), n.shape[0], ptr(t), t.shape[0], ptr(v), v.shape[0],
                              node_offset, node_count, C.byref(h)))
    try:
        np_, nn, tp, nt = C.c_void_p(), C.c_int64(), C.c_void_p(), C.c_int64()
        check(lib().rq_bvh8_buffers(h, C.byref(np_), C.byref(nn), C.byref(tp), C.byref(nt)))
        nodes8 = np.frombuffer(C.string_at(np_.value, nn.value * 80), dtype=np.uint32).reshape(-1, 20).copy()
        recs = (np.frombuffer(C.string_at(tp.value, nt.value * 64), dtype=np.float32).reshape(-1, 16).copy()
                if nt.value else np.zeros((0, 16), np.float32))
        return nodes8, recs
    finally:
        lib().rq_bvh8_free(h)


def validate_scene(layout, vertices, tris, nodes, entities) -> tuple[bool, str]:
    """rq_scene_validate: host-only check of the buffers a scene upload would receive."""
    msg = C.create_string_buffer(512)
    v = np.ascontiguousarray(vertices)
    t = np.ascontiguousarray(tris, dtype=np.int32)
    n = np.ascontiguousarray(nodes, dtype=np.float32)
    e = np.ascontiguousarray(entities, dtype=ENTITY_DTYPE)
    s = lib().rq_scene_validate(layout, ptr(v), v.shape[0], ptr(t), t.shape[0], ptr(n), n.shape[0],
                                ptr(e), e.shape[0], msg, 512)
    return s == L.RQ_OK, msg.value.decode()


def identity_entity(node_offset: int, node_count: int, emissive: float = 0.0,
                    alpha: float = 1.0, model=None) -> np.ndarray:
    """A BVHEntity record (Intersector.h:43-49, PushEntity :200-216)."""
    e = np.zeros(1, dtype=ENTITY_DTYPE)
    m = np.eye(4, dtype=np.float32) if model is None else np.asarray(model, dtype=np.float32)
    inv = np.linalg.inv(m.astype(np.float64)).astype(np.float32) if model is not None else m
    e["model"] = m.T.ravel()      # glm column-major
    e["inverse"] = inv.T.ravel()
    e["node_offset"] = node_offset
    e["node_count"] = node_count
    e["data"][0, 0] = np.float32(emissive).view(np.int32)
    e["data"][0, 1] = np.float32(alpha).view(np.int32)
    return e


class Context:
    """rq_ctx on one CUDA device."""

    def __init__(self, device: int = 0):
        self.handle = C.c_void_p()
        check(lib().rq_create(device, C.byref(self.handle)))
        self.device = device

    def close(self):
        if self.handle:
            lib().rq_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_status(self, reset: bool = True) -> int:
        """Kernel status bits since the last reset (1 = BVH8 stack overflow, 2 = visit budget)."""
        b = C.c_uint32()
        check(lib().rq_device_status(self.handle, C.byref(b), int(reset)), self.handle)
        return b.value

    def read_counters(self, reset: bool = True) -> dict:
        """Node visits / triangle tests accumulated by queries run with FLAG_COUNT."""
        c = (C.c_int64 * 2)()
        check(lib().rq_counters_read(self.handle, C.byref(c), int(reset)), self.handle)
        return {"node_visits": c[0], "triangle_tests": c[1]}

    def read_bandwidth(self, nbytes: int, reps: int = 50) -> float:
        """Measured read bandwidth (GB/s) over a device buffer of nbytes (rq_measure_read_gbs)."""
        g = C.c_double()
        check(lib().rq_measure_read_gbs(self.handle, int(nbytes), int(reps), C.byref(g)), self.handle)
        return g.value

    def scene(self, layout, vertices, tris, nodes, entities) -> "Scene":
        return Scene(self, layout, vertices, tris, nodes, entities)


def _stream(t, stream):
    """Stream for a device-tensor call: the caller's, else torch's current stream on the
    tensor's device, so results are ordered with the torch work that consumes them."""
    if stream is not None or t is None or isinstance(t, np.ndarray):
        return stream
    import torch
    return torch.cuda.current_stream(t.device).cuda_stream


def _opts(layout=0, mode=0, tie=0, flags=0, block_size=0, min_blocks=0, persistent=0, stack_depth=0) -> L.RqOpts:
    return L.RqOpts(layout, mode, tie, flags, block_size, min_blocks, persistent, stack_depth)


class Scene:
    """Device-resident scene (rq_scene): global vertex / triangle / node buffers + entities."""

    def __init__(self, ctx: Context, layout, vertices, tris, nodes, entities):
        self.ctx = ctx
        self.layout = layout
        v = np.ascontiguousarray(vertices)
        t = np.ascontiguousarray(tris, dtype=np.int32)
        n = np.ascontiguousarray(nodes, dtype=np.float32)
        e = np.ascontiguousarray(entities, dtype=ENTITY_DTYPE)
        self.handle = C.c_void_p()
        self.n_verts = v.shape[0]
        check(lib().rq_scene_create(ctx.handle, layout, ptr(v), v.shape[0], ptr(t), t.shape[0],
                                    ptr(n), n.shape[0], ptr(e), e.shape[0], C.byref(self.handle)),
              ctx.handle)

    def set_entities(self, entities):
        e = np.ascontiguousarray(entities, dtype=ENTITY_DTYPE)
        check(lib().rq_scene_set_entities(self.handle, ptr(e), e.shape[0]), self.ctx.handle)

    def autotune(self, rays, query: int = 0, layout: int = 0) -> dict:
        """rq_autotune on device rays: times each launch variant, keeps the fastest."""
        n = rays.numel() * rays.element_size() // 32
        r = L.RqTuneResult()
        check(lib().rq_autotune(self.ctx.handle, self.handle, ptr(rays), n, query,
                                layout or self.layout, C.byref(r)), self.ctx.handle)
        variants = [dict(block=r.block[i], min_blocks=r.min_blocks_of[i],
                         persistent=r.persistent_of[i], stack_depth=r.depth_of[i], ms=round(r.ms[i], 4))
                    for i in range(r.n_variants)]
        return dict(variant=r.variant, block_size=r.block_size, min_blocks=r.min_blocks,
                    persistent=r.persistent, stack_depth=r.depth, variants=variants)

    def verify(self, rays, hits, stream=None):
        """rq_verify_hits: FP64 relative t error and barycentric error per hit ((n, 2), NaN = miss)."""
        import torch
        n = rays.numel() * rays.element_size() // 32
        err = torch.empty((n, 2), dtype=torch.float32, device=rays.device)
        check(lib().rq_verify_hits(self.ctx.handle, self.handle, ptr(rays), ptr(hits), n, ptr(err),
                                   _stream(rays, stream)), self.ctx.handle)
        return err

    def build_bvh8(self) -> dict:
        """rq_scene_build_bvh8: enables RQ_LAYOUT_BVH8Q queries on this scene."""
        info = L.RqBvh8Info()
        check(lib().rq_scene_build_bvh8(self.handle, C.byref(info)), self.ctx.handle)
        return {k: getattr(info, k) for k, _ in L.RqBvh8Info._fields_}

    def device_bytes(self) -> int:
        b = C.c_int64()
        check(lib().rq_scene_bytes(self.handle, C.byref(b)))
        return b.value

    def close(self):
        if self.handle:
            lib().rq_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- queries -----------------------------------------------------------------------------
    def closest(self, rays, hits=None, *, layout=0, mode=0, tie=0, flags=0, block_size=0,
                min_blocks=0, persistent=0, stack_depth=0, stream=None):
        """Closest hit.  `rays` is a numpy RAY_DTYPE array (host path, copies inside the call)
        or a torch uint8/float tensor on the device holding 32-byte rays."""
        host = isinstance(rays, np.ndarray)
        n = rays.shape[0] if host else rays.numel() * rays.element_size() // 32
        if hits is None:
            if host:
                hits = np.empty(n, dtype=HIT_DTYPE)
            else:
                import torch
                hits = torch.empty((n, 8), dtype=torch.float32, device=rays.device)
        f = flags | (L.FLAG_HOST_BUFFERS if host else 0)
        o = _opts(layout, mode, tie, f, block_size, min_blocks, persistent, stack_depth)
        check(lib().rq_closest(self.ctx.handle, self.handle, ptr(rays), n, ptr(hits), C.byref(o),
                               _stream(rays, stream)), self.ctx.handle)
        return hits

    def hit_attribs(self, hits, out=None, *, stream=None):
        """GetData over hit records: (n, 8) float32 = normal xyz, alpha, albedo rgb, emissive
        (rq_hit_attribs).  numpy hits -> host path."""
        host = isinstance(hits, np.ndarray)
        n = hits.shape[0] if host else hits.numel() * hits.element_size() // 32
        if out is None:
            out = np.empty((n, 8), dtype=np.float32) if host else _empty_like_dev(hits, (n, 8), __import__("torch").float32)
        o = _opts(0, 0, 0, L.FLAG_HOST_BUFFERS if host else 0)
        check(lib().rq_hit_attribs(self.ctx.handle, self.handle, ptr(hits), n, ptr(out), C.byref(o),
                                   _stream(hits, stream)), self.ctx.handle)
        return out

    def closest_attribs(self, rays, *, layout=0, mode=0, tie=0, flags=0, block_size=0, min_blocks=0,
                        persistent=0, stack_depth=0, stream=None):
        """Closest hit + GetData (rq_closest_attribs): (hits, attribs)."""
        host = isinstance(rays, np.ndarray)
        n = rays.shape[0] if host else rays.numel() * rays.element_size() // 32
        if host:
            hits, att = np.empty(n, dtype=HIT_DTYPE), np.empty((n, 8), dtype=np.float32)
        else:
            import torch
            hits = torch.empty((n, 8), dtype=torch.float32, device=rays.device)
            att = torch.empty((n, 8), dtype=torch.float32, device=rays.device)
        o = _opts(layout, mode, tie, flags | (L.FLAG_HOST_BUFFERS if host else 0), block_size, min_blocks, persistent,
                  stack_depth)
        check(lib().rq_closest_attribs(self.ctx.handle, self.handle, ptr(rays), n, ptr(hits), ptr(att), C.byref(o),
                                       _stream(rays, stream)), self.ctx.handle)
        return hits, att

    def anyhit(self, rays, out=None, *, layout=0, mode=0, flags=0, block_size=0, min_blocks=0,
               persistent=0, stack_depth=0, stream=None):
        host = isinstance(rays, np.ndarray)
        n = rays.shape[0] if host else rays.numel() * rays.element_size() // 32
        if out is None:
            if host:
                out = np.empty(n, dtype=np.uint8)
            else:
                import torch
                out = torch.empty(n, dtype=torch.uint8, device=rays.device)
        f = flags | (L.FLAG_HOST_BUFFERS if host else 0)
        o = _opts(layout, mode, 0, f, block_size, min_blocks, persistent, stack_depth)
        check(lib().rq_anyhit(self.ctx.handle, self.handle, ptr(rays), n, ptr(out), C.byref(o),
                              _stream(rays, stream)), self.ctx.handle)
        return out

    def tlas_info(self) -> dict:
        """rq_scene_tlas_info: the top level over the entities (nodes 0 = every entity walked)."""
        buf = (C.c_int64 * 3)()
        check(lib().rq_scene_tlas_info(self.handle, C.byref(buf)), self.ctx.handle)
        w = np.frombuffer(bytes(buf), dtype=np.int32)
        return {"nodes": int(w[0]), "entities": int(w[1]), "cullable": int(w[2]), "bytes": int(buf[2])}

    def collide(self, boxes, out=None, *, flags=0, stream=None):
        """First (entity, mesh, triangle) each box overlaps (rq_collide; CollideScene of
        Collide.comp).  `boxes` is a float32 (n, 8) array {min.xyzw, max.xyzw} on the host
        (copies inside the call) or a CUDA tensor; returns int32 (n, 4) rows
        {collided, entity, mesh, tri}, {0, -1, -1, -1} for a box that overlaps nothing."""
        host = isinstance(boxes, np.ndarray)
        if host:
            boxes = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 8)
            n = boxes.shape[0]
        else:
            n = boxes.numel() * boxes.element_size() // 32
        if out is None:
            if host:
                out = np.empty((n, 4), dtype=np.int32)
            else:
                import torch
                out = torch.empty((n, 4), dtype=torch.int32, device=boxes.device)
        o = _opts(flags=flags | (L.FLAG_HOST_BUFFERS if host else 0))
        check(lib().rq_collide(self.ctx.handle, self.handle, ptr(boxes), n, ptr(out), C.byref(o),
                               _stream(boxes, stream)), self.ctx.handle)
        return out

    def collide_box(self, bmin, bmax, **kw) -> bool:
        """Physics::CollideBox (Physics.cpp:203-228): does the world-space box touch the scene."""
        b = np.array([[*bmin, 0.0, *bmax, 0.0]], dtype=np.float32)
        return bool(self.collide(b, **kw)[0, 0])

    def collide_points(self, points, half=0.01, **kw):
        """Physics::CollidePoint (Physics.cpp:176-201) for many points: each point is the box
        point -/+ half (0.01 in the reference); returns the rq_collide rows."""
        p = np.asarray(points, dtype=np.float32).reshape(-1, 3)
        b = np.zeros((p.shape[0], 8), dtype=np.float32)
        b[:, 0:3] = p - np.float32(half)
        b[:, 4:7] = p + np.float32(half)
        return self.collide(b, **kw)


def gi_params(spp=4, seed=0, origin_offset=0.05, ray_tmax=1000000.0, normal_mode=0, query=0,
              shadow_rays=False, shadow_offset=1e-3, sun_dir=(0.3, 0.4, -0.866),
              sun_color=(4.0, 3.8, 3.5), sky_color=(0.5, 0.7, 1.0), sort_rays=False,
              unfused=False, bounces=0, compact_below=0.0, pixel_format=0) -> L.RqGiParams:
    """rq_gi_params for the diffuse-GI (query=0) or RTAO (query=1) pass; `bounces` further
    bounces per GI hit (the RT second-bounce loop); `compact_below` the compaction threshold (0 =
    the scene's tuned value); `pixel_format` L.PIXELS_RGBA32F or L.PIXELS_RGBA16F (the output
    pixels as float16, the reference's rgba16f output image)."""
    sd = np.asarray(sun_dir, dtype=np.float64)
    sd = (sd / np.sqrt(sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2])).astype(np.float32)
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in v])  # noqa: E731
    return L.RqGiParams(spp, seed & 0xFFFFFFFF, origin_offset, ray_tmax, normal_mode, query,
                        int(shadow_rays), shadow_offset, f3(sd), f3(sun_color), f3(sky_color),
                        int(sort_rays), int(unfused), int(bounces), float(compact_below), int(pixel_format))


def specular_params(seed=0, roughness=0.3, ray_tmax=1000000.0, normal_mode=0, shadow_rays=False,
                    shadow_offset=1e-3, sun_dir=(0.3, 0.4, -0.866), sun_color=(4.0, 3.8, 3.5),
                    sky_color=(0.5, 0.7, 1.0), ambient=(0.1, 0.1, 0.12)) -> L.RqSpecularParams:
    """rq_specular_params for the specular reflection pass."""
    sd = np.asarray(sun_dir, dtype=np.float64)
    sd = (sd / np.sqrt(sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2])).astype(np.float32)
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in v])  # noqa: E731
    return L.RqSpecularParams(seed & 0xFFFFFFFF, roughness, ray_tmax, normal_mode, int(shadow_rays), shadow_offset,
                              f3(sd), f3(sun_color), f3(sky_color), f3(ambient))


def probe_params(grid=(128, 64, 128), origin=(0.0, 0.0, 0.0), prev_origin=None, size=(64.0, 32.0, 64.0), seed=0,
                 temporal=True, normal_mode=0, shadow_rays=True, shadow_offset=1e-3, ray_tmax=1000000.0,
                 sun_dir=(0.3, 0.4, -0.866), sun_color=(4.0, 3.8, 3.5), sky_color=(0.5, 0.7, 1.0)) -> L.RqProbeParams:
    """rq_probe_params for one frame of the radiance-probe update; prev_origin defaults to origin
    (a volume that did not move)."""
    sd = np.asarray(sun_dir, dtype=np.float64)
    sd = (sd / np.sqrt(sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2])).astype(np.float32)
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in v])  # noqa: E731
    return L.RqProbeParams((C.c_int32 * 3)(*[int(g) for g in grid]), f3(origin),
                           f3(origin if prev_origin is None else prev_origin), f3(size), seed & 0xFFFFFFFF,
                           int(temporal), normal_mode, int(shadow_rays), shadow_offset, ray_tmax, f3(sd),
                           f3(sun_color), f3(sky_color))


def probe_volumes(params, device=None):
    """Zeroed (sh (n, 8) int32 bit patterns, raw (n, 4), map (n, 128)) for a probe grid: numpy when
    device is None, else torch tensors on that device."""
    n = int(params.grid[0]) * int(params.grid[1]) * int(params.grid[2])
    if device is None:
        return (np.zeros((n, 8), dtype=np.uint32), np.zeros((n, 4), dtype=np.float32),
                np.zeros((n, 128), dtype=np.float32))
    import torch
    return (torch.zeros((n, 8), dtype=torch.int32, device=device), torch.zeros((n, 4), dtype=torch.float32, device=device),
            torch.zeros((n, 128), dtype=torch.float32, device=device))


def _empty_like_dev(ref, shape, dtype):
    import torch
    return torch.empty(shape, dtype=dtype, device=ref.device)


class _GiMixin:
    def set_materials(self, albedo_rgb):
        a = np.ascontiguousarray(albedo_rgb, dtype=np.float32).reshape(-1, 3)
        check(lib().rq_scene_set_materials(self.handle, ptr(a), a.shape[0]), self.ctx.handle)

    def set_textures(self, textures, mesh_texture):
        """rq_scene_set_textures.  textures: list of (rgba8 uint8 array (H, W, 4), srgb, wrap);
        mesh_texture: texture index per mesh id (-1: ModelColor)."""
        keep = [np.ascontiguousarray(t[0], dtype=np.uint8) for t in textures]
        arr = (L.RqTexture * max(1, len(keep)))()
        for k, (img, (_, srgb, wrap)) in enumerate(zip(keep, textures)):
            arr[k] = L.RqTexture(img.shape[1], img.shape[0], int(srgb), int(wrap), img.ctypes.data)
        mt = np.ascontiguousarray(mesh_texture, dtype=np.int32)
        check(lib().rq_scene_set_textures(self.handle, C.cast(arr, C.c_void_p), len(keep), ptr(mt), mt.size),
              self.ctx.handle)

    def gi_raygen(self, primary, hits, params, out=None, stream=None):
        """Device tensors: primary (n*32 bytes), hits (n, 8) -> secondary rays (n*spp*32 bytes)."""
        import torch
        n = primary.numel() * primary.element_size() // 32
        if out is None:
            out = torch.empty(n * params.spp * 32, dtype=torch.uint8, device=primary.device)
        check(lib().rq_gi_raygen(self.ctx.handle, self.handle, ptr(primary), ptr(hits), n,
                                 C.byref(params), ptr(out), _stream(primary, stream)), self.ctx.handle)
        return out

    def shadow_raygen(self, rays, hits, params, out=None, stream=None):
        import torch
        n = rays.numel() * rays.element_size() // 32
        if out is None:
            out = torch.empty(n * 32, dtype=torch.uint8, device=rays.device)
        check(lib().rq_shadow_raygen(self.ctx.handle, self.handle, ptr(rays), ptr(hits), n,
                                     C.byref(params), ptr(out), _stream(rays, stream)),
              self.ctx.handle)
        return out

    def shade(self, rays, hits, params, lit=None, out=None, stream=None):
        import torch
        n = rays.numel() * rays.element_size() // 32
        if out is None:
            out = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
        check(lib().rq_shade(self.ctx.handle, self.handle, ptr(rays), ptr(hits), n, ptr(lit),
                             C.byref(params), ptr(out), _stream(rays, stream)), self.ctx.handle)
        return out

    def specular_frame(self, primary, params, out=None, *, layout=0, mode=0, tie=0, flags=0, stream=None):
        """Specular reflection pass (rq_specular_frame): (n, 4) radiance and t / 48 per pixel."""
        host = isinstance(primary, np.ndarray)
        n = primary.shape[0] if host else primary.numel() * primary.element_size() // 32
        if out is None:
            out = (np.empty((n, 4), dtype=np.float32) if host
                   else _empty_like_dev(primary, (n, 4), __import__("torch").float32))
        o = _opts(layout, mode, tie, flags | (L.FLAG_HOST_BUFFERS if host else 0))
        check(lib().rq_specular_frame(self.ctx.handle, self.handle, ptr(primary), n, C.byref(params), C.byref(o),
                                      ptr(out), _stream(primary, stream)), self.ctx.handle)
        return out

    def probe_update(self, params, prev_sh, prev_raw, probe_map, out_sh=None, out_raw=None, *, layout=0, mode=0,
                     tie=0, flags=0, block_size=0, min_blocks=0, persistent=0, stack_depth=0, stream=None):
        """One frame of the radiance-probe update (rq_probe_update).  numpy volumes -> host path.
        probe_map is updated in place; returns (out_sh, out_raw)."""
        host = isinstance(prev_sh, np.ndarray)
        n = int(params.grid[0]) * int(params.grid[1]) * int(params.grid[2])
        if out_sh is None:
            out_sh = np.empty((n, 8), dtype=np.uint32) if host else _empty_like_dev(prev_sh, (n, 8), prev_sh.dtype)
        if out_raw is None:
            out_raw = (np.empty((n, 4), dtype=np.float32) if host
                       else _empty_like_dev(prev_raw, (n, 4), __import__("torch").float32))
        o = _opts(layout, mode, tie, flags | (L.FLAG_HOST_BUFFERS if host else 0), block_size, min_blocks,
                  persistent, stack_depth)
        check(lib().rq_probe_update(self.ctx.handle, self.handle, C.byref(params), ptr(prev_sh), ptr(prev_raw),
                                    ptr(probe_map), ptr(out_sh), ptr(out_raw), C.byref(o),
                                    _stream(prev_sh, stream)), self.ctx.handle)
        return out_sh, out_raw

    def gi_autotune(self, primary, params, out=None, *, layout=0, flags=0, block_size=0, min_blocks=0,
                    persistent=0, stack_depth=0) -> dict:
        """rq_gi_autotune on device primary rays: the compaction threshold of the GI pass."""
        n = primary.numel() * primary.element_size() // 32
        if out is None:
            out = _empty_like_dev(primary, (n, 4), __import__("torch").float32)
        r = L.RqGiTune()
        o = _opts(layout, 0, 0, flags, block_size, min_blocks, persistent, stack_depth)
        check(lib().rq_gi_autotune(self.ctx.handle, self.handle, ptr(primary), n, C.byref(params), C.byref(o),
                                   ptr(out), C.byref(r)), self.ctx.handle)
        return dict(compact_below=r.compact_below, live_fraction=r.live_fraction, ms_compact=round(r.ms_compact, 4),
                    ms_in_place=round(r.ms_in_place, 4))

    def gi_frame(self, primary, params, out=None, *, layout=0, mode=0, tie=0, flags=0,
                 block_size=0, min_blocks=0, persistent=0, stack_depth=0, stats=False, stream=None):
        """Whole GI / AO pass.  numpy primary rays -> host path (copies inside the call)."""
        host = isinstance(primary, np.ndarray)
        n = primary.shape[0] if host else primary.numel() * primary.element_size() // 32
        if out is None:
            half = params.pixel_format == L.PIXELS_RGBA16F
            if host:
                out = np.empty((n, 4), dtype=np.float16 if half else np.float32)
            else:
                torch = __import__("torch")
                out = _empty_like_dev(primary, (n, 4), torch.float16 if half else torch.float32)
        st = L.RqFrameStats() if stats else None
        o = _opts(layout, mode, tie, flags | (L.FLAG_HOST_BUFFERS if host else 0), block_size,
                  min_blocks, persistent, stack_depth)
        check(lib().rq_gi_frame(self.ctx.handle, self.handle, ptr(primary), n, C.byref(params),
                                C.byref(o), ptr(out), C.byref(st) if st is not None else None,
                                _stream(primary, stream)), self.ctx.handle)
        if stats:
            return out, {k: getattr(st, k) for k, _ in L.RqFrameStats._fields_}
        return out


for _name, _fn in list(vars(_GiMixin).items()):
    if callable(_fn) and not _name.startswith("__"):
        setattr(Scene, _name, _fn)


def diff_params(sun_dir=(0.4, 0.3, -0.866), sun_color=3.0, albedo=0.7, w_depth=1.0,
                w_radiance=1.0, shadow_rays=True, shadow_offset=1e-3, recompute=False, layout=0):
    """rq_diff_params; layout 0 = the scene's BVH2, BVH8Q = trace the (refitted) BVH8."""
    sd = np.asarray(sun_dir, dtype=np.float64)
    sd = (sd / np.sqrt(sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2])).astype(np.float32)
    return L.RqDiffParams((C.c_float * 3)(*[float(x) for x in sd]), sun_color, albedo, w_depth,
                          w_radiance, int(shadow_rays), shadow_offset, int(recompute), int(layout), 0)


class Tape:
    """rq_tape: what rq_fwd saved for rq_bwd."""

    def __init__(self, scene, handle, rays):
        self.scene, self.handle, self.rays = scene, handle, rays

    def nbytes(self) -> int:
        b = C.c_int64()
        check(lib().rq_tape_bytes(self.handle, C.byref(b)))
        return b.value

    def backward(self, grad=None, stream=None):
        """dloss/dposition for every vertex as an (n_verts, 3) float32 device tensor."""
        import torch
        sc = self.scene
        if grad is None:
            grad = torch.empty((sc.n_verts, 3), dtype=torch.float32, device=self.rays.device)
        check(lib().rq_bwd(sc.ctx.handle, self.handle, ptr(grad), _stream(self.rays, stream)),
              sc.ctx.handle)
        return grad

    def close(self):
        if self.handle:
            lib().rq_tape_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _scene_forward(self, rays, target, params, image=None, want_loss=True, stream=None):
    """rq_fwd: returns (image (n, 2) device tensor, loss float or None, Tape)."""
    import torch
    n = rays.numel() * rays.element_size() // 32
    if image is None:
        image = torch.empty((n, 2), dtype=torch.float32, device=rays.device)
    loss = C.c_double(0.0)
    h = C.c_void_p()
    check(lib().rq_fwd(self.ctx.handle, self.handle, ptr(rays), n, ptr(target), C.byref(params),
                       ptr(image), C.byref(loss) if want_loss else None, C.byref(h),
                       _stream(rays, stream)), self.ctx.handle)
    return image, (loss.value if want_loss else None), Tape(self, h, rays)


def _scene_update_positions(self, xyz, stream=None):
    """rq_scene_update_positions: xyz is an (n_verts, 3) float32 device tensor; refits the BVH."""
    check(lib().rq_scene_update_positions(self.handle, ptr(xyz), _stream(xyz, stream)),
          self.ctx.handle)


Scene.forward = _scene_forward
Scene.update_positions = _scene_update_positions


def _queries(queries):
    """[(scene, device rays, kind, out)] -> ctypes array of rq_query (kind 0 closest, 1 any)."""
    arr = (L.RqQuery * len(queries))()
    for k, (sc, rays, kind, out) in enumerate(queries):
        n = rays.numel() * rays.element_size() // 32
        arr[k] = L.RqQuery(sc.handle, ptr(rays), n, kind, 0, ptr(out) if kind == 0 else None,
                           ptr(out) if kind == 1 else None)
    return arr


def batch(ctx: Context, queries, layout=0, mode=0, flags=0, block_size=0, min_blocks=0, stack_depth=0,
          stream=None):
    """rq_batch: every query in one persistent launch."""
    arr = _queries(queries)
    o = _opts(layout, mode, 0, flags, block_size, min_blocks, 0, stack_depth)
    st = stream
    if st is None and queries:
        st = _stream(queries[0][1], None)
    check(lib().rq_batch(ctx.handle, arr, len(queries), C.byref(o), st), ctx.handle)


class BatchPlan:
    """rq_batch_plan: a fixed batch replayed as a captured CUDA graph."""

    def __init__(self, ctx: Context, queries, layout=0, mode=0, flags=0):
        self.ctx = ctx
        self._keep = queries
        arr = _queries(queries)
        o = _opts(layout, mode, 0, flags)
        self.handle = C.c_void_p()
        check(lib().rq_batch_plan_create(ctx.handle, arr, len(queries), C.byref(o),
                                         C.byref(self.handle)), ctx.handle)

    def launch(self, stream=None):
        st = stream if stream is not None else _stream(self._keep[0][1], None)
        check(lib().rq_batch_plan_launch(self.handle, st), self.ctx.handle)

    def autotune(self, allow_bvh8=True) -> dict:
        r = L.RqBatchTune()
        check(lib().rq_batch_plan_autotune(self.handle, int(allow_bvh8), C.byref(r)), self.ctx.handle)
        combos = [dict(family=r.family_of[i], block=r.block_of[i], min_blocks=r.min_blocks_of[i],
                       stack_depth=r.depth_of[i], ms=round(r.ms[i], 4)) for i in range(r.n)]
        return dict(family=r.family, block_size=r.block_size, min_blocks=r.min_blocks, stack_depth=r.depth,
                    combos=combos)

    def close(self):
        if self.handle:
            lib().rq_batch_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RayIntersector:
    """Mirror of Candela::RayIntersector<T> (Intersector.h:60-451) over the C ABI.

    layout: STACK (RayIntersector<FlattenedStackNode>) or STACKLESS
    (RayIntersector<FlattenedNode>)."""

    def __init__(self, layout: int = STACK, leaf_size: int = 2, swap_children: bool = False,
                 swap_seed: int = 0):
        self.layout = layout
        self.leaf_size = leaf_size
        self.swap_children = swap_children
        self.swap_seed = swap_seed
        self.nodes = []          # m_BVHNodes
        self.vertices = []       # m_BVHVertices
        self.triangles = []      # m_BVHTriangles
        self._n_nodes = 0
        self._n_tris = 0
        self._index_offset = 0   # m_IndexOffset
        self.object_data = {}    # m_ObjectData: id -> (tri offset, vertex offset, node offset, count)
        self._pending = []       # m_Entities
        self.entities = np.zeros(0, dtype=ENTITY_DTYPE)  # m_BVHEntities
        self.scene: Scene | None = None

    def add_object(self, object_id: int, meshes) -> None:
        """AddObject (:169-198).  `meshes`: list of scenes.Mesh (merged like BuildBVH :981-1002:
        indices offset by the running vertex count, one mesh id per triangle)."""
        verts, idx, mids, off = [], [], [], 0
        for m in meshes:
            verts.append(m.vertices)
            idx.append(m.indices.astype(np.uint64) + off)
            mids.append(m.mesh_ids)
            off += m.vertices.shape[0]
        v = np.concatenate(verts)
        bvh = build_bvh(v, np.concatenate(idx).astype(np.uint32), np.concatenate(mids),
                        tri_offset=self._n_tris, layout=self.layout, leaf_size=self.leaf_size,
                        swap_children=self.swap_children, swap_seed=self.swap_seed)
        self.object_data[object_id] = (self._n_tris, sum(x.shape[0] for x in self.vertices),
                                       self._n_nodes, bvh.nodes.shape[0])
        tris = bvh.tris.copy()
        tris[:, :3] += self._index_offset
        self.vertices.append(v)
        self.nodes.append(bvh.nodes)
        self.triangles.append(tris)
        self._n_nodes += bvh.nodes.shape[0]
        self._n_tris += tris.shape[0]
        self._index_offset += v.shape[0]

    def push_entity(self, object_id: int, model=None, emissive: float = 0.0,
                    translucency: float = 0.0) -> None:
        """PushEntity (:200-216).  Raises like the reference when the object was never added."""
        if object_id not in self.object_data:
            raise KeyError("Trying to push entity whose parent object hasn't been added to global BVH")
        _, _, noff, ncount = self.object_data[object_id]
        self._pending.append(identity_entity(noff, ncount, emissive, 1.0 - translucency, model))

    def buffer_entities(self) -> None:
        """BufferEntities (:226-239)."""
        self.entities = (np.concatenate(self._pending) if self._pending
                         else np.zeros(0, dtype=ENTITY_DTYPE))
        self._pending = []
        if self.scene is not None:
            self.scene.set_entities(self.entities)

    def buffer_data(self, ctx: Context) -> Scene:
        """BufferData (:321-351): uploads the global buffers (and the current entities)."""
        self.scene = ctx.scene(self.layout, np.concatenate(self.vertices),
                               np.concatenate(self.triangles), np.concatenate(self.nodes),
                               self.entities)
        return self.scene

    def global_buffers(self):
        return (np.concatenate(self.vertices), np.concatenate(self.triangles),
                np.concatenate(self.nodes), self.entities)
