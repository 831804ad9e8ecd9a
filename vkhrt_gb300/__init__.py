"""vkhrt_gb300 -- GB300 hair ray tracer: Python host mirror of the C ABI in include/hrt.h.

The classes mirror the reference's (mmzala/vkhrt) acceleration-structure interface:
  BottomLevelAccelerationStructure(BLASInput, context)   include/bottom_level_acceleration_structure.hpp:34
      .Structure() .Type() .Transform()                   (hpp:40-42)
  TopLevelAccelerationStructure([blas, ...], context)     include/top_level_acceleration_structure.hpp:12
  Renderer-style tracing: Context.trace(tlas, camera, ...) (source/renderer.cpp:83-166)
Errors raise HrtError (the reference logs and aborts, vk_common.cpp:5-15).

All work runs in libhrt.so (CUDA kernels for sm_103a); there is no CPU fallback: loading fails
loudly if the library cannot be built or loaded.
"""
from __future__ import annotations

import ctypes
import enum
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhrt.so")

# ------------------------------------------------------------------------------------ C types
c_f, c_u32, c_i32, c_u64, c_p = ctypes.c_float, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p


ABI_VERSION = 10  # HRT_ABI_VERSION of include/hrt.h that the structures below mirror


class BLASInputC(ctypes.Structure):
    _fields_ = [("type", c_i32), ("precision", c_i32), ("memory", c_i32), ("max_leaf", c_u32),
                ("vertices", c_p), ("radius", c_p), ("strand_offsets", c_p), ("line_indices", c_p),
                ("nvertices", c_u64), ("nstrands", c_u64), ("nlines", c_u64), ("const_radius", c_f),
                ("transform", c_f * 16), ("width", c_u32), ("flags", c_u32), ("tri_indices", c_p),
                ("ntris", c_u64), ("normals", c_p), ("voxel_size", c_f), ("texcoords", c_p),
                ("albedo_factor", c_f * 4), ("albedo_map", c_p), ("albedo_map_width", c_u32),
                ("albedo_map_height", c_u32)]


class BLASInfoC(ctypes.Structure):
    _fields_ = [("nprims", c_u64), ("nnodes", c_u64), ("node_bytes", c_u64), ("prim_bytes", c_u64),
                ("device_bytes", c_u64), ("bounds", c_f * 6), ("build_ms", c_f)]


class CameraC(ctypes.Structure):
    _fields_ = [("view_inverse", c_f * 16), ("proj_inverse", c_f * 16)]


class TraceParamsC(ctypes.Structure):
    _fields_ = [("tmin", c_f), ("tmax", c_f), ("spp", c_u32), ("jitter", c_u32), ("seed", c_u32),
                ("shading", c_u32), ("shadow_tmin", c_f), ("fp64_resolve", c_u32), ("record_hits", c_u32),
                ("async_", c_u32), ("count_stats", c_u32), ("kernel_variant", c_u32), ("refill", c_u32),
                ("speculative", c_u32), ("split_types", c_u32), ("env_map", c_p), ("env_width", c_u32),
                ("env_height", c_u32), ("leaf_again", c_u32), ("max_steps", c_u32), ("max_depth", c_u32),
                ("variant_by_type", c_u32)]


class FrameStatsC(ctypes.Structure):
    _fields_ = [("primary_rays", c_u64), ("shadow_rays", c_u64), ("nodes_visited", c_u64),
                ("prims_tested", c_u64), ("fp64_resolves", c_u64), ("fp64_hits", c_u64),
                ("warp_cycles_node", c_u64), ("warp_cycles_leaf", c_u64), ("warp_cycles_other", c_u64)]


class SceneDescC(ctypes.Structure):
    _fields_ = [("tlas", c_p), ("camera", CameraC), ("frame", c_p)]


class StrandParamsC(ctypes.Structure):
    _fields_ = [("seed", c_u64), ("nstrands", c_u32), ("nverts", c_u32), ("step", c_f), ("droop", c_f),
                ("curl", c_f), ("curl_freq", c_f), ("r_root", c_f), ("r_tip", c_f), ("cap_deg", c_f)]


HIT_DTYPE = np.dtype([("t", np.float32), ("prim", np.uint32), ("inst", np.uint32), ("flags", np.uint32)])
HIT_SHADOWED, HIT_FP64 = 1, 2

# the public symbols of include/hrt.h: (restype, argtypes)
SIGNATURES = {
    "hrt_abi_version": (c_i32, []),
    "hrt_status_string": (ctypes.c_char_p, [c_i32]),
    "hrt_context_create": (c_i32, [c_i32, ctypes.POINTER(c_p)]),
    "hrt_context_destroy": (c_i32, [c_p]),
    "hrt_last_error": (ctypes.c_char_p, [c_p]),
    "hrt_blas_input_default": (None, [ctypes.POINTER(BLASInputC)]),
    "hrt_blas_build": (c_i32, [c_p, ctypes.POINTER(BLASInputC), c_p, ctypes.POINTER(c_p)]),
    "hrt_blas_destroy": (c_i32, [c_p]),
    "hrt_blas_refit": (c_i32, [c_p, c_p, c_p, c_i32, c_p]),
    "hrt_blas_serialized_size": (c_u64, [c_p]),
    "hrt_blas_serialize": (c_i32, [c_p, c_p, c_u64]),
    "hrt_blas_deserialize": (c_i32, [c_p, c_p, c_u64, c_p, ctypes.POINTER(c_p)]),
    "hrt_blas_type": (c_i32, [c_p]),
    "hrt_blas_transform": (c_i32, [c_p, c_p]),
    "hrt_blas_get_info": (c_i32, [c_p, ctypes.POINTER(BLASInfoC)]),
    "hrt_blas_get": (c_i32, [c_p, c_i32, c_p, c_u64]),
    "hrt_tlas_build": (c_i32, [c_p, ctypes.POINTER(c_p), c_u32, c_p, ctypes.POINTER(c_p)]),
    "hrt_tlas_destroy": (c_i32, [c_p]),
    "hrt_camera_look_at": (c_i32, [c_p, c_p, c_p, c_f, c_f, c_f, c_f, ctypes.POINTER(CameraC)]),
    "hrt_trace_params_default": (None, [ctypes.POINTER(TraceParamsC)]),
    "hrt_frame_create": (c_i32, [c_p, c_u32, c_u32, c_u32, c_i32, ctypes.POINTER(c_p)]),
    "hrt_frame_destroy": (c_i32, [c_p]),
    "hrt_frame_device_ptrs": (c_i32, [c_p, ctypes.POINTER(c_p), ctypes.POINTER(c_p)]),
    "hrt_frame_download": (c_i32, [c_p, c_p, c_p, c_p]),
    "hrt_frame_get_stats": (c_i32, [c_p, ctypes.POINTER(FrameStatsC)]),
    "hrt_trace": (c_i32, [c_p, c_p, ctypes.POINTER(CameraC), ctypes.POINTER(TraceParamsC), c_p, c_p]),
    "hrt_trace_rays": (c_i32, [c_p, c_p, c_p, c_u64, ctypes.POINTER(TraceParamsC), c_p, c_i32, c_p]),
    "hrt_trace_rays_noalloc": (c_i32, [c_p, c_p, c_p, c_u64, ctypes.POINTER(TraceParamsC), c_p, c_p]),
    "hrt_batch_create": (c_i32, [c_p, ctypes.POINTER(SceneDescC), c_u32, ctypes.POINTER(TraceParamsC), c_p,
                                 ctypes.POINTER(c_p)]),
    "hrt_batch_launch": (c_i32, [c_p, c_p]),
    "hrt_autotune": (c_i32, [c_p, ctypes.POINTER(SceneDescC), c_u32, ctypes.POINTER(TraceParamsC), c_u32, c_p,
                             ctypes.POINTER(TraceParamsC), ctypes.POINTER(c_f)]),
    "hrt_batch_destroy": (c_i32, [c_p]),
    "hrt_batch_set_cameras": (c_i32, [c_p, ctypes.POINTER(CameraC), c_u32, c_p]),
    "hrt_batch_table_bytes": (c_u64, [c_p]),
    "hrt_batch_download": (c_i32, [c_p, c_p, c_p, c_i32]),
    "hrt_strand_params_default": (None, [ctypes.POINTER(StrandParamsC)]),
    "hrt_generate_strands": (c_i32, [ctypes.POINTER(StrandParamsC), c_p, c_p, c_p]),
    "hrt_checksum": (c_u64, [c_p, c_u64, c_p, c_u64]),
}

_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libhrt.so (building it with nvcc if it is missing or stale). The environment
    variable HRT_LIBRARY names another build of the same library to load instead."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("HRT_LIBRARY") or LIB_PATH
    if build_if_missing and path == LIB_PATH:
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: the CUDA library must be built (vkhrt_gb300.build.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.hrt_abi_version() != ABI_VERSION:  # the structures below follow this version of hrt.h
        raise RuntimeError(f"{path} implements ABI {lib.hrt_abi_version()}, this binding ABI {ABI_VERSION}")
    _lib = lib
    return lib


class HrtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hrt status {status}: {message}")
        self.status = status


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(c_p)


class BLASType(enum.IntEnum):
    """Intersector of a BLAS (the reference's BLASType and LSS geometry flag)."""
    ePhantom = 0   # cubic Bezier curves, Phantom ray-hair intersector (BLASType::eHair)
    eLSS = 1       # linear swept spheres (BLASType::eMesh with LSS geometry)
    eDOTS = 2      # disjoint orthogonal triangle strips (BLASType::eMesh triangles)
    eMesh = 3      # indexed triangle mesh (BLASType::eMesh), optional vertex normals
    eVoxels = 4    # strands voxelised as capsules into box primitives (BLASType::eVoxels)


class Precision(enum.IntEnum):
    FP32 = 0
    QUANTISED = 1


class Shading(enum.IntEnum):
    DEBUG = 0
    LAMBERT = 1
    LAMBERT_SHADOW = 2


class Part(enum.IntEnum):
    PRIM_BOXES = 0
    MORTON_SORTED = 1
    SORTED_INDEX = 2
    BIN_LEFT = 3
    BIN_RIGHT = 4
    BIN_BOXES = 5
    NODES = 6
    PRIM_ORDER = 7
    PRIMS = 8
    CURVES = 9
    DOTS_VERTICES = 10
    LSS = 11
    QNODES = 12
    STRAND_VERTICES = 13
    TRI_TEXCOORDS = 14


@dataclass
class BLASInput:
    """Geometry of one BLAS (hrt_blas_input): hair (strand_offsets or line_indices) or, for
    BLASType.eMesh, indexed triangles (tri_indices, optional per-vertex normals) and a material
    (albedo_factor, and albedo_map sampled at texcoords; the Lambert shading modes multiply by the
    albedo). BLASType.eVoxels voxelises the strands' lines as capsules of radius const_radius on
    cubes of voxel_size (0 = 0.1); each filled voxel reports its grid index as primitive id."""
    type: BLASType
    vertices: np.ndarray                      # (nv, 3) float32
    radius: np.ndarray | None = None          # (nv,) float32 per vertex
    strand_offsets: np.ndarray | None = None  # (ns + 1,) uint32
    line_indices: np.ndarray | None = None    # (nl, 2) uint32
    tri_indices: np.ndarray | None = None     # (nt, 3) uint32 (mesh)
    normals: np.ndarray | None = None         # (nv, 3) float32 (mesh)
    const_radius: float = 0.02
    transform: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))  # object->world
    precision: Precision = Precision.FP32
    max_leaf: int = 1
    width: int = 0                            # BVH node fan-out 2..8 (0 = 8)
    keep_intermediate: bool = False
    voxel_size: float = 0.0
    texcoords: np.ndarray | None = None       # (nv, 2) float32 (mesh)
    albedo_factor: tuple = (1.0, 1.0, 1.0, 1.0)
    albedo_map: np.ndarray | None = None      # (h, w, 4) float32 RGBA, row 0 at v = 0 (mesh)


class Context:
    """A device context (hrt_context)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = c_p()
        st = self.lib.hrt_context_create(device, ctypes.byref(h))
        if st != 0:
            raise HrtError(st, f"hrt_context_create({device}) failed: {self.lib.hrt_status_string(st).decode()}")
        self.handle = h

    def check(self, st: int):
        if st != 0:
            raise HrtError(st, self.lib.hrt_last_error(self.handle).decode())

    def close(self):
        if self.handle:
            self.lib.hrt_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BottomLevelAccelerationStructure:
    """hrt_blas: geometry processing + BVH8 build for one hair model."""

    def __init__(self, inp: BLASInput, ctx: Context, stream: int | None = None):
        self.ctx = ctx
        lib = ctx.lib
        c = BLASInputC()
        lib.hrt_blas_input_default(ctypes.byref(c))
        self._keep = []
        v = np.ascontiguousarray(inp.vertices, dtype=np.float32).reshape(-1, 3)
        self._keep.append(v)
        c.type = int(inp.type)
        c.precision = int(inp.precision)
        c.memory = 0
        c.max_leaf = inp.max_leaf
        c.width = inp.width
        c.voxel_size = inp.voxel_size
        c.vertices = _ptr(v)
        c.nvertices = v.shape[0]
        if inp.radius is not None:
            r = np.ascontiguousarray(inp.radius, dtype=np.float32).reshape(-1)
            self._keep.append(r)
            c.radius = _ptr(r)
        if inp.strand_offsets is not None:
            so = np.ascontiguousarray(inp.strand_offsets, dtype=np.uint32).reshape(-1)
            self._keep.append(so)
            c.strand_offsets = _ptr(so)
            c.nstrands = so.shape[0] - 1
        if inp.line_indices is not None:
            li = np.ascontiguousarray(inp.line_indices, dtype=np.uint32).reshape(-1, 2)
            self._keep.append(li)
            c.line_indices = _ptr(li)
            c.nlines = li.shape[0]
        if inp.tri_indices is not None:
            ti = np.ascontiguousarray(inp.tri_indices, dtype=np.uint32).reshape(-1, 3)
            self._keep.append(ti)
            c.tri_indices = _ptr(ti)
            c.ntris = ti.shape[0]
        if inp.normals is not None:
            nm = np.ascontiguousarray(inp.normals, dtype=np.float32).reshape(-1, 3)
            self._keep.append(nm)
            c.normals = _ptr(nm)
        if inp.texcoords is not None:
            tc = np.ascontiguousarray(inp.texcoords, dtype=np.float32).reshape(-1, 2)
            self._keep.append(tc)
            c.texcoords = _ptr(tc)
        for k in range(4):
            c.albedo_factor[k] = float(inp.albedo_factor[k])
        if inp.albedo_map is not None:
            am = np.ascontiguousarray(inp.albedo_map, dtype=np.float32)
            if am.ndim != 3 or am.shape[2] != 4:
                raise ValueError("albedo_map must be (height, width, 4)")
            self._keep.append(am)
            c.albedo_map = _ptr(am)
            c.albedo_map_height, c.albedo_map_width = am.shape[0], am.shape[1]
        c.const_radius = inp.const_radius
        xf = np.asarray(inp.transform, dtype=np.float32).reshape(4, 4)
        for i, val in enumerate(xf.T.reshape(-1)):  # column major
            c.transform[i] = float(val)
        c.flags = 1 if inp.keep_intermediate else 0
        h = c_p()
        ctx.check(lib.hrt_blas_build(ctx.handle, ctypes.byref(c), c_p(stream) if stream else None, ctypes.byref(h)))
        self.handle = h
        self._keep = []
        info = BLASInfoC()
        ctx.check(lib.hrt_blas_get_info(self.handle, ctypes.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in BLASInfoC._fields_}
        self.info["bounds"] = list(info.bounds)

    def Structure(self):
        return self.handle

    def serialize(self) -> bytes:
        """hrt_blas_serialize: the BLAS as bytes (load with BottomLevelAccelerationStructure.load)."""
        n = int(self.ctx.lib.hrt_blas_serialized_size(self.handle))
        buf = np.zeros(n, np.uint8)
        self.ctx.check(self.ctx.lib.hrt_blas_serialize(self.handle, _ptr(buf), n))
        return buf.tobytes()

    @classmethod
    def load(cls, data: bytes, ctx: Context, stream: int | None = None) -> "BottomLevelAccelerationStructure":
        """hrt_blas_deserialize: a BLAS from serialize()'s bytes (validated before use)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self._keep = []
        buf = np.frombuffer(data, np.uint8)
        h = c_p()
        ctx.check(ctx.lib.hrt_blas_deserialize(ctx.handle, _ptr(buf), len(buf), c_p(stream) if stream else None,
                                               ctypes.byref(h)))
        self.handle = h
        info = BLASInfoC()
        ctx.check(ctx.lib.hrt_blas_get_info(h, ctypes.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in BLASInfoC._fields_}
        self.info["bounds"] = list(info.bounds)
        return self

    def refit(self, vertices: np.ndarray, per_vertex: np.ndarray | None = None, stream: int | None = None):
        """hrt_blas_refit: new vertex positions (and radii or normals when the build had them)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32)
        pv = None if per_vertex is None else np.ascontiguousarray(per_vertex, dtype=np.float32)
        self.ctx.check(self.ctx.lib.hrt_blas_refit(self.handle, _ptr(v), _ptr(pv), 0, c_p(stream) if stream else None))
        info = BLASInfoC()
        self.ctx.check(self.ctx.lib.hrt_blas_get_info(self.handle, ctypes.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in BLASInfoC._fields_}
        self.info["bounds"] = list(info.bounds)

    def Type(self) -> BLASType:
        return BLASType(self.ctx.lib.hrt_blas_type(self.handle))

    def Transform(self) -> np.ndarray:
        out = np.zeros(16, np.float32)
        self.ctx.check(self.ctx.lib.hrt_blas_transform(self.handle, _ptr(out)))
        return out.reshape(4, 4).T.copy()  # back to row-major numpy

    def get(self, part: Part, dtype, shape) -> np.ndarray:
        out = np.zeros(shape, dtype)
        self.ctx.check(self.ctx.lib.hrt_blas_get(self.handle, int(part), _ptr(out), out.nbytes))
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.hrt_blas_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TopLevelAccelerationStructure:
    """hrt_tlas: instance i = blases[i] with its transform and custom index i."""

    def __init__(self, blases: list[BottomLevelAccelerationStructure], ctx: Context):
        self.ctx = ctx
        self.blases = list(blases)
        arr = (c_p * len(blases))(*[b.handle for b in blases])
        h = c_p()
        ctx.check(ctx.lib.hrt_tlas_build(ctx.handle, arr, len(blases), None, ctypes.byref(h)))
        self.handle = h

    def Structure(self):
        return self.handle

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.hrt_tlas_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# The workload generator (synthetic strands, camera matrices) is host code that the CPU oracle's
# library compiles too; `lib` selects which library runs it (default libhrt.so).
WORKLOAD_SYMBOLS = ("hrt_camera_look_at", "hrt_strand_params_default", "hrt_generate_strands", "hrt_checksum")


def bind_workload(lib: ctypes.CDLL) -> ctypes.CDLL:
    """Declares the workload generator's symbols on a library that exports them."""
    for name in WORKLOAD_SYMBOLS:
        res, args = SIGNATURES[name]
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def look_at(eye, center, up, fovy_deg: float, aspect: float, znear: float = 0.1, zfar: float = 1000.0,
            lib: ctypes.CDLL | None = None) -> CameraC:
    lib = lib or load()
    cam = CameraC()
    e = np.asarray(eye, np.float32)
    c = np.asarray(center, np.float32)
    u = np.asarray(up, np.float32)
    st = lib.hrt_camera_look_at(_ptr(e), _ptr(c), _ptr(u), fovy_deg, aspect, znear, zfar, ctypes.byref(cam))
    if st != 0:
        raise HrtError(st, "hrt_camera_look_at: invalid camera")
    return cam


def camera_arrays(cam: CameraC) -> tuple[np.ndarray, np.ndarray]:
    return (np.ctypeslib.as_array(cam.view_inverse).copy(), np.ctypeslib.as_array(cam.proj_inverse).copy())


def trace_params(**kw) -> TraceParamsC:
    p = TraceParamsC()
    load().hrt_trace_params_default(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, "async_" if k == "async" else k, v)
    return p


class Frame:
    """hrt_frame: device RGBA32F framebuffer (+ per-sample hit records)."""

    def __init__(self, ctx: Context, width: int, height: int, spp: int = 1, with_hits: bool = False):
        self.ctx = ctx
        self.width, self.height, self.spp = width, height, spp
        h = c_p()
        ctx.check(ctx.lib.hrt_frame_create(ctx.handle, width, height, spp, 1 if with_hits else 0, ctypes.byref(h)))
        self.handle = h
        self.with_hits = with_hits

    def download(self, hits: bool = False):
        rgba = np.zeros((self.height, self.width, 4), np.float32)
        hh = np.zeros(self.height * self.width * self.spp, HIT_DTYPE) if hits else None
        self.ctx.check(self.ctx.lib.hrt_frame_download(self.handle, _ptr(rgba), _ptr(hh), None))
        return (rgba, hh) if hits else rgba

    def stats(self) -> dict:
        s = FrameStatsC()
        self.ctx.check(self.ctx.lib.hrt_frame_get_stats(self.handle, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in FrameStatsC._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.hrt_frame_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def trace(ctx: Context, tlas: TopLevelAccelerationStructure, cam: CameraC, frame: Frame,
          params: TraceParamsC | None = None, stream: int | None = None):
    p = params if params is not None else trace_params()
    ctx.check(ctx.lib.hrt_trace(ctx.handle, tlas.handle, ctypes.byref(cam), ctypes.byref(p), frame.handle,
                                c_p(stream) if stream else None))


def trace_rays(ctx: Context, tlas: TopLevelAccelerationStructure, rays: np.ndarray,
               params: TraceParamsC | None = None, stream: int | None = None) -> np.ndarray:
    """Closest hit for explicit rays (n, 6) float32 = origin xyz, direction xyz."""
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    hits = np.zeros(r.shape[0], HIT_DTYPE)
    p = params if params is not None else trace_params()
    ctx.check(ctx.lib.hrt_trace_rays(ctx.handle, tlas.handle, _ptr(r), r.shape[0], ctypes.byref(p), _ptr(hits), 0,
                                     c_p(stream) if stream else None))
    return hits


NOALLOC_MAX_RAYS = 65536


def trace_rays_noalloc(ctx: Context, tlas: TopLevelAccelerationStructure, rays: np.ndarray,
                       params: TraceParamsC | None = None, stream: int | None = None) -> np.ndarray:
    """hrt_trace_rays_noalloc: closest hit for at most NOALLOC_MAX_RAYS host rays without any
    device allocation (for callers that cannot call cudaMalloc/cudaFree; see include/hrt.h)."""
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    hits = np.zeros(r.shape[0], HIT_DTYPE)
    p = params if params is not None else trace_params()
    ctx.check(ctx.lib.hrt_trace_rays_noalloc(ctx.handle, tlas.handle, _ptr(r), r.shape[0], ctypes.byref(p), _ptr(hits),
                                             c_p(stream) if stream else None))
    return hits


TUNED_FIELDS = ("kernel_variant", "refill", "speculative", "split_types", "leaf_again", "variant_by_type")


def autotune(ctx: Context, scenes: list[tuple[TopLevelAccelerationStructure, CameraC, Frame]],
             params: TraceParamsC | None = None, reps: int = 3, cache: str | None = None,
             key: str | None = None) -> tuple[TraceParamsC, float]:
    """hrt_autotune on `scenes`; with `cache` (a JSON file) and `key`, a stored choice is reused
    and a new one is stored. Returns (parameters, mean frame ms of the choice, the stored one when
    cached, or -1 when the cache holds none)."""
    import json
    base = params if params is not None else trace_params()
    if cache and key and os.path.exists(cache):
        try:
            stored = json.load(open(cache)).get(key)
        except (OSError, ValueError):
            stored = None
        if stored:
            best = TraceParamsC.from_buffer_copy(base)
            for f in TUNED_FIELDS:
                setattr(best, f, int(stored.get(f, getattr(base, f))))
            return best, float(stored.get("ms", -1.0))
    descs = (SceneDescC * len(scenes))()
    for i, (t, cam, fr) in enumerate(scenes):
        descs[i].tlas = t.handle
        descs[i].camera = cam
        descs[i].frame = fr.handle
    best = TraceParamsC()
    ms = c_f()
    ctx.check(ctx.lib.hrt_autotune(ctx.handle, descs, len(scenes), ctypes.byref(base), reps, None, ctypes.byref(best),
                                   ctypes.byref(ms)))
    if cache and key:
        try:
            data = json.load(open(cache)) if os.path.exists(cache) else {}
        except (OSError, ValueError):
            data = {}
        data[key] = {f: int(getattr(best, f)) for f in TUNED_FIELDS} | {"ms": round(float(ms.value), 4)}
        with open(cache, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
    return best, float(ms.value)


class Batch:
    """hrt_batch: many scenes in one persistent launch replayed from a CUDA graph."""

    def __init__(self, ctx: Context, scenes: list[tuple[TopLevelAccelerationStructure, CameraC, Frame]],
                 params: TraceParamsC | None = None):
        self.ctx = ctx
        self.scenes = scenes
        descs = (SceneDescC * len(scenes))()
        for i, (t, cam, fr) in enumerate(scenes):
            descs[i].tlas = t.handle
            descs[i].camera = cam
            descs[i].frame = fr.handle
        p = params if params is not None else trace_params()
        h = c_p()
        ctx.check(ctx.lib.hrt_batch_create(ctx.handle, descs, len(scenes), ctypes.byref(p), None, ctypes.byref(h)))
        self.handle = h

    def launch(self, stream: int | None = None):
        self.ctx.check(self.ctx.lib.hrt_batch_launch(self.handle, c_p(stream) if stream else None))

    def set_cameras(self, cams: list[CameraC], stream: int | None = None):
        arr = (CameraC * len(cams))(*cams)
        self.ctx.check(self.ctx.lib.hrt_batch_set_cameras(self.handle, arr, len(cams), c_p(stream) if stream else None))

    @property
    def table_bytes(self) -> int:
        return int(self.ctx.lib.hrt_batch_table_bytes(self.handle))

    def download(self, dst: list, stream: int | None = None, synchronise: bool = True):
        """Every scene's framebuffer into dst[i] (host arrays or pinned tensors of height x width x 4
        float32, or None to skip), enqueued on `stream`; one synchronisation when `synchronise`."""
        def addr(d):
            if d is None:
                return None
            if hasattr(d, "data_ptr"):  # a (pinned) torch tensor
                return d.data_ptr()
            a = np.asarray(d)
            if a.dtype != np.float32 or not a.flags.c_contiguous:
                raise ValueError("download destinations must be C-contiguous float32")
            return a.ctypes.data
        if len(dst) != len(self.scenes):
            raise ValueError(f"need one destination per scene ({len(self.scenes)})")
        ptrs = (c_p * len(dst))(*[addr(d) for d in dst])
        self.ctx.check(self.ctx.lib.hrt_batch_download(self.handle, ptrs, c_p(stream) if stream else None,
                                                       1 if synchronise else 0))

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.hrt_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class StrandParams:
    seed: int = 1001
    nstrands: int = 2000
    nverts: int = 32
    step: float = 0.05
    droop: float = 0.02
    curl: float = 0.01
    curl_freq: float = 0.7
    r_root: float = 0.004
    r_tip: float = 0.001
    cap_deg: float = 60.0


def generate_strands(p: StrandParams, lib: ctypes.CDLL | None = None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Seeded synthetic strands: (vertices (nv,3), radius (nv,), strand_offsets (ns+1,))."""
    lib = lib or load()
    c = StrandParamsC()
    for k, _ in StrandParamsC._fields_:
        setattr(c, k, getattr(p, k))
    nv = p.nstrands * p.nverts
    v = np.zeros((nv, 3), np.float32)
    r = np.zeros(nv, np.float32)
    o = np.zeros(p.nstrands + 1, np.uint32)
    st = lib.hrt_generate_strands(ctypes.byref(c), _ptr(v), _ptr(r), _ptr(o))
    if st != 0:
        raise HrtError(st, "hrt_generate_strands: invalid parameters")
    return v, r, o


def checksum(*arrays: np.ndarray, lib: ctypes.CDLL | None = None) -> int:
    lib = lib or load()
    a = np.ascontiguousarray(arrays[0])
    b = np.ascontiguousarray(arrays[1]) if len(arrays) > 1 else None
    return int(lib.hrt_checksum(_ptr(a), a.nbytes, _ptr(b), 0 if b is None else b.nbytes))


# Workloads of the benchmark configurations (strands x vertices, radius taper, image, spp).
CONFIGS = {
    "c1_phantom_fp32": dict(seed=1001, nstrands=2000, nverts=32, r_root=0.004, r_tip=0.001, type=BLASType.ePhantom,
                            precision=Precision.FP32, width=512, height=512, spp=1),
    "c2_lss_fp32": dict(seed=1002, nstrands=50000, nverts=64, r_root=0.003, r_tip=0.0008, type=BLASType.eLSS,
                        precision=Precision.FP32, width=1920, height=1080, spp=1),
    "c3_dots_fp32": dict(seed=1003, nstrands=50000, nverts=64, r_root=0.003, r_tip=0.0008, type=BLASType.eDOTS,
                         precision=Precision.FP32, width=1920, height=1080, spp=1),
    "c4_phantom_quantised": dict(seed=1004, nstrands=150000, nverts=128, r_root=0.003, r_tip=0.0008,
                                 type=BLASType.ePhantom, precision=Precision.QUANTISED, width=1920, height=1080, spp=4),
}


def scene_camera(width: int, height: int, lib: ctypes.CDLL | None = None) -> CameraC:
    """Camera of the benchmark scenes: eye (0,0,3) looking at the origin, +y up, 40 deg FOV."""
    return look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, width / height, 0.1, 1000.0, lib)


def orbit_camera(width: int, height: int, azimuth: float, elevation: float, dist: float = 3.0,
                 lib: ctypes.CDLL | None = None) -> CameraC:
    """scene_camera moved on the sphere of radius `dist` (angles in radians, azimuth 0 = +z)."""
    import math
    eye = (dist * math.cos(elevation) * math.sin(azimuth), dist * math.sin(elevation),
           dist * math.cos(elevation) * math.cos(azimuth))
    return look_at(eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, width / height, 0.1, 1000.0, lib)


def batch_workload(seed: int = 1005, nscenes: int = 16) -> list[dict]:
    """The batched multi-scene workload: `nscenes` hair models with strand counts log-uniform in
    [2,000, 200,000], vertices per strand uniform in {16, 32, 64, 128}, intersector modes in turn
    Phantom, LSS, DOTS; each with its own orbit camera, a resolution log-uniform from 256x256 to
    1920x1080 (width and height at the same fraction) and 1-4 samples per pixel."""
    import math
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nscenes):
        ns = int(round(math.exp(rng.uniform(math.log(2000.0), math.log(200000.0)))))
        nv = int(rng.choice([16, 32, 64, 128]))
        f = float(rng.uniform())
        w = int(round(256 * (1920 / 256) ** f))
        h = int(round(256 * (1080 / 256) ** f))
        spp = int(rng.integers(1, 5))
        az = float(rng.uniform(0.0, 2.0 * math.pi))
        el = float(rng.uniform(-0.2, 0.6))
        out.append(dict(seed=seed * 1000 + i, nstrands=ns, nverts=nv, r_root=0.003, r_tip=0.0008,
                        type=BLASType(i % 3), width=w, height=h, spp=spp, azimuth=az, elevation=el))
    return out
