"""oracle/build.py -- TEST INFRASTRUCTURE: builds the CPU oracle (and, where the reference
checkout is present, oracle/_ref). Used by __graft_entry__.build() and the test fixtures.

The oracle is test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg load it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libhrtoracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libhrtref.so")
ROOT = os.path.dirname(HERE)
# the workload generator (synthetic strands, camera matrices) is compiled from the GPU library's
# own host source, so that CPU-only runs trace exactly the same inputs without loading libhrt.so
WORKLOAD_SRC = os.path.join(ROOT, "vkhrt_gb300", "csrc", "workload.cpp")
SRC = [os.path.join(HERE, "hrt_oracle.cpp"), WORKLOAD_SRC]
DEPS = SRC + [os.path.join(HERE, "glsl_shim.hpp"), os.path.join(ROOT, "include", "hrt.h")]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, with_ref: bool = True) -> str:
    """Compile oracle/hrt_oracle.cpp (portable C++17, no FMA contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or _stale(LIB, DEPS):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-pthread", "-I" + HERE, "-I" + os.path.join(ROOT, "include")] + SRC + ["-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    if with_ref:
        ref_deps = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "glsl_shim.hpp"),
                    os.path.join(HERE, "build_ref.sh")]
        # the reference checkout: HRT_REFERENCE, else a `reference` directory beside the repository
        ref_root = os.environ.get("HRT_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
        if os.path.isdir(os.path.join(ref_root, "shaders")) and (force or _stale(REF_LIB, ref_deps)):
            subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True,
                           env=dict(os.environ, HRT_REFERENCE=ref_root))
    return LIB


_lib = None


def load() -> ctypes.CDLL:
    """Load the oracle library (building it if needed) with its argument types declared."""
    global _lib
    if _lib is not None:
        return _lib
    build(with_ref=False)
    lib = ctypes.CDLL(LIB)
    P = ctypes.c_void_p
    i64, i32, u32, f32, f64 = ctypes.c_int64, ctypes.c_int, ctypes.c_uint32, ctypes.c_float, ctypes.c_double
    sig = {
        "orc_prhi_f32": (f32, [P, P, f32, f32, P, P]),
        "orc_prhi_f64": (f64, [P, P, f64, f64, P, P]),
        "orc_cone_f32": (None, [P, P]),
        "orc_cylinder_f32": (i32, [P, P]),
        "orc_curve_sample_f32": (None, [P, f32, P]),
        "orc_rcc_matrix_f32": (None, [P, P]),
        "orc_shade_f32": (None, [P, P]),
        "orc_raygen_f32": (None, [P, P, u32, u32, u32, u32, f32, f32, P, P]),
        "orc_generate_curves": (None, [P, i64, P]),
        "orc_generate_aabbs": (None, [P, i64, f32, P]),
        "orc_generate_dots": (None, [P, P, f32, i64, P]),
        "orc_generate_lss": (None, [P, i64, f32, P, P]),
        "orc_strand_stream": (i64, [P, P, i64, P, P]),
        "orc_prim_boxes": (None, [i32, P, P, i64, P]),
        "orc_ref_boxes": (i64, [i32, P, P, i64, P]),
        "orc_morton": (None, [P, i64, P]),
        "orc_lbvh": (None, [P, i64, P, P, P, P, P, P, P, P, P]),
        "orc_bvh8": (i64, [P, i64, i32, i64, P, P, P, P, P, P, P, P, P]),
        "orc_voxelize": (i64, [P, i64, f32, f32, P, P, i64]),
        "orc_scene_create": (P, []),
        "orc_scene_destroy": (None, [P]),
        "orc_scene_add_blas": (i32, [P, i32, i64, P, P]),
        "orc_scene_add_instance": (i32, [P, i32, P]),
        "orc_scene_set_material": (i32, [P, i32, P, P, P, u32, u32]),
        "orc_trace_rays": (None, [P, P, i64, f32, f32, i32, i32, P, P, P, P]),
        "orc_render": (None, [P, P, P, u32, u32, u32, i32, u32, f32, f32, i32, f32, i32, i32, i64, i64,
                              P, P, P, P, P, P, P, u32, u32]),
        "orc_hardware_threads": (i32, []),
        "orc_resolve_stats": (None, [P, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def load_ref() -> ctypes.CDLL | None:
    """The reference's own code compiled here (None when oracle/_ref was not built)."""
    if not os.path.exists(REF_LIB):
        return None
    lib = ctypes.CDLL(REF_LIB)
    P = ctypes.c_void_p
    f32, i64, u32 = ctypes.c_float, ctypes.c_int64, ctypes.c_uint32
    lib.ref_prhi_f32.restype = f32
    lib.ref_prhi_f32.argtypes = [P, P, P]
    lib.ref_prhi_f64.restype = ctypes.c_double
    lib.ref_prhi_f64.argtypes = [P, P, P]
    lib.ref_cone_f32.argtypes = [P, P]
    lib.ref_cylinder_f32.restype = ctypes.c_int
    lib.ref_cylinder_f32.argtypes = [P, P]
    lib.ref_curve_sample_f32.argtypes = [P, f32, P]
    lib.ref_rcc_matrix_f32.argtypes = [P, P]
    lib.ref_shade_f32.argtypes = [P, P]
    lib.ref_raygen_f32.argtypes = [P, P, u32, u32, u32, u32, P, P]
    lib.ref_generate_curves.argtypes = [P, i64, P]
    lib.ref_generate_aabbs.argtypes = [P, i64, f32, P]
    lib.ref_generate_dots.argtypes = [P, i64, f32, P, P]
    lib.ref_generate_lss.argtypes = [P, i64, f32, P, P]
    return lib


if __name__ == "__main__":
    print(build(force=True))
