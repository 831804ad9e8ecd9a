"""Builds vkhrt_gb300/libhrt.so (the C ABI of include/hrt.h) for sm_103a with nvcc.

Translation units compile in parallel:
  csrc/build.cu         --fmad=false (bit-exact BVH build)
  csrc/trace.cu         explicit-ray and no-allocation trace entry points
  csrc/trace_frames.cu  frame kernels, once each for FP32 nodes, 8-bit nodes and per-instance formats
  csrc/api.cu           C ABI (host code)
  csrc/workload.cpp     synthetic strands and camera matrices (host, -ffp-contract=off)

build(checked=True) makes libhrt_checked.so instead: the same sources with -DHRT_CHECKED, whose
kernels test every node, leaf-slot and stream index before loading and report HRT_ERR_BOUNDS.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhrt.so")
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(HERE, "libhrt_checked.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


# object name -> (source, extra flags); trace_frames.cu is compiled once per node layout
UNITS = {
    "build": ("build.cu", ["--fmad=false"]),
    "trace": ("trace.cu", []),
    "trace_frames_f": ("trace_frames.cu", ["-DHRT_FRAMES_QUANT=0"]),
    "trace_frames_q": ("trace_frames.cu", ["-DHRT_FRAMES_QUANT=1"]),
    "trace_frames_m": ("trace_frames.cu", ["-DHRT_FRAMES_QUANT=2"]),
    "api": ("api.cu", []),
    "workload": ("workload.cpp", ["-x", "c++", "-Xcompiler", "-ffp-contract=off"]),
}


def _deps() -> list[str]:
    out = [os.path.join(INCLUDE, "hrt.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def _compile(nvcc: str, name: str, src: str, extra: list[str], verbose: bool, build_dir: str = BUILD) -> str:
    obj = os.path.join(build_dir, name + ".o")
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-I" + INCLUDE, "-I" + CSRC,
           "-Xcompiler", "-fPIC", *extra, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    """Compile and link libhrt.so (or, checked, libhrt_checked.so) in-tree; a no-op when it is
    newer than its sources."""
    lib, build_dir = (LIB_CHECKED, BUILD_CHECKED) if checked else (LIB, BUILD)
    if not force and os.path.exists(lib):
        t = os.path.getmtime(lib)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return lib
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    flag = ["-DHRT_CHECKED"] if checked else []
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, nvcc, name, os.path.join(CSRC, f), extra + flag, verbose, build_dir)
                for name, (f, extra) in UNITS.items()]
        objs = [f.result() for f in futs]
    tmp = lib + ".tmp"
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
