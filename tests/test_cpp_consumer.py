"""A C++ consumer of include/hrt.hpp and include/hrt.h: compiled with g++ against the headers and
linked to libhrt.so, it runs host-only calls on any machine and one frame on a GPU; the frame
equals the same scene traced through the Python binding, bit for bit, and meets the FP64 oracle."""
import os
import subprocess

import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import LSS, PHANTOM, OracleScene, compare_hits, lines_from_strands, oracle_geometry

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def consumer(tmp_path_factory):
    from vkhrt_gb300 import build as hb
    hb.build()
    out = str(tmp_path_factory.mktemp("cpp") / "consumer")
    libdir = os.path.join(ROOT, "vkhrt_gb300")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "consumer.cpp"), "-L" + libdir, "-lhrt", "-Wl,-rpath," + libdir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_consumer_host_calls(consumer):
    r = subprocess.run([consumer, "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)
    assert r.stdout.split() == ["host", "ok", "5bcfa8db0563635e"]  # the C1 strands' checksum


@pytest.mark.gpu
def test_cpp_consumer_frame_matches_python_and_oracle(consumer, tmp_path, ctx, orc):
    path = str(tmp_path / "frame.bin")
    r = subprocess.run([consumer, "gpu", path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr)
    raw = open(path, "rb").read()
    w, h = np.frombuffer(raw[:8], np.uint32)
    rgba = np.frombuffer(raw[8:8 + w * h * 16], np.float32).reshape(h, w, 4)
    hits = np.frombuffer(raw[8 + w * h * 16:], H.HIT_DTYPE)
    # the same scene through the Python binding
    blases, data = [], []
    for seed, gt, dx in ((501, PHANTOM, 0.0), (502, LSS, 0.35)):
        v, rr, off = H.generate_strands(H.StrandParams(seed=seed, nstrands=300, nverts=24))
        xf = np.eye(4, dtype=np.float32)
        xf[0, 3] = dx
        blases.append(H.BottomLevelAccelerationStructure(
            H.BLASInput(type=H.BLASType(gt), vertices=v, radius=rr, strand_offsets=off, transform=xf,
                        precision=H.Precision.QUANTISED), ctx))
        lines, lrad = lines_from_strands(v, rr, off)
        data.append(((gt, *oracle_geometry(orc, gt, lines, lrad)), xf))
    tlas = H.TopLevelAccelerationStructure(blases, ctx)
    cam = H.scene_camera(int(w), int(h))
    fr = H.Frame(ctx, int(w), int(h), 1, with_hits=True)
    H.trace(ctx, tlas, cam, fr, H.trace_params(shading=2, record_hits=1))
    p_rgba, p_hits = fr.download(hits=True)
    assert p_rgba.tobytes() == rgba.tobytes() and p_hits.tobytes() == hits.tobytes()
    osc = OracleScene(orc, [d for d, _ in data], [xf for _, xf in data])
    vi, pi = H.camera_arrays(cam)
    o = osc.render(vi, pi, int(w), int(h), shading=2, precision=64)
    st = compare_hits(np.where(hits["t"] >= 0, hits["t"].astype(np.float64), -1.0), hits["prim"], hits["inst"],
                      o["t"], o["prim"], o["inst"])
    assert st["hits"] > 500 and st["agreement"] >= 0.9999, st
    assert set(np.unique(hits["inst"][hits["t"] >= 0])) == {0, 1}
