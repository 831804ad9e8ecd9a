"""The checked build (libhrt_checked.so, -DHRT_CHECKED): every node index, leaf slot, strand-stream
entry and TLAS leaf is tested against its array before the loads that use it; a failed test stops
the ray and the launch returns HRT_ERR_BOUNDS.

* On valid scenes the checked build renders and traces exactly what the normal build does.
* Its test hook HRT_CHECKED_NODE_LIMIT makes a TLAS report fewer nodes per BLAS than the BLAS
  holds, so traversal meets node indices past the reported count: the check fires there, while
  the loads it prevents would still have been inside the real array (nothing can fault). The
  context stays usable and a TLAS built without the hook traces normally.

Each build runs in its own process (the library is chosen by HRT_LIBRARY at load).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import os, sys
import numpy as np
sys.path.insert(0, os.environ["HRT_ROOT"])
sys.path.insert(0, os.path.join(os.environ["HRT_ROOT"], "tests"))
import vkhrt_gb300 as H
from hairscene import aimed_rays, lines_from_strands
out, mode = sys.argv[1], sys.argv[2]
ctx = H.Context(0)
blases, lines_all = [], []
for k, (gt, prec) in enumerate([(H.BLASType.ePhantom, H.Precision.QUANTISED), (H.BLASType.eLSS, H.Precision.FP32)]):
    v, r, off = H.generate_strands(H.StrandParams(seed=700 + k, nstrands=500, nverts=20))
    xf = np.eye(4, dtype=np.float32)
    xf[0, 3] = 0.3 * k
    blases.append(H.BottomLevelAccelerationStructure(
        H.BLASInput(type=gt, vertices=v, radius=r, strand_offsets=off, precision=prec, transform=xf), ctx))
    ln, _ = lines_from_strands(v, r, off)
    ln = ln.reshape(-1, 3).copy(); ln[:, 0] += 0.3 * k
    lines_all.append(ln.reshape(-1, 6))
rays = aimed_rays(np.random.default_rng(5), np.concatenate(lines_all), 4000, spread=0.006)
cam = H.scene_camera(96, 64)
res = {}
def run(tag, tlas):
    try:
        fr = H.Frame(ctx, 96, 64, 2, with_hits=True)
        H.trace(ctx, tlas, cam, fr, H.trace_params(shading=2, spp=2, jitter=1, seed=3, record_hits=1))
        rgba, hits = fr.download(hits=True)
        res[tag + "_rgba"], res[tag + "_hits"] = rgba, hits.view(np.uint32)
        res[tag + "_frame_status"] = np.array(0)
    except H.HrtError as e:
        res[tag + "_frame_status"] = np.array(e.status)
    try:
        g = H.trace_rays(ctx, tlas, rays)
        res[tag + "_rays"] = np.stack([g["t"].view(np.uint32), g["prim"], g["inst"]])
        res[tag + "_rays_status"] = np.array(0)
    except H.HrtError as e:
        res[tag + "_rays_status"] = np.array(e.status)
if mode == "limit":
    os.environ["HRT_CHECKED_NODE_LIMIT"] = "6"
    run("limited", H.TopLevelAccelerationStructure(blases, ctx))
    del os.environ["HRT_CHECKED_NODE_LIMIT"]
    run("single", H.TopLevelAccelerationStructure(blases[:1], ctx))
run("plain", H.TopLevelAccelerationStructure(blases, ctx))
np.savez(out, **res)
'''


@pytest.fixture(scope="module")
def checked_lib():
    from vkhrt_gb300 import build as hb
    hb.build()
    return hb.build(checked=True)


def _run(tmp_path, lib, mode, tag):
    script = tmp_path / "checked_case.py"
    script.write_text(SCRIPT)
    out = str(tmp_path / f"{tag}.npz")
    env = dict(os.environ, HRT_ROOT=ROOT)
    env.pop("HRT_CHECKED_NODE_LIMIT", None)
    if lib:
        env["HRT_LIBRARY"] = lib
    else:
        env.pop("HRT_LIBRARY", None)
    r = subprocess.run([sys.executable, str(script), out, mode], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return dict(np.load(out))


def test_checked_build_matches_the_normal_build(tmp_path, checked_lib):
    a = _run(tmp_path, None, "plain", "normal")
    b = _run(tmp_path, checked_lib, "plain", "checked")
    assert int(a["plain_frame_status"]) == 0 and int(b["plain_frame_status"]) == 0
    assert np.array_equal(a["plain_hits"], b["plain_hits"]) and np.array_equal(a["plain_rgba"], b["plain_rgba"])
    assert np.array_equal(a["plain_rays"], b["plain_rays"])
    assert (a["plain_rays"][0].view(np.float32) >= 0).sum() > 1000


def test_checked_build_reports_indices_past_the_reported_nodes(tmp_path, checked_lib):
    ref = _run(tmp_path, None, "plain", "normal")
    c = _run(tmp_path, checked_lib, "limit", "limited")
    assert int(c["limited_frame_status"]) == 7 and int(c["limited_rays_status"]) == 7  # HRT_ERR_BOUNDS
    # the same context afterwards: TLASes built without the hook trace as the normal build does
    assert int(c["plain_frame_status"]) == 0 and np.array_equal(c["plain_hits"], ref["plain_hits"])
    assert np.array_equal(c["plain_rays"], ref["plain_rays"])
    assert int(c["single_frame_status"]) == 0
