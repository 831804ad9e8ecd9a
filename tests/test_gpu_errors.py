"""The bounded device loops' failure paths, made to fire with small bounds.

Every traversal loop counts its steps and its stack entries (hrt_trace_params.max_steps,
max_depth); a ray that runs out stops, sets a bit in the launch's device error word and the
launch stops taking work, so the kernel returns. The host maps the bit to HRT_ERR_TIMEOUT or
HRT_ERR_STACK_OVERFLOW, and the context stays usable: the next trace with the default bounds
matches the FP64 oracle. Nothing here faults or hangs a GPU: the bounds only end loops early.
"""
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import PHANTOM, OracleScene, aimed_rays, compare_hits, lines_from_strands, oracle_geometry

pytestmark = pytest.mark.gpu

TIMEOUT, OVERFLOW, INVALID = 5, 4, 1


def _scene(ctx, orc, seed=301, ns=1500, nv=17):
    v, r, off = H.generate_strands(H.StrandParams(seed=seed, nstrands=ns, nverts=nv))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r, strand_offsets=off,
                    precision=H.Precision.QUANTISED), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    lines, lrad = lines_from_strands(v, r, off)
    osc = OracleScene(orc, [(PHANTOM, *oracle_geometry(orc, PHANTOM, lines, lrad))])
    return blas, tlas, osc


def _frame_matches_oracle(ctx, tlas, osc):
    w, h = 96, 64
    cam = H.scene_camera(w, h)
    fr = H.Frame(ctx, w, h, 1, with_hits=True)
    H.trace(ctx, tlas, cam, fr, H.trace_params(shading=2, record_hits=1))
    _, hits = fr.download(hits=True)
    vi, pi = H.camera_arrays(cam)
    o = osc.render(vi, pi, w, h, shading=2, precision=64)
    st = compare_hits(np.where(hits["t"] >= 0, hits["t"].astype(np.float64), -1.0), hits["prim"], hits["inst"],
                      o["t"], o["prim"], o["inst"])
    assert st["hits"] > 300 and st["agreement"] >= 0.9999, st


@pytest.mark.parametrize("bound,status", [({"max_steps": 2}, TIMEOUT), ({"max_depth": 2}, OVERFLOW)])
def test_frame_bounds_return_their_status_and_the_context_recovers(ctx, orc, bound, status):
    blas, tlas, osc = _scene(ctx, orc)
    fr = H.Frame(ctx, 96, 64, 2)
    with pytest.raises(H.HrtError) as e:
        H.trace(ctx, tlas, H.scene_camera(96, 64), fr, H.trace_params(shading=2, spp=2, jitter=1, **bound))
    assert e.value.status == status
    _frame_matches_oracle(ctx, tlas, osc)


@pytest.mark.parametrize("bound,status", [({"max_steps": 2}, TIMEOUT), ({"max_depth": 2}, OVERFLOW)])
def test_explicit_ray_bounds_return_their_status(ctx, orc, bound, status):
    blas, tlas, osc = _scene(ctx, orc)
    v, r, off = H.generate_strands(H.StrandParams(seed=301, nstrands=1500, nverts=17))
    lines, _ = lines_from_strands(v, r, off)
    rays = aimed_rays(np.random.default_rng(9), lines, 2000, spread=0.006)
    with pytest.raises(H.HrtError) as e:
        H.trace_rays(ctx, tlas, rays, H.trace_params(**bound))
    assert e.value.status == status
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
    st = compare_hits(np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0), g["prim"], g["inst"], o_t, o_prim, o_inst)
    assert st["agreement"] >= 0.9999, st


def test_async_frame_error_surfaces_at_the_download(ctx, orc):
    blas, tlas, osc = _scene(ctx, orc)
    fr = H.Frame(ctx, 96, 64, 1)
    H.trace(ctx, tlas, H.scene_camera(96, 64), fr, H.trace_params(shading=2, max_steps=2, **{"async": 1}))
    with pytest.raises(H.HrtError) as e:
        fr.download()
    assert e.value.status == TIMEOUT
    _frame_matches_oracle(ctx, tlas, osc)


def test_async_batch_error_surfaces_at_the_download_and_the_next_launch(ctx, orc):
    blas, tlas, osc = _scene(ctx, orc)
    cams = [H.orbit_camera(80, 48, a, 0.1) for a in (0.0, 0.7)]
    frames = [H.Frame(ctx, 80, 48, 1) for _ in cams]
    bad = H.Batch(ctx, [(tlas, c, f) for c, f in zip(cams, frames)],
                  H.trace_params(shading=2, max_depth=2, **{"async": 1}))
    bad.launch()  # asynchronous: returns before the replay ends
    dst = [np.zeros((48, 80, 4), np.float32) for _ in cams]
    with pytest.raises(H.HrtError) as e:
        bad.download(dst, synchronise=True)
    assert e.value.status == OVERFLOW
    with pytest.raises(H.HrtError) as e:
        bad.launch()  # the finished replay's error is reported before replaying again
    assert e.value.status == OVERFLOW
    good = H.Batch(ctx, [(tlas, c, f) for c, f in zip(cams, frames)], H.trace_params(shading=2, **{"async": 1}))
    good.launch()
    good.download(dst, synchronise=True)
    for c, d in zip(cams, dst):
        ref = H.Frame(ctx, 80, 48, 1)
        H.trace(ctx, tlas, c, ref, H.trace_params(shading=2))
        assert np.array_equal(ref.download(), d)


def test_bounds_beyond_the_stack_are_refused(ctx, orc):
    blas, tlas, osc = _scene(ctx, orc, ns=50)
    fr = H.Frame(ctx, 16, 16, 1)
    with pytest.raises(H.HrtError) as e:
        H.trace(ctx, tlas, H.scene_camera(16, 16), fr, H.trace_params(max_depth=65))
    assert e.value.status == INVALID


def test_log_level_prints_builds_and_failures(tmp_path):
    """HRT_LOG=2 prints one line per built BLAS and one per failure on stderr, prefixed [hrt]."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import numpy as np, vkhrt_gb300 as H\n"
            "ctx = H.Context(0)\n"
            "v, r, off = H.generate_strands(H.StrandParams(seed=5, nstrands=40, nverts=8))\n"
            "H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r,"
            " strand_offsets=off), ctx)\n"
            "try:\n"
            "    H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r,"
            " strand_offsets=off, width=9), ctx)\n"
            "except H.HrtError as e:\n"
            "    print('status', e.status)\n") % root
    r = subprocess.run([sys.executable, "-c", code], env=dict(os.environ, HRT_LOG="2"), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "status 1" in r.stdout
    lines = [x for x in r.stderr.splitlines() if x.startswith("[hrt]")]
    assert any("BLAS type 0 precision 0: 280 primitives" in x for x in lines), lines
    assert any("error 1" in x and "width" in x for x in lines), lines
