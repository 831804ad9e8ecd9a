"""hrt_trace_rays_noalloc: closest hit without any device allocation.

This entry point exists for callers that cannot allocate device memory, for example a picking
query issued from an interactive render loop, where the implicit device-wide synchronisation of
cudaFree would stall the frames in flight, or an integration that must stay within a fixed
device-memory budget. Its scratch (the device staging of rays and hits and the kernel's
counters) is one static device array of fixed size, so it accepts at most
HRT_NOALLOC_MAX_RAYS rays per call.

The file is named to be collected last, so a run that stops at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import time

import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import PHANTOM, OracleScene, aimed_rays, compare_hits, lines_from_strands, oracle_geometry

pytestmark = pytest.mark.gpu

T_REL = 1e-5   # hit distance, relative (as in the other trace tests)
AGREE = 0.9999


def _scene(ctx):
    v, r, off = H.generate_strands(H.StrandParams(seed=77, nstrands=400, nverts=24))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType(PHANTOM), vertices=v, radius=r, strand_offsets=off), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    lines, lrad = lines_from_strands(v, r, off)
    return blas, tlas, lines, lrad


def test_noalloc_matches_trace_rays_on_two_calls(ctx, orc):
    """Two calls in a row (the scratch array keeps the first call's contents): the same kernel as
    hrt_trace_rays, so the hits are the same bit for bit; the first call's hits also meet the
    FP64 oracle's at the trace tests' bar."""
    blas, tlas, lines, lrad = _scene(ctx)
    rng = np.random.default_rng(123)
    for call in range(2):
        n = [H.NOALLOC_MAX_RAYS, 5000][call]
        rays = aimed_rays(rng, lines, n, spread=0.006)
        ref = H.trace_rays(ctx, tlas, rays)
        got = H.trace_rays_noalloc(ctx, tlas, rays)
        assert (got["t"] >= 0).sum() > n // 4
        assert got.tobytes() == ref.tobytes()
        if call == 0:
            osc = OracleScene(orc, [(PHANTOM, *oracle_geometry(orc, PHANTOM, lines, lrad))])
            o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
            st = compare_hits(np.where(got["t"] >= 0, got["t"].astype(np.float64), -1.0), got["prim"], got["inst"],
                              o_t, o_prim, o_inst)
            assert st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL, st


def test_noalloc_does_not_wait_for_other_streams(ctx):
    """No allocation means no cudaMalloc/cudaFree and so none of their implicit device-wide
    synchronisation: a call on its own stream returns while a long (bounded, about 0.5 s) sleep
    kernel still runs on another stream."""
    torch = pytest.importorskip("torch")
    blas, tlas, lines, _ = _scene(ctx)
    rays = aimed_rays(np.random.default_rng(5), lines, 4096, spread=0.006)
    side, mine = torch.cuda.Stream(), torch.cuda.Stream()
    H.trace_rays_noalloc(ctx, tlas, rays, stream=mine.cuda_stream)  # the device's one-time set-up
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(side):
        start.record()
        torch.cuda._sleep(1_000_000_000)  # about 0.5 s of clock cycles
        end.record()
    t0 = time.perf_counter()
    got = H.trace_rays_noalloc(ctx, tlas, rays, stream=mine.cuda_stream)
    dt = time.perf_counter() - t0
    running = not end.query()  # the sleep kernel had not finished when the call returned
    side.synchronize()
    slept = start.elapsed_time(end) * 1e-3
    assert slept > 0.2, slept
    assert running and dt < 0.5 * slept, (dt, slept)
    assert got.tobytes() == H.trace_rays(ctx, tlas, rays).tobytes()


def test_noalloc_refuses_a_capturing_stream(ctx):
    """The call copies through pageable host memory and synchronises its stream, which a stream
    capture does not allow: on a capturing stream it enqueues nothing and returns
    HRT_ERR_INVALID_ARG."""
    torch = pytest.importorskip("torch")
    blas, tlas, lines, _ = _scene(ctx)
    rays = aimed_rays(np.random.default_rng(6), lines, 64)
    H.trace_rays_noalloc(ctx, tlas, rays)  # the device's one-time set-up, outside any capture
    x = torch.zeros(4, device="cuda")
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.graph(g):
        x.add_(1.0)
        try:
            H.trace_rays_noalloc(ctx, tlas, rays, stream=torch.cuda.current_stream().cuda_stream)
        except H.HrtError as e:
            err = e
    g.replay()
    torch.cuda.synchronize()
    assert err is not None and err.status == 1 and "captured" in str(err)
    assert x.tolist() == [1.0] * 4


def test_noalloc_rejects_more_rays_than_its_scratch(ctx):
    blas, tlas, lines, _ = _scene(ctx)
    rays = np.zeros((H.NOALLOC_MAX_RAYS + 1, 6), np.float32)
    with pytest.raises(H.HrtError) as e:
        H.trace_rays_noalloc(ctx, tlas, rays)
    assert e.value.status == 1 and "at most" in str(e.value)
