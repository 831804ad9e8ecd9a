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
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import PHANTOM, aimed_rays, compare_hits, lines_from_strands

pytestmark = pytest.mark.gpu

T_REL = 1e-5   # hit distance, relative (as in the other trace tests)
AGREE = 0.9999


def _scene(ctx):
    v, r, off = H.generate_strands(H.StrandParams(seed=77, nstrands=400, nverts=24))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType(PHANTOM), vertices=v, radius=r, strand_offsets=off), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    lines, _ = lines_from_strands(v, r, off)
    return blas, tlas, lines


def _same(a, b):
    st = compare_hits(np.where(a["t"] >= 0, a["t"].astype(np.float64), -1.0), a["prim"], a["inst"],
                      np.where(b["t"] >= 0, b["t"].astype(np.float64), -1.0), b["prim"], b["inst"])
    return st


def test_noalloc_matches_trace_rays_on_two_calls(ctx):
    blas, tlas, lines = _scene(ctx)
    rng = np.random.default_rng(123)
    for call in range(2):  # the scratch array keeps the previous call's contents
        n = [H.NOALLOC_MAX_RAYS, 5000][call]
        rays = aimed_rays(rng, lines, n, spread=0.006)
        ref = H.trace_rays(ctx, tlas, rays)
        got = H.trace_rays_noalloc(ctx, tlas, rays)
        st = _same(got, ref)
        assert st["hits"] > n // 4
        assert st["agreement"] >= AGREE and st["max_rel_t"] <= T_REL
        assert np.array_equal(got["flags"], ref["flags"])


def test_noalloc_rejects_more_rays_than_its_scratch(ctx):
    blas, tlas, lines = _scene(ctx)
    rays = np.zeros((H.NOALLOC_MAX_RAYS + 1, 6), np.float32)
    with pytest.raises(H.HrtError) as e:
        H.trace_rays_noalloc(ctx, tlas, rays)
    assert e.value.status == 1 and "at most" in str(e.value)
