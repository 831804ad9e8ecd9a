"""The CUDA trace pass vs the FP64 CPU oracle on the same seeded scenes.

Closest-hit primitive ids must agree except within t-ties (|t1 - t2| <= 1e-5 t), at >= 99.99 %
of the rays; distances of agreeing hits within 1e-5 relative; pixels within 1e-4 where the hits
(and shadow rays) agree.
"""
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import (DOTS, LSS, PHANTOM, VOXELS, P, OracleScene, aimed_rays, compare_hits, lines_from_strands,
                       oracle_geometry, oracle_voxels)

pytestmark = pytest.mark.gpu

T_REL = 1e-5     # hit distance, relative
RGB_ABS = 1e-4   # pixel colour, absolute
AGREE = 0.9999   # closest-hit id agreement outside t-ties


def make_scene(ctx, orc, gtype, precision=0, seed=21, ns=300, nv=17, radius=True, const_radius=0.02,
               transform=None):
    v, r, off = H.generate_strands(H.StrandParams(seed=seed, nstrands=ns, nverts=nv))
    if not radius:
        r = None
    xf = np.eye(4, dtype=np.float32) if transform is None else transform
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r, strand_offsets=off, precision=H.Precision(precision),
                    const_radius=const_radius, transform=xf), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    lines, lrad = lines_from_strands(v, r, off, const_radius)
    data, rad = oracle_geometry(orc, gtype, lines, lrad)
    osc = OracleScene(orc, [(gtype, data, rad)], [None if transform is None else transform])
    return blas, tlas, osc, lines


@pytest.mark.parametrize("gtype", [PHANTOM, LSS, DOTS])
@pytest.mark.parametrize("precision", [0, 1])
def test_trace_rays_vs_fp64_oracle(ctx, orc, gtype, precision):
    blas, tlas, osc, lines = make_scene(ctx, orc, gtype, precision)
    rng = np.random.default_rng(100 + gtype)
    rays = aimed_rays(rng, lines, 20000, spread=0.006)
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
    g_t = np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0)
    st = compare_hits(g_t, g["prim"], g["inst"], o_t, o_prim, o_inst)
    print(gtype, precision, {k: v for k, v in st.items() if k != "mism_idx"})
    assert st["hits"] > 3000
    assert st["agreement"] >= AGREE
    assert st["p9999_rel_t"] <= T_REL


@pytest.mark.parametrize("rays_kind", ["camera", "aimed"])
def test_quantised_phantom_vs_fp64_on_the_original_strands(ctx, orc, rays_kind):
    """The precision pattern against the real geometry: a quantised Phantom BLAS of C4-like
    strands (3,000 x 128 vertices, radius 0.003 -> 0.0008, seed 1004) against the FP64 oracle on
    the strands' own FP32 curves, on camera rays (480x270, the C4 camera) and on rays aimed at
    the hair."""
    v, r, off = H.generate_strands(H.StrandParams(seed=1004, nstrands=3000, nverts=128, r_root=0.003, r_tip=0.0008))
    blas = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r,
                                                          strand_offsets=off, precision=H.Precision.QUANTISED), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    lines, lrad = lines_from_strands(v, r, off)
    curves = np.zeros((len(lines), 12), np.float32)
    orc.orc_generate_curves(P(lines), len(lines), P(curves))
    osc = OracleScene(orc, [(PHANTOM, curves, lrad)])
    if rays_kind == "camera":
        w, h = 480, 270
        cam = H.scene_camera(w, h)
        fr = H.Frame(ctx, w, h, 1, with_hits=True)
        H.trace(ctx, tlas, cam, fr, H.trace_params(shading=2, record_hits=1))
        _, hits = fr.download(hits=True)
        vi, pi = H.camera_arrays(cam)
        o = osc.render(vi, pi, w, h, shading=2, precision=64)
        g_t = np.where(hits["t"] >= 0, hits["t"].astype(np.float64), -1.0)
        st = compare_hits(g_t, hits["prim"], hits["inst"], o["t"], o["prim"], o["inst"])
        assert st["hits"] > 40000
    else:
        rays = aimed_rays(np.random.default_rng(1004), lines, 20000)
        g = H.trace_rays(ctx, tlas, rays)
        o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
        g_t = np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0)
        st = compare_hits(g_t, g["prim"], g["inst"], o_t, o_prim, o_inst)
        assert st["hits"] > 10000
    print(rays_kind, {k: v for k, v in st.items() if k != "mism_idx"})
    assert st["agreement"] >= AGREE, st
    assert st["p9999_rel_t"] <= T_REL


def test_trace_rays_fp32_resolve_off_vs_fp32_oracle(ctx, orc):
    """Without the FP64 re-solve the GPU's FP32 Phantom is the oracle's FP32 algorithm evaluated
    from the shifted origin (oracle mode 33)."""
    blas, tlas, osc, lines = make_scene(ctx, orc, PHANTOM, 0, seed=22)
    rays = aimed_rays(np.random.default_rng(5), lines, 20000, spread=0.006)
    g = H.trace_rays(ctx, tlas, rays, H.trace_params(fp64_resolve=0))
    o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=33)
    g_t = np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0)
    st = compare_hits(g_t, g["prim"], g["inst"], o_t, o_prim, o_inst)
    assert st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL


def render_both(ctx, tlas, osc, w, h, spp=1, shading=2, jitter=0, seed=0):
    cam = H.scene_camera(w, h)
    vi, pi = H.camera_arrays(cam)
    fr = H.Frame(ctx, w, h, spp, with_hits=True)
    H.trace(ctx, tlas, cam, fr, H.trace_params(spp=spp, shading=shading, jitter=jitter, seed=seed, record_hits=1))
    rgba, hits = fr.download(hits=True)
    o = osc.render(vi, pi, w, h, spp=spp, jitter=jitter, seed=seed, shading=shading, precision=64)
    return fr, rgba, hits, o


def frame_checks(rgba, hits, o, spp):
    g_t = np.where(hits["t"] >= 0, hits["t"].astype(np.float64), -1.0)
    st = compare_hits(g_t, hits["prim"], hits["inst"], o["t"], o["prim"], o["inst"])
    # pixels whose samples all agree (ids and shadow flags) must match in colour
    shadow_g = (hits["flags"] & H.HIT_SHADOWED) != 0
    same = (hits["prim"] == o["prim"]) & (shadow_g == (o["shadow"] != 0))
    px_ok = same.reshape(-1, spp).all(axis=1)
    diff = np.abs(rgba.reshape(-1, 4) - o["fb"]).max(axis=1)
    return st, px_ok, diff


@pytest.mark.parametrize("gtype", [PHANTOM, LSS, DOTS])
def test_frame_shaded_with_shadows(ctx, orc, gtype):
    blas, tlas, osc, _ = make_scene(ctx, orc, gtype, 0, seed=31, ns=1000, nv=32)
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 160, 120, spp=1, shading=2)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    print(gtype, {k: v for k, v in st.items() if k != "mism_idx"}, "pixels agreeing", px_ok.mean(),
          "max rgb diff there", diff[px_ok].max())
    assert st["hits"] > 1000
    assert st["agreement"] >= AGREE
    assert st["p9999_rel_t"] <= T_REL
    assert px_ok.mean() >= 0.999
    assert diff[px_ok].max() <= RGB_ABS
    assert np.all(rgba[..., 3] == 1.0)
    s = fr.stats()
    assert s["primary_rays"] == 160 * 120 and s["shadow_rays"] == int((hits["t"] >= 0).sum())


def test_frame_reference_literal_debug_colours(ctx, orc):
    """Constant radius 0.02 and the debug palette: the reference's own closest-hit output."""
    blas, tlas, osc, _ = make_scene(ctx, orc, PHANTOM, 0, seed=32, ns=300, nv=16, radius=False, const_radius=0.02)
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 128, 96, spp=1, shading=0)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    assert st["agreement"] >= AGREE
    assert diff[px_ok].max() == 0.0  # palette colours are exact
    hit = hits["t"] >= 0
    pal = np.array([[1.0, 0.0, 0.3], [0.8, 0.2, 0.3], [0.6, 0.4, 0.3], [0.4, 0.6, 0.3], [0.2, 0.8, 0.3],
                    [0.0, 1.0, 0.3]], np.float32)
    assert np.array_equal(rgba.reshape(-1, 4)[hit, :3], pal[hits["prim"][hit] % 6])
    assert np.all(rgba.reshape(-1, 4)[~hit, :3] == 0.0)  # miss: black background


def test_frame_quantised_jittered_spp4(ctx, orc):
    blas, tlas, osc, _ = make_scene(ctx, orc, PHANTOM, 1, seed=33, ns=600, nv=64)
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 96, 64, spp=4, shading=2, jitter=1, seed=9)
    st, px_ok, diff = frame_checks(rgba, hits, o, 4)
    print({k: v for k, v in st.items() if k != "mism_idx"}, px_ok.mean())
    assert st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL
    assert px_ok.mean() >= 0.998 and diff[px_ok].max() <= RGB_ABS


def test_instance_transform(ctx, orc):
    xf = np.array([[0.0, -1.2, 0.0, 0.1], [1.2, 0.0, 0.0, -0.3], [0.0, 0.0, 1.2, 0.2], [0, 0, 0, 1]], np.float32)
    blas, tlas, osc, lines = make_scene(ctx, orc, LSS, 0, seed=34, transform=xf)
    np.testing.assert_array_equal(blas.Transform(), xf)
    assert blas.Type() == H.BLASType.eLSS
    wl = lines.reshape(-1, 3) @ xf[:3, :3].T + xf[:3, 3]
    rays = aimed_rays(np.random.default_rng(8), wl.reshape(-1, 6).astype(np.float32), 10000, spread=0.006)
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
    st = compare_hits(np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0), g["prim"], g["inst"], o_t, o_prim, o_inst)
    assert st["hits"] > 1000 and st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL


def test_two_instances_ids(ctx, orc):
    v1, r1, o1 = H.generate_strands(H.StrandParams(seed=40, nstrands=200, nverts=16))
    v2, r2, o2 = H.generate_strands(H.StrandParams(seed=41, nstrands=200, nverts=16))
    b1 = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.eDOTS, vertices=v1, radius=r1, strand_offsets=o1), ctx)
    b2 = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v2, radius=r2, strand_offsets=o2), ctx)
    tlas = H.TopLevelAccelerationStructure([b1, b2], ctx)
    l1, lr1 = lines_from_strands(v1, r1, o1)
    l2, lr2 = lines_from_strands(v2, r2, o2)
    osc = OracleScene(orc, [(DOTS, *oracle_geometry(orc, DOTS, l1, lr1)), (PHANTOM, *oracle_geometry(orc, PHANTOM, l2, lr2))])
    rng = np.random.default_rng(3)
    rays = np.concatenate([aimed_rays(rng, l1, 5000, 0.006), aimed_rays(rng, l2, 5000, 0.006)])
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
    st = compare_hits(np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0), g["prim"], g["inst"], o_t, o_prim, o_inst)
    assert set(np.unique(g["inst"][g["t"] >= 0])) == {0, 1}
    assert st["agreement"] >= AGREE


@pytest.mark.parametrize("split", [0, 1])
def test_batch_equals_single_launches(ctx, orc, split):
    scenes = []
    for k, (gt, ns, w, h, spp) in enumerate([(PHANTOM, 200, 64, 48, 1), (LSS, 300, 80, 40, 2), (DOTS, 150, 40, 40, 3),
                                             (VOXELS, 250, 48, 40, 2)]):
        v, r, off = H.generate_strands(H.StrandParams(seed=50 + k, nstrands=ns, nverts=16))
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType(gt), vertices=v, radius=r, strand_offsets=off,
                                                           voxel_size=0.05), ctx)
        t = H.TopLevelAccelerationStructure([b], ctx)
        scenes.append((b, t, H.scene_camera(w, h), H.Frame(ctx, w, h, spp, with_hits=True), w, h, spp))
    p = H.trace_params(shading=2, record_hits=1, jitter=1, seed=4, split_types=split)
    batch = H.Batch(ctx, [(t, cam, fr) for (_, t, cam, fr, *_r) in scenes], p)
    batch.launch()
    batch_out = [fr.download(hits=True) for (_, _, _, fr, *_r) in scenes]
    batch.launch()  # graph replay is repeatable
    for (rgba, hits), (_, _, _, fr, *_r) in zip(batch_out, scenes):
        rgba2, hits2 = fr.download(hits=True)
        assert np.array_equal(rgba, rgba2) and np.array_equal(hits, hits2)
    # a mixed-type batch runs the kernel compiled for every primitive type; single launches run
    # the per-type kernels: identical hits, pixels within 1e-6 (last-bit rounding of the
    # separately compiled FP32 Phantom solve moves shaded normals by a few ulps)
    for (rgba, hits), (b, t, cam, _, w, h, spp) in zip(batch_out, scenes):
        fr = H.Frame(ctx, w, h, spp, with_hits=True)
        H.trace(ctx, t, cam, fr, p)
        rgba1, hits1 = fr.download(hits=True)
        assert np.array_equal(hits, hits1) and np.abs(rgba - rgba1).max() <= 1e-6


def test_empty_scene_and_misses(ctx):
    v = np.zeros((2, 3), np.float32)
    b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v,
                                                       strand_offsets=np.array([0, 1, 2], np.uint32)), ctx)
    t = H.TopLevelAccelerationStructure([b], ctx)
    fr = H.Frame(ctx, 16, 16, 1, with_hits=True)
    H.trace(ctx, t, H.scene_camera(16, 16), fr, H.trace_params(shading=2, record_hits=1))
    rgba, hits = fr.download(hits=True)
    assert np.all(hits["t"] == -1.0) and np.all(hits["prim"] == 0xffffffff)
    assert np.all(rgba[..., :3] == 0.0) and np.all(rgba[..., 3] == 1.0)
    t0 = H.TopLevelAccelerationStructure([], ctx)
    H.trace(ctx, t0, H.scene_camera(16, 16), fr, H.trace_params())


def test_trace_rejects_bad_arguments(ctx):
    v, r, off = H.generate_strands(H.StrandParams(seed=60, nstrands=10, nverts=8))
    b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r, strand_offsets=off), ctx)
    xf = np.eye(4, dtype=np.float32)
    xf[0, 0] = 0.0  # singular
    with pytest.raises(H.HrtError) as e:
        H.TopLevelAccelerationStructure([H.BottomLevelAccelerationStructure(
            H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r, strand_offsets=off, transform=xf), ctx)], ctx)
    assert e.value.status == 1
    t = H.TopLevelAccelerationStructure([b], ctx)
    fr = H.Frame(ctx, 8, 8, 1, with_hits=False)
    with pytest.raises(H.HrtError) as e:
        H.trace(ctx, t, H.scene_camera(8, 8), fr, H.trace_params(record_hits=1))
    assert e.value.status == 1
    with pytest.raises(H.HrtError):
        H.trace(ctx, t, H.scene_camera(8, 8), fr, H.trace_params(shading=7))
    with pytest.raises(H.HrtError):
        H.Frame(ctx, 0, 8, 1)


def test_generator_checksum_on_this_host():
    """The strand generator gives the same bits on an aarch64 host as on x86-64 (no libm calls)."""
    from test_abi import C1_CHECKSUM
    v, r, _ = H.generate_strands(H.StrandParams())
    assert H.checksum(v, r) == C1_CHECKSUM


def test_quantised_node_visits_close_to_fp32(ctx):
    """The 8-bit boxes are the FP32 boxes rounded outward: same tree, a few more visits at most.
    Shadow rays run along +y, so some slab distances use the clamped reciprocal of a zero."""
    v, r, off = H.generate_strands(H.StrandParams(seed=35, nstrands=3000, nverts=48))
    stats = {}
    for prec in (H.Precision.FP32, H.Precision.QUANTISED):
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r,
                                                           strand_offsets=off, precision=prec), ctx)
        t = H.TopLevelAccelerationStructure([b], ctx)
        fr = H.Frame(ctx, 192, 128, 1)
        H.trace(ctx, t, H.scene_camera(192, 128), fr, H.trace_params(shading=2, count_stats=1))
        stats[int(prec)] = fr.stats()
    f, q = stats[0], stats[1]
    # both formats hold the same curves: the same rays hit, so the shadow-ray counts agree
    assert f["shadow_rays"] > 1000 and q["shadow_rays"] > 1000
    assert abs(f["shadow_rays"] - q["shadow_rays"]) <= 2
    per_ray = lambda s: s["nodes_visited"] / (s["primary_rays"] + s["shadow_rays"])
    assert 0.9 * per_ray(f) <= per_ray(q) <= 1.3 * per_ray(f)


def test_kernel_variants_and_autotune_give_identical_frames(ctx, tmp_path):
    """Every configuration the autotuner may pick records the same hits (t, id, flags bit for
    bit) and pixels within 1e-6 (the occupancy variants are separate compilations of the FP32
    Phantom solver, whose last-bit rounding of the hit's curve parameter may differ, moving
    the shaded normal by a few ulps); the autotuner's choice is one of its candidates, and
    cached choices (with their timing) are reused."""
    scenes = []
    for k, (gt, ns, w, h, spp) in enumerate([(PHANTOM, 300, 72, 40, 2), (LSS, 200, 48, 48, 1), (DOTS, 120, 40, 56, 3)]):
        v, r, off = H.generate_strands(H.StrandParams(seed=90 + k, nstrands=ns, nverts=32))
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType(gt), vertices=v, radius=r, strand_offsets=off,
                                                           precision=H.Precision.QUANTISED), ctx)
        t = H.TopLevelAccelerationStructure([b], ctx)
        scenes.append((b, t, H.orbit_camera(w, h, 0.4 * k, 0.1), H.Frame(ctx, w, h, spp, with_hits=True)))
    ref = None
    for variant in (1, 2, 3):
        for refill, spec, again in ((4, 0, 0), (8, 1, 8), (16, 1, 16), (16, 0, 1)):
                p = H.trace_params(shading=2, record_hits=1, jitter=1, seed=5, kernel_variant=variant, refill=refill,
                                   speculative=spec, leaf_again=again)
                out = []
                for (_, t, cam, fr) in scenes:
                    H.trace(ctx, t, cam, fr, p)
                    out.append(fr.download(hits=True))
                if ref is None:
                    ref = out
                for (a, ha), (b2, hb) in zip(ref, out):
                    assert np.array_equal(ha, hb), (variant, refill, spec)
                    assert np.abs(a - b2).max() <= 1e-6, (variant, refill, spec)
    cache = str(tmp_path / "tune.json")
    sc = [(t, cam, fr) for (_, t, cam, fr) in scenes]
    best, ms = H.autotune(ctx, sc, H.trace_params(shading=2, jitter=1, seed=5), reps=1, cache=cache, key="three")
    assert ms > 0 and best.kernel_variant in (1, 2, 3) and best.refill in (8, 16) and best.leaf_again in (2, 4, 8)
    again, ms2 = H.autotune(ctx, sc, H.trace_params(shading=2, jitter=1, seed=5), reps=1, cache=cache, key="three")
    assert abs(ms2 - ms) < 1e-3 and all(getattr(again, f) == getattr(best, f) for f in H.TUNED_FIELDS)  # the stored time
    p = H.trace_params(shading=2, record_hits=1, jitter=1, seed=5, **{f: getattr(best, f) for f in H.TUNED_FIELDS})
    batch = H.Batch(ctx, sc, p)
    batch.launch()
    for (a, ha), (_, _, _, fr) in zip(ref, scenes):
        b2, hb = fr.download(hits=True)
        assert np.array_equal(ha, hb) and np.abs(a - b2).max() <= 1e-6


@pytest.mark.parametrize("precision", [0, 1])
def test_frame_primary_hits_equal_explicit_rays(ctx, orc, precision):
    """A frame's primary hits (node-group traversal, FP64 re-solve as a second pass over the
    listed pixels) equal hrt_trace_rays on the same rays (sorted traversal, FP64 re-solve
    inline): same ids and flags, t within 1e-6 relative. The rays come from the oracle's ray
    generation, which matches the GPU's bit for bit."""
    w, h = 192, 160
    v, r, off = H.generate_strands(H.StrandParams(seed=1001, nstrands=2000, nverts=32))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r, strand_offsets=off,
                    precision=H.Precision(precision)), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    cam = H.scene_camera(w, h)
    vi, pi = H.camera_arrays(cam)
    fr = H.Frame(ctx, w, h, 1, with_hits=True)
    H.trace(ctx, tlas, cam, fr, H.trace_params(shading=2, record_hits=1, count_stats=1))
    _, fh = fr.download(hits=True)
    rays = np.zeros((h * w, 6), np.float32)
    o3 = np.zeros(3, np.float32)
    d3 = np.zeros(3, np.float32)
    for py in range(h):
        for px in range(w):
            orc.orc_raygen_f32(P(vi), P(pi), px, py, w, h, 0.5, 0.5, P(o3), P(d3))
            rays[py * w + px, :3] = o3
            rays[py * w + px, 3:] = d3
    rh = H.trace_rays(ctx, tlas, rays)
    assert (fh["t"] >= 0).sum() > 1000
    assert np.array_equal(fh["prim"], rh["prim"]) and np.array_equal(fh["inst"], rh["inst"])
    assert np.array_equal(fh["flags"] & H.HIT_FP64, rh["flags"] & H.HIT_FP64)
    hit = fh["t"] >= 0
    assert np.array_equal(hit, rh["t"] >= 0)
    assert np.max(np.abs(fh["t"][hit] - rh["t"][hit]) / rh["t"][hit]) <= 1e-6
    print("fp64 resolves", fr.stats()["fp64_resolves"], "fp64 hits", int(((fh["flags"] & H.HIT_FP64) != 0).sum()))


def test_batch_set_cameras_matches_single_launch(ctx):
    """New cameras reach a captured batch through its scene table: the replay equals single
    launches with those cameras."""
    scenes = []
    for k, (gt, ns, w, h) in enumerate([(PHANTOM, 250, 64, 40), (DOTS, 200, 48, 48)]):
        v, r, off = H.generate_strands(H.StrandParams(seed=70 + k, nstrands=ns, nverts=16))
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType(gt), vertices=v, radius=r, strand_offsets=off), ctx)
        t = H.TopLevelAccelerationStructure([b], ctx)
        scenes.append((b, t, H.scene_camera(w, h), H.Frame(ctx, w, h, 1, with_hits=True), w, h))
    p = H.trace_params(shading=2, record_hits=1, split_types=1)
    batch = H.Batch(ctx, [(t, cam, fr) for (_, t, cam, fr, *_r) in scenes], p)
    new = [H.orbit_camera(w, h, 0.7 + k, 0.2) for k, (*_a, w, h) in enumerate(scenes)]
    batch.set_cameras(new)
    batch.launch()
    assert batch.table_bytes > 0
    for (b, t, _, fr, w, h), cam in zip(scenes, new):
        rgba, hits = fr.download(hits=True)
        f1 = H.Frame(ctx, w, h, 1, with_hits=True)
        H.trace(ctx, t, cam, f1, p)
        rgba1, hits1 = f1.download(hits=True)
        assert (hits["t"] >= 0).sum() > 50
        assert np.array_equal(hits, hits1) and np.abs(rgba - rgba1).max() <= 1e-6
    with pytest.raises(H.HrtError):
        batch.set_cameras(new[:1])
    # every framebuffer in one call (one skipped), equal to the per-frame downloads
    batch.launch()
    dst = [np.full((h, w, 4), -1.0, np.float32) for (*_a, w, h) in scenes]
    batch.download([dst[0], None])
    assert np.array_equal(dst[0], scenes[0][3].download().reshape(dst[0].shape))
    assert (dst[1] == -1.0).all()
    batch.download(dst)
    for (_b, _t, _c, fr, w, h), d in zip(scenes, dst):
        assert np.array_equal(d, fr.download().reshape(d.shape))
    with pytest.raises(ValueError):
        batch.download(dst[:1])


def _mesh_scene(ctx, orc, precision, with_normals, hair=False):
    from hairscene import MESH, mesh_oracle_data, sphere_mesh
    rng = np.random.default_rng(43)
    v, tri, nrm = sphere_mesh(rng)
    mb = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri, normals=nrm if with_normals else None,
                    precision=H.Precision(precision)), ctx)
    data, nd = mesh_oracle_data(v, tri, nrm if with_normals else None)
    blases, obl = [mb], [(MESH, data, nd)]
    if hair:
        hv, hr, hoff = H.generate_strands(H.StrandParams(seed=44, nstrands=800, nverts=24))
        hb = H.BottomLevelAccelerationStructure(
            H.BLASInput(type=H.BLASType.ePhantom, vertices=hv, radius=hr, strand_offsets=hoff,
                        precision=H.Precision(precision)), ctx)
        lines, lrad = lines_from_strands(hv, hr, hoff)
        hd, hrad = oracle_geometry(orc, PHANTOM, lines, lrad)
        blases.append(hb)
        obl.append((PHANTOM, hd, hrad))
    tlas = H.TopLevelAccelerationStructure(blases, ctx)
    return blases, tlas, OracleScene(orc, obl), v, tri


@pytest.mark.parametrize("precision", [0, 1])
def test_mesh_trace_rays_vs_fp64_oracle(ctx, orc, precision):
    _, tlas, osc, v, tri = _mesh_scene(ctx, orc, precision, True)
    rng = np.random.default_rng(45)
    c = v[tri].mean(axis=1)
    tgt = c[rng.integers(0, len(c), 20000)] + rng.normal(size=(20000, 3)) * 0.01
    d = rng.normal(size=(20000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([tgt - 3.0 * d, d], axis=1).astype(np.float32)
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_p, o_i, _ = osc.trace_rays(rays, precision=64)
    st = compare_hits(np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0), g["prim"], g["inst"], o_t, o_p, o_i)
    assert st["hits"] > 10000 and st["agreement"] >= AGREE and st["max_rel_t"] <= T_REL


@pytest.mark.parametrize("with_normals", [True, False])
def test_mesh_frame_shaded_vs_oracle(ctx, orc, with_normals):
    """Interpolated vertex normals (or face normals), Shade() and the shadow ray, with a Phantom
    hair BLAS in the same TLAS (the mixed-type kernel)."""
    _, tlas, osc, *_ = _mesh_scene(ctx, orc, 0, with_normals, hair=True)
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 200, 150, spp=1, shading=2)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    assert (hits["inst"] == 0).sum() > 500 and (hits["inst"] == 1).sum() > 500  # both instances are seen
    assert st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL
    assert px_ok.mean() >= 0.999 and diff[px_ok].max() <= RGB_ABS


@pytest.mark.parametrize("gtype,precision", [(PHANTOM, 0), (PHANTOM, 1), (LSS, 1), (DOTS, 0)])
def test_refit_trace_vs_fp64_oracle(ctx, orc, gtype, precision):
    """Trace a refitted BLAS (moved strands, topology kept) against the oracle on the moved
    geometry: the same agreement bar as a fresh build."""
    v, r, off = H.generate_strands(H.StrandParams(seed=12, nstrands=600, nverts=24))
    blas = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r,
                                                          strand_offsets=off, precision=H.Precision(precision)), ctx)
    v2 = (v + 0.04 * np.sin(2.0 * v[:, [2, 0, 1]])).astype(np.float32)
    blas.refit(v2, r)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)  # TLASes copy the bounds: build after a refit
    lines, lrad = lines_from_strands(v2, r, off)
    data, rad = oracle_geometry(orc, gtype, lines, lrad)
    osc = OracleScene(orc, [(gtype, data, rad)])
    rays = aimed_rays(np.random.default_rng(13), lines, 20000, spread=0.006)
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_p, o_i, _ = osc.trace_rays(rays, precision=64)
    st = compare_hits(np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0), g["prim"], g["inst"], o_t, o_p, o_i)
    assert st["hits"] > 5000 and st["agreement"] >= AGREE and st["max_rel_t"] <= T_REL


def test_mesh_refit_trace(ctx, orc):
    from hairscene import MESH, mesh_oracle_data, sphere_mesh
    v, tri, nrm = sphere_mesh(np.random.default_rng(14))
    blas = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri,
                                                          normals=nrm), ctx)
    v2 = (v * np.float32(1.2) + np.float32(0.05)).astype(np.float32)
    blas.refit(v2, nrm)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    data, nd = mesh_oracle_data(v2, tri, nrm)
    osc = OracleScene(orc, [(MESH, data, nd)])
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 128, 96, spp=1, shading=2)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    assert st["hits"] > 1000 and st["agreement"] >= AGREE and diff[px_ok].max() <= RGB_ABS


def test_environment_map_miss_shading(ctx, orc):
    """Primary rays that miss take the environment map's colour (miss.rmiss:17-37): equal to the
    oracle's within the RGB bar, with hits unchanged."""
    import torch
    blas, tlas, osc, _ = make_scene(ctx, orc, PHANTOM, 0, seed=34, ns=500, nv=24)
    rng = np.random.default_rng(35)
    env = rng.uniform(0.0, 3.0, (32, 64, 4)).astype(np.float32)
    denv = torch.as_tensor(env).cuda()
    w, h = 160, 120
    cam = H.scene_camera(w, h)
    vi, pi = H.camera_arrays(cam)
    fr = H.Frame(ctx, w, h, 2, with_hits=True)
    H.trace(ctx, tlas, cam, fr, H.trace_params(spp=2, shading=2, jitter=1, seed=3, record_hits=1,
                                               env_map=denv.data_ptr(), env_width=64, env_height=32))
    rgba, hits = fr.download(hits=True)
    o = osc.render(vi, pi, w, h, spp=2, jitter=1, seed=3, shading=2, precision=64, env=env)
    st, px_ok, diff = frame_checks(rgba, hits, o, 2)
    miss_px = (hits["t"].reshape(-1, 2) < 0).all(axis=1)
    assert miss_px.sum() > 1000 and st["agreement"] >= AGREE
    assert diff[px_ok].max() <= RGB_ABS
    assert rgba.reshape(-1, 4)[miss_px, :3].min() > 0.05  # the background is the map, not black


def test_gltf_model_builds_and_traces(ctx, tmp_path):
    """Primitives read from a glTF file build BLASes (hair lines with their radii and node
    transform, a triangle mesh) whose hits equal a build from the same arrays."""
    import json
    from test_gltf import _doc_and_blob
    from vkhrt_gb300 import gltf
    doc, blob, e = _doc_and_blob(False, True)
    doc["buffers"][0]["uri"] = "m.bin"
    (tmp_path / "m.bin").write_bytes(blob)
    (tmp_path / "m.gltf").write_text(json.dumps(doc))
    prims = gltf.load(str(tmp_path / "m.gltf"))
    blases = [H.BottomLevelAccelerationStructure(p.blas_input(H.BLASType.ePhantom), ctx) for p in prims]
    tlas = H.TopLevelAccelerationStructure(blases, ctx)
    direct = [H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=e["sv"], radius=e["rad"],
                                                             line_indices=e["pairs"][0], transform=e["hair_w"]), ctx),
              H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.eMesh, vertices=e["mv"], tri_indices=e["tri"],
                                                             normals=e["mn"], transform=e["mesh_w"]), ctx)]
    tlas2 = H.TopLevelAccelerationStructure(direct, ctx)
    rng = np.random.default_rng(21)
    tgt = np.concatenate([(e["hair_w"] @ np.c_[e["sv"], np.ones(10)].T).T[:, :3],
                          (e["mesh_w"] @ np.c_[e["mv"], np.ones(4)].T).T[:, :3]])
    tgt = tgt[rng.integers(0, len(tgt), 4000)] + rng.normal(size=(4000, 3)) * 0.02
    d = rng.normal(size=(4000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([tgt - 2.0 * d, d], axis=1).astype(np.float32)
    a, b = H.trace_rays(ctx, tlas, rays), H.trace_rays(ctx, tlas2, rays)
    assert (a["t"] >= 0).sum() > 200 and np.array_equal(a, b)


@pytest.mark.parametrize("gtype,precision", [(PHANTOM, 1), (PHANTOM, 0), (LSS, 1), (DOTS, 0)])
def test_serialized_blas_traces_identically(ctx, gtype, precision):
    """serialize -> load gives a BLAS whose hits equal the original's; a loaded BLAS refits; a
    truncated or corrupt image is refused on the host (nothing reaches the device)."""
    v, r, off = H.generate_strands(H.StrandParams(seed=15, nstrands=400, nverts=20))
    blas = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r,
                                                          strand_offsets=off, precision=H.Precision(precision)), ctx)
    data = blas.serialize()
    b2 = H.BottomLevelAccelerationStructure.load(data, ctx)
    assert b2.info["nnodes"] == blas.info["nnodes"] and b2.info["bounds"] == blas.info["bounds"]
    lines, _ = lines_from_strands(v, r, off)
    rays = aimed_rays(np.random.default_rng(16), lines, 8000, spread=0.006)
    t1, t2 = H.TopLevelAccelerationStructure([blas], ctx), H.TopLevelAccelerationStructure([b2], ctx)
    assert np.array_equal(H.trace_rays(ctx, t1, rays), H.trace_rays(ctx, t2, rays))
    v2 = (v + 0.02 * np.sin(4.0 * v)).astype(np.float32)
    blas.refit(v2, r)
    b2.refit(v2, r)
    t1, t2 = H.TopLevelAccelerationStructure([blas], ctx), H.TopLevelAccelerationStructure([b2], ctx)
    assert np.array_equal(H.trace_rays(ctx, t1, rays), H.trace_rays(ctx, t2, rays))
    with pytest.raises(H.HrtError):
        H.BottomLevelAccelerationStructure.load(data[: len(data) // 2], ctx)
    bad = bytearray(data)
    bad[:4] = b"XXXX"
    with pytest.raises(H.HrtError):
        H.BottomLevelAccelerationStructure.load(bytes(bad), ctx)
    # a node whose children lie past the tree: the header is 256 bytes (its five table counts at
    # byte 184), then the five u32 tables
    import struct
    ntab = sum(struct.unpack_from("<5Q", data, 184))
    node0 = 256 + 4 * ntab
    bad = bytearray(data)
    struct.pack_into("<I", bad, node0 + (16 if precision == 1 else 192), 0x7FFFFFF0)
    with pytest.raises(H.HrtError) as e:
        H.BottomLevelAccelerationStructure.load(bytes(bad), ctx)
    assert "out of range" in str(e.value)
    if gtype in (LSS, DOTS):
        # two references per segment: the image ends with the slot map (2 x nprims reference
        # ids), from which the loader rebuilds the partner map; a repeated id is refused
        nslots = 2 * blas.info["nprims"]
        ids = np.frombuffer(data, np.uint32, nslots, len(data) - 4 * nslots)
        assert np.array_equal(np.sort(ids), np.arange(nslots))
        bad = bytearray(data)
        struct.pack_into("<I", bad, len(data) - 4 * nslots + 4, int(ids[0]))
        with pytest.raises(H.HrtError) as e:
            H.BottomLevelAccelerationStructure.load(bytes(bad), ctx)
        assert "permutation" in str(e.value)


@pytest.mark.parametrize("size", [0.03, 0.1])
def test_voxel_frame_vs_oracle(ctx, orc, size):
    """Voxel hair: box hits (grid index ids, entry distances, face normals) against the FP64
    oracle on the same voxels. Shadow rays start on a voxel face and run along the plane it
    shares with its neighbours, so whether they start inside a neighbour depends on the hit
    point's last bits: colours are compared where the shadow flags agree, and every pixel of the
    unshadowed debug shading must match."""
    v, _, off = H.generate_strands(H.StrandParams(seed=23, nstrands=300, nverts=24))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eVoxels, vertices=v, strand_offsets=off, const_radius=0.01, voxel_size=size), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    lines, _ = lines_from_strands(v, None, off)
    m, g, vox = oracle_voxels(orc, lines, 0.01, size)
    assert blas.info["nprims"] == m
    osc = OracleScene(orc, [(VOXELS, vox, None)])
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 128, 96, spp=1, shading=2)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    print(size, {k: v for k, v in st.items() if k != "mism_idx"}, "pixels agreeing", px_ok.mean())
    assert st["hits"] > 1000
    assert st["mismatches"] == 0 and st["max_rel_t"] < 1e-5
    assert px_ok.mean() > 0.98 and diff[px_ok].max() <= 1e-4
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 128, 96, spp=1, shading=1)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    assert st["mismatches"] == 0 and px_ok.all() and diff.max() <= 1e-6


def test_voxel_blas_serializes(ctx):
    """A voxel BLAS round-trips through serialize/load (identical hits on explicit rays) and
    stays non-refittable."""
    v, _, off = H.generate_strands(H.StrandParams(seed=25, nstrands=200, nverts=16))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eVoxels, vertices=v, strand_offsets=off, voxel_size=0.05), ctx)
    b2 = H.BottomLevelAccelerationStructure.load(blas.serialize(), ctx)
    assert b2.info["nprims"] == blas.info["nprims"] and b2.info["nnodes"] == blas.info["nnodes"]
    lines, _ = lines_from_strands(v, None, off)
    rays = aimed_rays(np.random.default_rng(26), lines, 4000, spread=0.02)
    t1, t2 = H.TopLevelAccelerationStructure([blas], ctx), H.TopLevelAccelerationStructure([b2], ctx)
    h1 = H.trace_rays(ctx, t1, rays)
    assert (h1["t"] >= 0).sum() > 1000 and np.array_equal(h1, H.trace_rays(ctx, t2, rays))
    with pytest.raises(H.HrtError):
        b2.refit(v)


@pytest.mark.parametrize("gtype", [PHANTOM, DOTS])
def test_node_width_changes_no_hit(ctx, gtype):
    """The BVH's node fan-out changes which nodes a ray visits, never its closest hit: BLASes of
    width 4 and 8 give the same hits bit for bit, with more node visits at width 4."""
    v, r, off = H.generate_strands(H.StrandParams(seed=70, nstrands=800, nverts=24))
    out = {}
    for width in (4, 8):
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r,
                                                           strand_offsets=off, precision=H.Precision.QUANTISED,
                                                           width=width), ctx)
        t = H.TopLevelAccelerationStructure([b], ctx)
        fr = H.Frame(ctx, 96, 64, 1, with_hits=True)
        H.trace(ctx, t, H.scene_camera(96, 64), fr, H.trace_params(shading=2, record_hits=1, count_stats=1))
        out[width] = (fr.download(hits=True)[1], fr.stats())
    assert out[4][0].tobytes() == out[8][0].tobytes()
    assert out[4][1]["nodes_visited"] > out[8][1]["nodes_visited"]
