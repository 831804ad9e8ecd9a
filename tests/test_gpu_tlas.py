"""TLAS over many instances of mixed types and precisions, against the FP64 oracle.

The TLAS is a binary BVH over the instances' world-space boxes (built on the host); a ray walks
it and traverses each instance's BLAS in that BLAS's own node format, so FP32 and quantised
BLASes share a TLAS (and a batch). The oracle walks every instance, so agreement also checks
that the instance BVH never loses one.
"""
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import (DOTS, LSS, MESH, PHANTOM, OracleScene, aimed_rays, compare_hits, lines_from_strands,
                       mesh_oracle_data, oracle_geometry, sphere_mesh)

pytestmark = pytest.mark.gpu

AGREE = 0.9999
T_REL = 1e-5
RGB_ABS = 1e-4


def _rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q *= np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _instances(ctx, orc, n=72, seed=77):
    """n instances cycling through Phantom, LSS, DOTS and a triangle mesh, alternately FP32 and
    quantised, each scaled, rotated and placed on its own; returns the TLAS, the oracle scene and
    the world-space lines of the hair instances (for aimed rays)."""
    rng = np.random.default_rng(seed)
    kinds = (PHANTOM, LSS, DOTS, MESH)
    base = {}
    for k, gt in enumerate(kinds[:3]):
        v, r, off = H.generate_strands(H.StrandParams(seed=seed + k, nstrands=80, nverts=12))
        lines, lrad = lines_from_strands(v, r, off)
        base[gt] = (v, r, off, lines, oracle_geometry(orc, gt, lines, lrad))
    mv, mtri, mnrm = sphere_mesh(rng, nu=24, nv=12)
    base[MESH] = (mv, mtri, mnrm, None, mesh_oracle_data(mv, mtri, mnrm))
    blases, odata, xfs, world_lines = [], [], [], []
    for i in range(n):
        gt = kinds[i % 4]
        prec = H.Precision((i // 4) % 2)
        xf = np.eye(4, dtype=np.float32)
        xf[:3, :3] = (rng.uniform(0.12, 0.25) * _rotation(rng)).astype(np.float32)
        xf[:3, 3] = [rng.uniform(-1.3, 1.3), rng.uniform(-0.9, 0.9), rng.uniform(-0.6, 0.6)]
        v, a2, a3, lines, od = base[gt]
        if gt == MESH:
            inp = H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=a2, normals=a3, transform=xf, precision=prec)
        else:
            inp = H.BLASInput(type=H.BLASType(gt), vertices=v, radius=a2, strand_offsets=a3, transform=xf, precision=prec)
            wl = (lines.reshape(-1, 3) @ xf[:3, :3].T + xf[:3, 3]).reshape(-1, 6).astype(np.float32)
            world_lines.append((i, wl))
        blases.append(H.BottomLevelAccelerationStructure(inp, ctx))
        odata.append((gt, *od))
        xfs.append(xf)
    tlas = H.TopLevelAccelerationStructure(blases, ctx)
    return blases, tlas, OracleScene(orc, odata, xfs), world_lines


def test_tlas_frame_of_72_mixed_instances_vs_oracle(ctx, orc):
    """Hit ids and distances at the trace tests' bars. Colours: the instances are scaled by
    0.12-0.25, so a hair's radius is about 1e-4 in world units, and the ray's object-space origin
    and direction carry the FP32 rounding of the world-to-object transform (about 1e-7 of the
    camera distance, as in a GPU's hardware instance transform); the oracle transforms in FP64.
    Normals of such thin, scaled hair move by up to about 1e-3 (the oracle's own FP32 tracer
    against its FP64 tracer shows the same), so colours are held to 1e-4 on 99.8 % of the agreeing
    pixels and to 5e-3 on all."""
    blases, tlas, osc, _ = _instances(ctx, orc)
    w, h = 320, 200
    cam = H.scene_camera(w, h)
    fr = H.Frame(ctx, w, h, 1, with_hits=True)
    H.trace(ctx, tlas, cam, fr, H.trace_params(shading=2, record_hits=1))
    rgba, hits = fr.download(hits=True)
    vi, pi = H.camera_arrays(cam)
    o = osc.render(vi, pi, w, h, shading=2, precision=64)
    st = compare_hits(np.where(hits["t"] >= 0, hits["t"].astype(np.float64), -1.0), hits["prim"], hits["inst"],
                      o["t"], o["prim"], o["inst"])
    print({k: v for k, v in st.items() if k != "mism_idx"})
    assert st["hits"] > 4000 and st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL
    assert len(np.unique(hits["inst"][hits["t"] >= 0])) >= 40  # most instances are seen
    same = (hits["prim"] == o["prim"]) & (hits["inst"] == o["inst"]) & \
        (((hits["flags"] & H.HIT_SHADOWED) != 0) == (o["shadow"] != 0))
    diff = np.abs(rgba.reshape(-1, 4) - o["fb"]).max(axis=1)
    assert same.mean() >= 0.999
    assert (diff[same] <= RGB_ABS).mean() >= 0.998 and diff[same].max() <= 5e-3


def test_tlas_explicit_rays_vs_oracle(ctx, orc):
    blases, tlas, osc, world_lines = _instances(ctx, orc, seed=78)
    rng = np.random.default_rng(5)
    rays = np.concatenate([aimed_rays(rng, wl, 300, spread=0.003) for _, wl in world_lines])
    g = H.trace_rays(ctx, tlas, rays)
    o_t, o_prim, o_inst, _ = osc.trace_rays(rays, precision=64)
    st = compare_hits(np.where(g["t"] >= 0, g["t"].astype(np.float64), -1.0), g["prim"], g["inst"], o_t, o_prim, o_inst)
    print({k: v for k, v in st.items() if k != "mism_idx"})
    assert st["hits"] > len(rays) // 4 and st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL
    hit_insts = set(np.unique(g["inst"][g["t"] >= 0]).tolist())
    assert len(hit_insts & {i for i, _ in world_lines}) >= 40


def test_tlas_mixed_precision_batch_equals_single_launches(ctx, orc):
    """A batch whose scenes (and one scene's TLAS) mix FP32 and quantised BLASes: the graph replay
    equals the scenes' single launches."""
    blases, tlas, osc, _ = _instances(ctx, orc, n=24, seed=79)
    v, r, off = H.generate_strands(H.StrandParams(seed=80, nstrands=200, nverts=16))
    singles = []
    for prec in (H.Precision.FP32, H.Precision.QUANTISED):
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r,
                                                           strand_offsets=off, precision=prec), ctx)
        singles.append((b, H.TopLevelAccelerationStructure([b], ctx)))
    scenes = [(tlas, H.orbit_camera(96, 64, 0.3, 0.1), H.Frame(ctx, 96, 64, 2, with_hits=True))] + \
             [(t, H.orbit_camera(64, 48, 0.9 * k, 0.2), H.Frame(ctx, 64, 48, 1, with_hits=True))
              for k, (_, t) in enumerate(singles)]
    for split in (0, 1):
        p = H.trace_params(shading=2, record_hits=1, jitter=1, seed=6, split_types=split)
        batch = H.Batch(ctx, scenes, p)
        batch.launch()
        got = [fr.download(hits=True) for (_, _, fr) in scenes]
        for (rgba, hits), (t, cam, fr) in zip(got, scenes):
            f2 = H.Frame(ctx, fr.width, fr.height, fr.spp, with_hits=True)
            H.trace(ctx, t, cam, f2, p)
            rgba1, hits1 = f2.download(hits=True)
            assert np.array_equal(hits, hits1) and np.abs(rgba - rgba1).max() <= 1e-6
