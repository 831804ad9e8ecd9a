"""Generates tests/golden/ref_vectors.npz from the reference's own code.

The reference (mmzala/vkhrt) ships no tests or golden data. Its shader math
(shaders/curve.glsl, cone.glsl, cylinder.glsl, ray.glsl, shading.glsl, the Prhi function of
hair_intersection.rint and the ray_gen.rgen body) and its host geometry processing
(source/resources/model/geometry_processor.cpp) are compiled as C++ by oracle/build_ref.sh into
oracle/_ref/libhrtref.so; this script runs that library on seeded inputs and stores inputs and
outputs. Needs the reference checkout, so it runs only where it is present:

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build as ob  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_vectors.npz")


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def prhi_cases(rng, n):
    """(ray, curve) pairs aimed near the curve, so a good share hit, graze or iterate."""
    rays = np.zeros((n, 6), np.float32)
    curves = np.zeros((n, 12), np.float32)
    for i in range(n):
        c = (rng.normal(size=(4, 3)) * rng.choice([0.02, 0.05, 0.2])).astype(np.float32)
        c[1:] += c[0]
        if i % 7 == 0:  # straight (collinear) curves
            a, b = c[0], c[3]
            c[1] = a + (b - a) / 3
            c[2] = a + 2 * (b - a) / 3
        tgt = c[0] + (c[3] - c[0]) * rng.random() + rng.normal(size=3) * 0.02
        org = rng.normal(size=3) * 3
        d = tgt - org
        d = d / np.linalg.norm(d)
        rays[i, :3] = org
        rays[i, 3:] = d
        curves[i] = c.reshape(-1)
    return rays, curves


def main():
    ref = ob.load_ref()
    if ref is None:
        ob.build(with_ref=True)
        ref = ob.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref was not built (reference checkout missing)")
    rng = np.random.default_rng(20261203)
    out = {}

    # Prhi, FP32 and FP64 (hair_intersection.rint:15-130)
    n = 4000
    rays, curves = prhi_cases(rng, n)
    t32 = np.zeros(n, np.float32)
    n32 = np.zeros((n, 3), np.float32)
    t64 = np.zeros(n, np.float64)
    n64 = np.zeros((n, 3), np.float64)
    for i in range(n):
        t32[i] = ref.ref_prhi_f32(P(rays[i]), P(curves[i]), P(n32[i]))
        r64 = rays[i].astype(np.float64)
        c64 = curves[i].astype(np.float64)
        t64[i] = ref.ref_prhi_f64(P(r64), P(c64), P(n64[i]))
    out.update(prhi_rays=rays, prhi_curves=curves, prhi_t32=t32, prhi_n32=n32, prhi_t64=t64, prhi_n64=n64)

    # cone.glsl / cylinder.glsl / curve.glsl / ray.glsl / shading.glsl
    m = 2000
    cones = rng.normal(size=(m, 8)).astype(np.float32)
    cone_out = np.zeros((m, 6), np.float32)
    cyl_rays = rng.normal(size=(m, 6)).astype(np.float32)
    cyls = rng.normal(size=(m, 7)).astype(np.float32)
    cyl_out = np.zeros(m, np.int32)
    samp_curves = rng.normal(size=(m, 12)).astype(np.float32)
    samp_t = rng.random(m).astype(np.float32)
    samp_out = np.zeros((m, 6), np.float32)
    rcc_out = np.zeros((m, 16), np.float32)
    normals = rng.normal(size=(m, 3)).astype(np.float32)
    shade_out = np.zeros((m, 3), np.float32)
    for i in range(m):
        ref.ref_cone_f32(P(cones[i]), P(cone_out[i]))
        cyl_out[i] = ref.ref_cylinder_f32(P(cyl_rays[i]), P(cyls[i]))
        ref.ref_curve_sample_f32(P(samp_curves[i]), float(samp_t[i]), P(samp_out[i]))
        ref.ref_rcc_matrix_f32(P(cyl_rays[i]), P(rcc_out[i]))
        ref.ref_shade_f32(P(normals[i]), P(shade_out[i]))
    out.update(cones=cones, cone_out=cone_out, cyl_rays=cyl_rays, cyls=cyls, cyl_out=cyl_out,
               samp_curves=samp_curves, samp_t=samp_t, samp_out=samp_out, rcc_out=rcc_out,
               normals=normals, shade_out=shade_out)

    # ray_gen.rgen:18-24 on a 37x23 launch with random camera matrices
    vi = rng.normal(size=16).astype(np.float32)
    pi = rng.normal(size=16).astype(np.float32)
    W, Hh = 37, 23
    rg_o = np.zeros((Hh, W, 3), np.float32)
    rg_d = np.zeros((Hh, W, 3), np.float32)
    for py in range(Hh):
        for px in range(W):
            ref.ref_raygen_f32(P(vi), P(pi), px, py, W, Hh, P(rg_o[py, px]), P(rg_d[py, px]))
    out.update(rg_view_inv=vi, rg_proj_inv=pi, rg_size=np.array([W, Hh], np.int32), rg_o=rg_o, rg_d=rg_d)

    # host geometry processing on connected strands (plus a few isolated and degenerate lines)
    S, V = 40, 12
    steps = (rng.normal(size=(S, V, 3)) * 0.05).astype(np.float32)
    verts = np.cumsum(steps, axis=1).astype(np.float32)
    lines = np.stack([verts[:, :-1], verts[:, 1:]], axis=2).reshape(-1, 6).astype(np.float32)
    lines[5, 3:] = lines[5, :3]  # zero-length line
    nl = lines.shape[0]
    g_curves = np.zeros((nl, 12), np.float32)
    ref.ref_generate_curves(P(lines), nl, P(g_curves))
    g_aabbs = np.zeros((nl, 6), np.float32)
    ref.ref_generate_aabbs(P(g_curves), nl, 0.02, P(g_aabbs))
    g_dots = np.zeros((nl * 12, 3), np.float32)
    g_idx = np.zeros(nl * 12, np.uint32)
    ok = np.ones(nl, bool)
    ok[5] = False  # the zero-length line normalises 0/0; keep it out of the DOTS vectors
    lines_ok = np.ascontiguousarray(lines[ok])
    nok = lines_ok.shape[0]
    g_dots = np.zeros((nok * 12, 3), np.float32)
    g_idx = np.zeros(nok * 12, np.uint32)
    ref.ref_generate_dots(P(lines_ok), nok, 0.02, P(g_dots), P(g_idx))
    g_lss_p = np.zeros((nl * 2, 3), np.float32)
    g_lss_r = np.zeros(nl * 2, np.float32)
    ref.ref_generate_lss(P(lines), nl, 0.0005, P(g_lss_p), P(g_lss_r))
    out.update(geo_lines=lines, geo_curves=g_curves, geo_aabbs=g_aabbs, geo_dots_lines=lines_ok,
               geo_dots=g_dots, geo_dots_idx=g_idx, geo_lss_p=g_lss_p, geo_lss_r=g_lss_r)

    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
