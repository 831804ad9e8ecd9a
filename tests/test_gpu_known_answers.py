"""Known answers of the CUDA intersectors, through the C ABI (hrt_trace_rays), on single strands
whose hits have closed forms: a straight Phantom curve is a cylinder (or a cone with tapered
radii), a ray along its axis is a miss (cone.glsl:55 divides by zero and the NaN fails every
test), an LSS segment is a round cone with analytic end-sphere and tangent-cone hits, and DOTS
and voxel hits lie on known planes. Each case checks both node layouts where the BLAS has them,
and FP32 distances to a few ulps of the ray length."""
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import DOTS, LSS, VOXELS, OracleScene, lines_from_strands, oracle_geometry, oracle_voxels

pytestmark = pytest.mark.gpu

ABS_T = 4e-6   # a few FP32 ulps at t ~ 5 (ulp 4.8e-7)


def build(ctx, gtype, verts, radius=None, const_radius=0.02, precision=0, voxel_size=0.0):
    v = np.ascontiguousarray(verts, np.float32)
    r = None if radius is None else np.ascontiguousarray(radius, np.float32)
    off = np.array([0, len(v)], np.uint32)
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r, strand_offsets=off,
                    precision=H.Precision(precision), const_radius=const_radius, voxel_size=voxel_size), ctx)
    return blas, H.TopLevelAccelerationStructure([blas], ctx)


def straight(axis, n=4):
    v = np.zeros((n, 3), np.float32)
    v[:, axis] = np.arange(n, dtype=np.float32) / np.float32(n - 1)
    return v


@pytest.mark.parametrize("precision", [0, 1])
def test_phantom_straight_curve_is_a_cylinder(ctx, precision):
    # strand along x from 0 to 1 (3 straight Bezier segments), constant radius 0.02: a ray down -z
    # at (x, y) meets the tube at z = sqrt(r^2 - y^2); both formats keep the FP32 radius
    blas, tlas = build(ctx, 0, straight(0), const_radius=0.02, precision=precision)
    r = float(np.float32(0.02))
    xs = [0.05, 0.3, 0.5, 0.7, 0.95]
    ys = [0.0, 0.01, -0.012, 0.0, 0.015]
    rays = np.array([[x, y, 5.0, 0.0, 0.0, -1.0] for x, y in zip(xs, ys)] + [[0.5, 0.05, 5.0, 0, 0, -1]], np.float32)
    g = H.trace_rays(ctx, tlas, rays)
    want = [5.0 - np.sqrt(r * r - y * y) for y in ys]
    assert np.all(np.abs(g["t"][:5] - want) <= ABS_T), (g["t"], want)
    assert g["t"][5] < 0  # 0.05 from the axis: outside the tube
    assert np.all(g["inst"][:5] == 0)


def test_phantom_tapered_middle_segment_is_a_cone(ctx):
    # radii 0.01, 0.02, 0.03, 0.04 at x = 0, 1/3, 2/3, 1: the middle segment's control points are
    # evenly spaced (Catmull-Rom of evenly spaced collinear points), so its radius is linear in x
    # and a ray down -z at x meets it at z = 0.02 + 0.03 (x - 1/3)
    blas, tlas = build(ctx, 0, straight(0), radius=[0.01, 0.02, 0.03, 0.04])
    xs = np.array([0.4, 0.5, 0.6], np.float64)
    rays = np.array([[x, 0.0, 5.0, 0.0, 0.0, -1.0] for x in xs], np.float32)
    g = H.trace_rays(ctx, tlas, rays)
    want = 5.0 - (0.02 + 0.03 * (np.float32(xs).astype(np.float64) - 1.0 / 3.0))
    assert np.all(np.abs(g["t"] - want) <= 2e-5), (g["t"], want)
    assert np.all(g["prim"] == 1)  # the middle segment


@pytest.mark.parametrize("fp64_resolve", [1, 0])
def test_phantom_ray_along_the_axis_is_a_miss(ctx, fp64_resolve):
    # a ray along a straight curve's axis: the cone step divides by zero (cone.glsl:55), the NaN
    # fails the convergence and range tests, and the reference reports nothing; neither the FP32
    # solve nor its FP64 re-solve may invent a hit
    blas, tlas = build(ctx, 0, straight(2), const_radius=0.02)
    rays = np.array([[0.0, 0.0, -5.0, 0.0, 0.0, 1.0], [0.0, 0.0, 6.0, 0.0, 0.0, -1.0]], np.float32)
    g = H.trace_rays(ctx, tlas, rays, H.trace_params(fp64_resolve=fp64_resolve))
    assert np.all(g["t"] < 0), g


@pytest.mark.parametrize("precision", [0, 1])
def test_lss_round_cone_known_answers(ctx, precision):
    # one swept sphere from (0,0,0) r=0.1 to (1,0,0) r=0.2
    blas, tlas = build(ctx, LSS, [[0, 0, 0], [1, 0, 0]], radius=[0.1, 0.2], precision=precision)
    rays = np.array([
        [-5, 0, 0, 1, 0, 0],      # along the axis: the start sphere at x = -0.1
        [6, 0, 0, -1, 0, 0],      # from the other side: the end sphere at x = 1.2
        [0.5, 5, 0, 0, -1, 0],    # side: the tangent cone
        [0.3, 0, 5, 0, 0, -1],    # side, along -z: the tangent cone again
        [0.5, 5, 0.5, 0, -1, 0],  # miss
    ], np.float32)
    g = H.trace_rays(ctx, tlas, rays)
    # in a plane through the axis the surface is the outer common tangent y = m x + c of the
    # circles (0,0; 0.1) and (1,0; 0.2): c = 0.1 s, m + c = 0.2 s with s = sqrt(1 + m^2)
    m = np.sqrt(0.01 / 0.99)
    c = 0.1 * np.sqrt(1 + m * m)
    r0, r1 = float(np.float32(0.1)), float(np.float32(0.2))
    want = [5.0 - r0, 5.0 - r1, 5.0 - (m * 0.5 + c), 5.0 - (m * float(np.float32(0.3)) + c)]
    assert np.all(np.abs(g["t"][:4] - want) <= ABS_T), (g["t"], want)
    assert g["t"][4] < 0


@pytest.mark.parametrize("precision", [0, 1])
def test_dots_quads_known_answer(ctx, orc, precision):
    # a vertical DOTS segment along +y, half-width 0.05: a ray down -z at x = 0.01 crosses the quad
    # that contains the x direction at z = 0 (t = 5), one at x = 0.2 misses both quads; the FP64
    # oracle on the same triangles gives the same ids and distances
    verts = [[0, 0, 0], [0, 1, 0]]
    blas, tlas = build(ctx, DOTS, verts, const_radius=0.05, precision=precision)
    rays = np.array([[0.01, 0.5, 5, 0, 0, -1], [-0.03, 0.25, 5, 0, 0, -1], [0.2, 0.5, 5, 0, 0, -1]], np.float32)
    g = H.trace_rays(ctx, tlas, rays)
    v = np.array(verts, np.float32)
    lines, lrad = lines_from_strands(v, None, np.array([0, 2], np.uint32), 0.05)
    data, rad = oracle_geometry(orc, DOTS, lines, lrad)
    o_t, o_prim, _, _ = OracleScene(orc, [(DOTS, data, rad)]).trace_rays(rays, precision=64)
    assert g["t"][2] < 0 and o_t[2] < 0
    assert np.all(np.abs(g["t"][:2] - 5.0) <= ABS_T) and np.all(np.abs(o_t[:2] - 5.0) <= 1e-12)
    assert np.array_equal(g["prim"][:2], o_prim[:2])
    assert np.all((g["prim"][:2] >> 2) == 0)  # triangle ids 4 i + k of segment 0


def test_voxel_box_faces_known_answer(ctx, orc):
    # a capsule along +y at x = z = 0.05, radius 0.02, voxel size 0.1: the grid starts at
    # (0.03, 0.03, 0.03), so the filled column's +z faces lie at z = 0.13 and a ray down -z
    # through it enters at t = 5 - 0.13; the voxel id is the grid index, as the oracle gives it
    verts = [[0.05, 0.05, 0.05], [0.05, 0.95, 0.05]]
    blas, tlas = build(ctx, VOXELS, verts, const_radius=0.02, voxel_size=0.1)
    rays = np.array([[0.06, 0.5, 5, 0, 0, -1], [0.1, 0.2, 5, 0, 0, -1], [0.3, 0.5, 5, 0, 0, -1]], np.float32)
    g = H.trace_rays(ctx, tlas, rays)
    v = np.array(verts, np.float32)
    lines, _ = lines_from_strands(v, None, np.array([0, 2], np.uint32), 0.02)
    _, grid, vox = oracle_voxels(orc, lines, 0.02, 0.1)
    o_t, o_prim, _, _ = OracleScene(orc, [(VOXELS, vox, None)]).trace_rays(rays, precision=64)
    assert grid[2] == np.float32(np.float32(0.05) - np.float32(0.02))  # the grid's z origin
    z_face = float(np.float32(grid[2] + np.float32(0.1)))
    assert np.all(np.abs(g["t"][:2] - (5.0 - z_face)) <= ABS_T), g["t"]
    assert g["t"][2] < 0 and o_t[2] < 0
    assert np.array_equal(g["prim"][:2], o_prim[:2])
