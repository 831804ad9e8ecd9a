"""Known-answer and property tests of the CPU oracle (no GPU)."""
import ctypes

import numpy as np
import pytest

from hairscene import DOTS, LSS, PHANTOM, P, OracleScene, lines_from_strands, strand_stream


def test_prhi_straight_curve_known_answer(orc):
    # straight curve along x at y = z = 0; a ray down -z at x = 0.3 meets the tube at z = r
    st = ctypes.c_int()
    curve = np.array([0, 0, 0, 1 / 3, 0, 0, 2 / 3, 0, 0, 1, 0, 0], np.float64)
    ray = np.array([0.3, 0.0, 5.0, 0.0, 0.0, -1.0], np.float64)
    nrm = np.zeros(3)
    t = orc.orc_prhi_f64(P(ray), P(curve), 0.02, 0.02, P(nrm), ctypes.byref(st))
    assert st.value == 1
    assert abs(t - 4.98) < 1e-9
    assert np.allclose(nrm, [0, 0, 1], atol=1e-6)
    # tapered radius 0.01 -> 0.03: at x = 0.3 the radius is 0.016
    t = orc.orc_prhi_f64(P(ray), P(curve), 0.01, 0.03, P(nrm), ctypes.byref(st))
    assert st.value == 1 and abs(t - (5.0 - 0.016)) < 1e-6


def test_prhi_axis_parallel_ray_is_a_miss(orc):
    # ray along the axis of a straight curve: c = 0 in cone.glsl:55 gives NaN -> no report
    st = ctypes.c_int()
    curve = np.array([0, 0, 0, 0, 0, 1 / 3, 0, 0, 2 / 3, 0, 0, 1], np.float32)
    ray = np.array([0, 0, -5, 0, 0, 1], np.float32)
    nrm = np.zeros(3, np.float32)
    t = orc.orc_prhi_f32(P(ray), P(curve), 0.02, 0.02, P(nrm), ctypes.byref(st))
    assert t == 0.0 and st.value != 1


def test_lss_known_answers(orc):
    # one swept sphere from (0,0,0) r=0.1 to (1,0,0) r=0.2
    data = np.array([[0, 0, 0, 1, 0, 0]], np.float32)
    rad = np.array([[0.1, 0.2]], np.float32)
    sc = OracleScene(orc, [(LSS, data, rad)])
    rays = np.array([
        [-5, 0, 0, 1, 0, 0],      # along the axis: hits the start sphere at x = -0.1
        [6, 0, 0, -1, 0, 0],      # from the other side: end sphere at x = 1.2
        [0.5, 5, 0, 0, -1, 0],    # side: tangent cone, analytic below
        [0.5, 5, 0.5, 0, -1, 0],  # miss
    ], np.float32)
    t, prim, inst, nrm = sc.trace_rays(rays)
    assert abs(t[0] - 4.9) < 1e-6 and abs(t[1] - 4.8) < 1e-6  # radii are float32
    # side hit on the tangent cone: in the xy-plane the surface is the outer common tangent
    # y = m x + c of the circles (0,0; 0.1) and (1,0; 0.2): c = 0.1 s, m + c = 0.2 s, s = sqrt(1+m^2)
    m = np.sqrt(0.01 / 0.99)
    c = 0.1 * np.sqrt(1 + m * m)
    assert abs(t[2] - (5.0 - (m * 0.5 + c))) < 1e-6
    assert np.allclose(nrm[2], [-m / np.sqrt(1 + m * m), 1 / np.sqrt(1 + m * m), 0], atol=1e-6)
    assert t[3] < 0


def test_triangle_dots_known_answer(orc):
    # one vertical DOTS segment along +y from the origin, radius 0.05
    lines = np.array([[0, 0, 0, 0, 1, 0]], np.float32)
    verts = np.zeros((1, 36), np.float32)
    orc.orc_generate_dots(P(lines), None, 0.05, 1, P(verts))
    sc = OracleScene(orc, [(DOTS, verts, np.zeros((1, 2), np.float32))])
    rays = np.array([[0.01, 0.5, 5, 0, 0, -1], [0.2, 0.5, 5, 0, 0, -1]], np.float32)
    t, prim, inst, _ = sc.trace_rays(rays)
    assert t[1] < 0
    assert t[0] > 4.9 and (prim[0] >> 2) == 0


def _random_boxes(rng, n):
    c = rng.random((n, 3)).astype(np.float32) * 4 - 2
    e = (rng.random((n, 3)) * 0.05).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([c - e, c + e], axis=1), np.float32)


@pytest.mark.parametrize("n,max_leaf", [(1, 1), (2, 1), (3, 2), (1000, 1), (1000, 3), (5000, 2)])
def test_bvh8_properties(orc, n, max_leaf):
    rng = np.random.default_rng(n + max_leaf)
    boxes = _random_boxes(rng, n)
    if n > 10:
        boxes[10:20] = boxes[10]  # duplicate boxes -> duplicate Morton codes
    mx = max(n, 1)
    cb = np.zeros(mx, np.uint32)
    pb = np.zeros(mx, np.uint32)
    meta = np.zeros((mx, 8), np.uint8)
    cbox = np.zeros((mx, 8, 6), np.float32)
    order = np.zeros(n, np.uint32)
    qp = np.zeros((mx, 3), np.float32)
    qe = np.zeros((mx, 3), np.uint8)
    qlo = np.zeros((mx, 3, 8), np.uint8)
    qhi = np.zeros((mx, 3, 8), np.uint8)
    nn = orc.orc_bvh8(P(boxes), n, max_leaf, mx, P(cb), P(pb), P(meta), P(cbox), P(order), P(qp), P(qe), P(qlo), P(qhi))
    assert nn > 0
    # every primitive exactly once
    assert np.array_equal(np.sort(order), np.arange(n))
    seen_nodes = {0}
    for i in range(nn):
        poff = 0
        rank = 0
        for q in range(8):
            m = int(meta[i, q])
            if m == 0:  # an empty slot holds an empty box
                assert np.all(cbox[i, q, :3] == np.inf) and np.all(cbox[i, q, 3:] == -np.inf)
                continue
            if m & 0x80:
                assert (m & 7) == rank  # internal children are numbered in slot order
                rank += 1
                child = int(cb[i]) + (m & 7)
                assert child < nn and child not in seen_nodes
                seen_nodes.add(child)
                # the child's boxes lie inside this slot's box
                inner = cbox[child][meta[child] != 0]
                assert (inner[:, :3] >= cbox[i, q, :3]).all() and (inner[:, 3:] <= cbox[i, q, 3:]).all()
            else:
                cnt, off = m >> 5, m & 31
                assert 1 <= cnt <= max_leaf and off == poff
                poff += cnt
                for j in range(cnt):
                    b = boxes[order[int(pb[i]) + off + j]]
                    assert (b[:3] >= cbox[i, q, :3]).all() and (b[3:] <= cbox[i, q, 3:]).all()
            # quantised box is conservative: p + q 2^e (one rounding) encloses the FP32 box
            for k in range(3):
                s = np.float32(2.0 ** (int(qe[i, k]) - 127))
                lo = np.float32(qp[i, k]) + np.float32(qlo[i, k, q]) * s
                hi = np.float32(qp[i, k]) + np.float32(qhi[i, k, q]) * s
                assert lo <= cbox[i, q, k] and hi >= cbox[i, q, 3 + k]
    assert len(seen_nodes) == nn


def test_karras_ranges(orc):
    rng = np.random.default_rng(11)
    n = 3000
    boxes = _random_boxes(rng, n)
    boxes[100:140] = boxes[100]
    codes = np.zeros(n, np.uint64)
    srt = np.zeros(n, np.uint32)
    L = np.zeros(n - 1, np.uint32)
    R = np.zeros(n - 1, np.uint32)
    F = np.zeros(n - 1, np.uint32)
    La = np.zeros(n - 1, np.uint32)
    pi = np.zeros(n - 1, np.uint32)
    pl = np.zeros(n, np.uint32)
    nb = np.zeros((n - 1, 6), np.float32)
    orc.orc_lbvh(P(boxes), n, P(codes), P(srt), P(L), P(R), P(F), P(La), P(pi), P(pl), P(nb))
    assert np.all(codes[1:] >= codes[:-1])
    assert np.array_equal(np.sort(srt), np.arange(n))
    leaf = 0x80000000

    def rng_of(c):
        return (c & ~leaf, c & ~leaf) if c & leaf else (F[c], La[c])

    for i in range(n - 1):
        a0, a1 = rng_of(int(L[i]))
        b0, b1 = rng_of(int(R[i]))
        assert a0 == F[i] and b1 == La[i] and a1 + 1 == b0
    assert F[0] == 0 and La[0] == n - 1
    # root box = union of all boxes
    assert np.array_equal(nb[0, :3], boxes[:, :3].min(0)) and np.array_equal(nb[0, 3:], boxes[:, 3:].max(0))


def test_bvh8_slots_follow_direction(orc):
    """Eight leaf boxes at the corners of a cube land in the slot of their octant."""
    corners = [(x, y, z) for z in (0, 1) for y in (0, 1) for x in (0, 1)]
    rng = np.random.default_rng(5)
    perm = rng.permutation(8)
    boxes = np.array([[10 * c[0], 10 * c[1], 10 * c[2], 10 * c[0] + 1, 10 * c[1] + 1, 10 * c[2] + 1]
                      for c in np.array(corners)[perm]], np.float32)
    mx = 8
    cb = np.zeros(mx, np.uint32)
    pb = np.zeros(mx, np.uint32)
    meta = np.zeros((mx, 8), np.uint8)
    cbox = np.zeros((mx, 8, 6), np.float32)
    order = np.zeros(8, np.uint32)
    qp = np.zeros((mx, 3), np.float32)
    qe = np.zeros((mx, 3), np.uint8)
    qlo = np.zeros((mx, 3, 8), np.uint8)
    qhi = np.zeros((mx, 3, 8), np.uint8)
    nn = orc.orc_bvh8(P(boxes), 8, 1, mx, P(cb), P(pb), P(meta), P(cbox), P(order), P(qp), P(qe), P(qlo), P(qhi))
    assert nn == 1
    for s in range(8):
        lo = cbox[0, s, :3]
        assert tuple(int(v > 5) for v in lo) == ((s & 1), (s >> 1) & 1, (s >> 2) & 1)


def test_mesh_triangle_known_answer(orc):
    """One triangle in the z = 1 plane, a ray down -z through a known point: t, id and the
    barycentric interpolation of its vertex normals (triangle_closest_hit.rchit:19-41)."""
    from hairscene import OracleScene
    tri = np.array([[0, 0, 1, 1, 0, 1, 0, 1, 1]], np.float32)
    nrm = np.array([[0, 0, 1, 1, 0, 0, 0, 1, 0]], np.float32)  # n0 = +z, n1 = +x, n2 = +y
    osc = OracleScene(orc, [(3, tri, nrm)])
    rays = np.array([[0.25, 0.5, 3.0, 0.0, 0.0, -1.0]], np.float32)  # hits at (0.25, 0.5, 1): b1 0.25, b2 0.5
    t, prim, inst, n = osc.trace_rays(rays, precision=64)
    assert abs(t[0] - 2.0) < 1e-12 and prim[0] == 0 and inst[0] == 0
    expect = np.array([0.25, 0.5, 0.25])  # w n0 + b1 n1 + b2 n2 with w = 0.25
    assert np.allclose(n[0], expect / np.linalg.norm(expect), atol=1e-12)
    osc2 = OracleScene(orc, [(3, tri, None)])  # no normals: the face normal
    t2, _, _, n2 = osc2.trace_rays(rays, precision=64)
    assert abs(t2[0] - 2.0) < 1e-12 and np.allclose(np.abs(n2[0]), [0, 0, 1])
    boxes = np.zeros((1, 6), np.float32)
    orc.orc_prim_boxes(3, P(tri), None, 1, P(boxes))
    assert boxes.tolist() == [[0, 0, 1, 1, 1, 1]]


def _bilinear_repeat(m, s, t):
    """Bilinear lookup with repeat addressing, texel centres at (i + 0.5) / size (numpy)."""
    hgt, wid = m.shape[:2]
    s = s - np.floor(s)
    t = t - np.floor(t)
    x, y = s * wid - 0.5, t * hgt - 0.5
    fx, fy = np.floor(x), np.floor(y)
    ax, ay = (x - fx)[:, None], (y - fy)[:, None]
    x0, y0 = fx.astype(np.int64) % wid, fy.astype(np.int64) % hgt
    x1, y1 = (x0 + 1) % wid, (y0 + 1) % hgt
    m = m.astype(np.float64)
    lo = m[y0, x0, :3] + ax * (m[y0, x1, :3] - m[y0, x0, :3])
    hi = m[y1, x0, :3] + ax * (m[y1, x1, :3] - m[y1, x0, :3])
    return lo + ay * (hi - lo)


def test_mesh_material_albedo_known_answer(orc):
    """triangle_closest_hit.rchit:71-81 restated: a quad in the z = 0 plane whose texture
    coordinates are an affine function of position, stretched past [0, 1) and negative so the
    repeat addressing wraps, with a 5 x 3 map. Lambert shading of a face normal along z gives the
    ambient 0.3 times the albedo; the albedo must equal the factor times a numpy bilinear lookup
    at the hit point's coordinate (FP64 oracle to 1e-9, FP32 oracle to 1e-5). Without a map the
    albedo is the factor alone; HRT_SHADE_DEBUG ignores the material."""
    from hairscene import OracleScene
    import vkhrt_gb300 as H
    quad = np.array([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], np.float32)  # covers the view
    tri = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    scale, off = np.array([2.5, 1.75]), np.array([-0.75, 0.3])
    tc = ((quad[:, :2] + 2.0) * 0.25 * scale + off).astype(np.float32)
    rng = np.random.default_rng(8)
    amap = rng.uniform(0.1, 1.0, (3, 5, 4)).astype(np.float32)
    factor = (0.9, 0.6, 0.8, 1.0)
    osc = OracleScene(orc, [(3, quad[tri].reshape(-1, 9), None)])
    osc.set_material(0, factor, tc[tri].reshape(-1, 6), amap)
    w, h = 16, 12
    vi, pi = H.camera_arrays(H.scene_camera(w, h, lib=H.bind_workload(orc)))
    o64 = osc.render(vi, pi, w, h, shading=1, precision=64)
    o32 = osc.render(vi, pi, w, h, shading=1, precision=32)
    assert (o64["t"] > 0).all() and (o64["prim"] <= 1).all()
    ro, rd = np.zeros(3, np.float32), np.zeros(3, np.float32)
    hitp = []
    for p in range(w * h):
        orc.orc_raygen_f32(P(vi), P(pi), p % w, p // w, w, h, ctypes.c_float(0.5), ctypes.c_float(0.5), P(ro), P(rd))
        hitp.append(ro.astype(np.float64) + o64["t"][p] * rd.astype(np.float64))
    hitp = np.array(hitp)
    uv = (hitp[:, :2] + 2.0) * 0.25 * scale + off
    expect = 0.3 * np.asarray(factor[:3]) * _bilinear_repeat(amap, uv[:, 0], uv[:, 1])
    assert np.abs(o64["fb"][:, :3] - expect).max() < 1e-6  # the FP32 framebuffer of FP64 colours
    assert np.abs(o32["fb"][:, :3] - expect).max() < 1e-5
    plain = OracleScene(orc, [(3, quad[tri].reshape(-1, 9), None)])
    plain.set_material(0, factor)
    assert np.allclose(plain.render(vi, pi, w, h, shading=1, precision=64)["fb"][:, :3],
                       0.3 * np.asarray(factor[:3]), atol=1e-7)
    dbg = osc.render(vi, pi, w, h, shading=0, precision=64)["fb"]
    unlit = OracleScene(orc, [(3, quad[tri].reshape(-1, 9), None)]).render(vi, pi, w, h, shading=0, precision=64)["fb"]
    assert np.array_equal(dbg, unlit)


def test_environment_map_miss(orc):
    """miss.rmiss:17-37 on an empty scene: a constant map gives 1 - exp(-c) under gamma 1/2.2;
    a map that varies only in u shows the direction -> (u, v) mapping and the bilinear blend."""
    from hairscene import OracleScene
    import vkhrt_gb300 as H
    osc = OracleScene(orc, [(0, np.zeros((0, 12), np.float32), np.zeros((0, 2), np.float32))])
    cam = H.scene_camera(8, 6)
    vi, pi = H.camera_arrays(cam)
    env = np.full((4, 8, 4), 0.7, np.float32)
    o = osc.render(vi, pi, 8, 6, shading=2, precision=64, env=env)
    expect = (1.0 - np.exp(-0.7)) ** (1.0 / 2.2)
    assert np.allclose(o["fb"][:, :3], expect, atol=1e-6) and np.all(o["t"] == -1.0)
    # the camera looks down -z, so -d points to +z: theta = atan2(x, -z) = +-pi -> u at the seam
    ramp = np.zeros((4, 8, 4), np.float32)
    ramp[:, :, 0] = np.arange(8)[None, :]
    o2 = osc.render(vi, pi, 8, 6, shading=2, precision=64, env=ramp)
    centre = o2["fb"].reshape(6, 8, 4)[3, 4, 0]
    c_lin = -np.log(1.0 - centre ** 2.2)  # undo the tone map
    assert 0.0 <= c_lin <= 7.0  # a blend of the ramp's texels around the seam (u = 0 / 1)


def _bvh8_nodes(orc, boxes, max_leaf=1):
    n = len(boxes)
    mx = max(n, 1)
    arrs = [np.zeros(mx, np.uint32), np.zeros(mx, np.uint32), np.zeros((mx, 8), np.uint8),
            np.zeros((mx, 8, 6), np.float32), np.zeros(n, np.uint32), np.zeros((mx, 3), np.float32),
            np.zeros((mx, 3), np.uint8), np.zeros((mx, 3, 8), np.uint8), np.zeros((mx, 3, 8), np.uint8)]
    nn = orc.orc_bvh8(P(np.ascontiguousarray(boxes, np.float32)), n, max_leaf, mx, *[P(a) for a in arrs])
    return nn, arrs[2][:max(nn, 0)], arrs[4]


@pytest.mark.parametrize("n", [2, 5, 8])
def test_collapse_by_cost_one_node_up_to_eight(orc, n):
    """Up to 8 primitives: one wide node with every primitive in a leaf slot (any extra node
    adds its own surface area to the cost)."""
    rng = np.random.default_rng(n)
    lo = rng.uniform(0, 10, (n, 3)).astype(np.float32)
    boxes = np.concatenate([lo, lo + rng.uniform(0.1, 1, (n, 3)).astype(np.float32)], axis=1)
    nn, meta, order = _bvh8_nodes(orc, boxes)
    assert nn == 1
    assert np.count_nonzero(meta[0]) == n and not (meta[0] & 0x80).any()
    assert np.array_equal(np.sort(order), np.arange(n))


def test_collapse_by_cost_nine_and_ties(orc):
    """Nine primitives need two wide nodes; identical boxes (every split costs the same) still
    give a valid tree with every primitive once and full nodes."""
    rng = np.random.default_rng(9)
    lo = rng.uniform(0, 10, (9, 3)).astype(np.float32)
    boxes = np.concatenate([lo, lo + 0.5], axis=1)
    nn, meta, order = _bvh8_nodes(orc, boxes)
    assert nn == 2 and np.count_nonzero(meta) == 9 + 1
    same = np.tile(np.float32([[0, 0, 0, 1, 1, 1]]), (200, 1))
    nn, meta, order = _bvh8_nodes(orc, same)
    assert np.array_equal(np.sort(order), np.arange(200))
    # 200 leaves in nodes of 8 slots: at least 29 nodes; ties must not degrade to tiny nodes
    assert 29 <= nn <= 40


def _voxelize(orc, lines, r=0.02, size=0.1, mx=200000):
    lines = np.ascontiguousarray(lines, np.float32).reshape(-1, 6)
    g = np.zeros(8, np.float32)
    out = np.zeros((mx, 7), np.float32)
    m = orc.orc_voxelize(P(lines), len(lines), ctypes.c_float(r), ctypes.c_float(size), P(g), P(out), mx)
    return m, g, out[:max(m, 0)]


def test_voxelize_known_answers(orc):
    """Capsule voxelisation: an axis-aligned segment fills its row; a zero-length one fills
    nothing; a diagonal one covers every point along it and its radius across the minor axes."""
    m, g, v = _voxelize(orc, [0.05, 0.05, 0.05, 0.95, 0.05, 0.05])
    assert m == 10 and tuple(g[4:7]) == (10, 1, 1)
    assert np.array_equal(v[:, 6].view(np.uint32), np.arange(10, dtype=np.uint32))
    assert np.allclose(v[:, 0], 0.03 + 0.1 * np.arange(10), atol=1e-6) and np.allclose(v[:, 3] - v[:, 0], 0.1)
    m, g, v = _voxelize(orc, [0.3, 0.3, 0.3, 0.3, 0.3, 0.3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.05])
    ids = set(v[:, 6].view(np.uint32).tolist())
    assert all(i < 4 for i in ids)  # only the short segment's cells (grid 4 x 4 x 4 from the first point)
    p0, p1 = np.array([0.0, 0.0, 0.0]), np.array([1.0, 1.0, 0.5])
    m, g, v = _voxelize(orc, np.concatenate([p0, p1]), r=0.04)
    res = g[4:7].astype(int)
    ids = set(v[:, 6].view(np.uint32).tolist())
    axis = (p1 - p0) / np.linalg.norm(p1 - p0)
    perp = np.cross(axis, [0, 0, 1.0])
    perp /= np.linalg.norm(perp)
    for t in np.linspace(0, 1, 101):
        for off in (0.0, 0.039, -0.039):
            pt = p0 + t * (p1 - p0) + off * perp
            ijk = np.floor((pt - g[:3]) / g[3]).astype(int)
            assert int(ijk[0] + ijk[1] * res[0] + ijk[2] * res[0] * res[1]) in ids, (t, off)
    # boxes come in ascending grid index and tile the grid exactly
    gi = v[:, 6].view(np.uint32)
    assert np.all(np.diff(gi.astype(np.int64)) > 0)


@pytest.mark.parametrize("gtype", [LSS, DOTS])
def test_two_reference_boxes_cover_each_segment(orc, gtype):
    """LSS and DOTS segments enter the BVH as two references: the boxes of the segment's halves
    (reference 2 i + h). Their union is the segment's own box bit for bit, the two halves share
    their midpoint face, and their surface area is smaller; Phantom keeps one reference."""
    import vkhrt_gb300 as H
    from hairscene import lines_from_strands, oracle_geometry, ref_boxes
    v, r, off = H.generate_strands(H.StrandParams(seed=31, nstrands=120, nverts=17))
    lines, lrad = lines_from_strands(v, r, off)
    n = len(lines)
    data, rad = oracle_geometry(orc, gtype, lines, lrad)
    seg = np.zeros((n, 6), np.float32)
    orc.orc_prim_boxes(gtype, P(np.ascontiguousarray(data)), P(np.ascontiguousarray(rad)), n, P(seg))
    h = ref_boxes(orc, gtype, data, rad, n).reshape(n, 2, 6)
    union = np.concatenate([np.minimum(h[:, 0, :3], h[:, 1, :3]), np.maximum(h[:, 0, 3:], h[:, 1, 3:])], axis=1)
    assert union.tobytes() == seg.tobytes()
    assert np.all(h[:, :, :3] <= h[:, :, 3:])
    # the halves overlap in a slab through the midpoint (no gap between them on any axis)
    assert np.all(np.maximum(h[:, 0, :3], h[:, 1, :3]) <= np.minimum(h[:, 0, 3:], h[:, 1, 3:]))

    def area(b):
        d = b[..., 3:] - b[..., :3]
        return d[..., 0] * d[..., 1] + d[..., 1] * d[..., 2] + d[..., 0] * d[..., 2]
    assert area(h).sum() < 0.8 * area(seg).sum()
    ph_data, ph_rad = oracle_geometry(orc, PHANTOM, lines, lrad)
    ph_seg = np.zeros((n, 6), np.float32)
    orc.orc_prim_boxes(PHANTOM, P(ph_data), P(ph_rad), n, P(ph_seg))
    assert ref_boxes(orc, PHANTOM, ph_data, ph_rad, n).tobytes() == ph_seg.tobytes()


def _rebuild(ent, first):
    k = np.float32(1.0) / np.float32(6.0)
    p0, p1, p2, p3 = (ent[first + j, :3] for j in range(4))
    return np.ascontiguousarray(np.concatenate([p1, p1 + (p2 - p0) * k, p2 - (p3 - p1) * k, p2], axis=1), np.float32)


@pytest.mark.parametrize("case", ["strands", "shuffled", "radius_joint", "touching_strands", "single"])
def test_strand_stream_rebuilds_the_curves(orc, case):
    """The quantised Phantom format keeps the strands' FP32 vertices (the strand vertex stream);
    the control points rebuilt from entries e .. e + 3 of each line equal GenerateCurves' output
    bit for bit, and entries e + 1, e + 2 carry the line's end radii."""
    rng = np.random.default_rng(11)
    if case == "single":
        lines = np.array([[0, 0, 0, 1, 0, 0]], np.float32)
        lrad = np.array([[0.01, 0.02]], np.float32)
    elif case == "radius_joint":  # joined lines whose radii differ at the joint
        lines = np.array([[0, 0, 0, 0, 1, 0], [0, 1, 0, 0, 2, 0], [0, 2, 0, 0, 3, 0]], np.float32)
        lrad = np.array([[0.01, 0.02], [0.03, 0.02], [0.02, 0.01]], np.float32)
    elif case == "touching_strands":  # strand 2 starts where strand 1 ends: GenerateCurves joins them
        v = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [2, 0, 0], [2, 1, 0], [2, 2, 0]], np.float32)
        lines, lrad = lines_from_strands(v, np.full(6, 0.01, np.float32), np.array([0, 3, 6]))
    else:
        ns, nv = 40, 9
        v = rng.normal(size=(ns * nv, 3)).astype(np.float32)
        r = rng.uniform(0.001, 0.01, ns * nv).astype(np.float32)
        lines, lrad = lines_from_strands(v, r, np.arange(0, ns * nv + 1, nv))
        if case == "shuffled":
            idx = np.arange(len(lines))
            rng.shuffle(idx[: len(idx) // 2])
            lines, lrad = np.ascontiguousarray(lines[idx]), np.ascontiguousarray(lrad[idx])
    n = len(lines)
    curves = np.zeros((n, 12), np.float32)
    orc.orc_generate_curves(P(lines), n, P(curves))
    ent, first = strand_stream(orc, lines, lrad)
    assert _rebuild(ent, first).tobytes() == curves.tobytes()
    assert np.ascontiguousarray(ent[first + 1, 3]).tobytes() == np.ascontiguousarray(lrad[:, 0]).tobytes()
    assert np.ascontiguousarray(ent[first + 2, 3]).tobytes() == np.ascontiguousarray(lrad[:, 1]).tobytes()
    # runs: 3 extra entries each; a joint with other radii on its two sides starts a run
    if case == "radius_joint":
        assert len(ent) == n + 3 * 2
    if case == "touching_strands":
        assert len(ent) == n + 3


@pytest.mark.parametrize("spread", [0.01, 0.004])
def test_shifted_origin_fp64_agrees_with_the_literal_fp64_prhi(orc, spread):
    """The oracle of record (precision code 64) evaluates Prhi in FP64 from the ray point nearest
    the chord midpoint; the golden vectors pin the literal FP64 evaluation (code 6400).
    * From 0.3 units away the two give the same closest hit on every aimed ray.
    * From 3 units away the literal form misses a few grazing hits (about 1 in 1,000): its
      bounding-cylinder test (hair_intersection.rint:29) rounds in proportion to the squared
      distance of the origin. Moved 0.3 units in front of the hair, the same rays give the literal
      form the shifted form's hits on every one of them, so the two differ only in that rounding."""
    import vkhrt_gb300 as H
    from hairscene import aimed_rays, compare_hits, oracle_geometry
    v, r, off = H.generate_strands(H.StrandParams(seed=1004, nstrands=400, nverts=64, r_root=0.003, r_tip=0.0008),
                                   lib=H.bind_workload(orc))
    lines, lrad = lines_from_strands(v, r, off)
    sc = OracleScene(orc, [(PHANTOM, *oracle_geometry(orc, PHANTOM, lines, lrad))])
    for dist in (0.3, 3.0):
        rays = aimed_rays(np.random.default_rng(64), lines, 20000, spread=spread, dist=dist)
        a = sc.trace_rays(rays, precision=64)
        b = sc.trace_rays(rays, precision=6400)
        st = compare_hits(a[0], a[1], a[2], b[0], b[1], b[2])
        assert st["hits"] > 5000 and st["p9999_rel_t"] <= 1e-6, st
        if dist < 1.0:
            assert st["mismatches"] == 0, st
            continue
        assert st["agreement"] >= 0.999, st
        idx = st["mism_idx"]
        assert (a[0][idx] >= 0).all()  # the shifted form finds a hit on every disputed ray
        near = rays[idx].copy()
        near[:, :3] += near[:, 3:] * np.float32(dist - 0.3)
        c = sc.trace_rays(near, precision=6400)
        assert np.array_equal(c[1][c[0] >= 0], a[1][idx][c[0] >= 0]) and (c[0] >= 0).all()


def test_scaled_instance_phantom_distances_are_ray_parameters(orc):
    """A transformed instance's object-space ray is o + t d with |d| != 1 under scaling. The
    oracle runs Prhi on the unit direction and converts its length to the parameter t, so a
    uniformly scaled, rotated and moved Phantom instance hits exactly where the same curves
    transformed into world space (radii scaled alike) are hit."""
    import vkhrt_gb300 as H
    from hairscene import aimed_rays, compare_hits, oracle_geometry
    v, r, off = H.generate_strands(H.StrandParams(seed=90, nstrands=200, nverts=16), lib=H.bind_workload(orc))
    lines, lrad = lines_from_strands(v, r, off)
    curves, rad = oracle_geometry(orc, PHANTOM, lines, lrad)
    s = 0.2
    c, sn = np.cos(0.7), np.sin(0.7)
    xf = np.array([[s * c, 0, s * sn, 0.3], [0, s, 0, -0.1], [-s * sn, 0, s * c, 0.2], [0, 0, 0, 1]], np.float64)
    world = (curves.reshape(-1, 3).astype(np.float64) @ xf[:3, :3].T + xf[:3, 3]).reshape(-1, 12).astype(np.float32)
    a = OracleScene(orc, [(PHANTOM, curves, rad)], [xf.astype(np.float32)])
    b = OracleScene(orc, [(PHANTOM, world, (rad * np.float32(s)).astype(np.float32))])
    wl = (lines.reshape(-1, 3).astype(np.float64) @ xf[:3, :3].T + xf[:3, 3]).reshape(-1, 6).astype(np.float32)
    rays = aimed_rays(np.random.default_rng(2), wl, 10000, spread=0.001)
    ta, pa, ia, _ = a.trace_rays(rays, precision=64)
    tb, pb, ib, _ = b.trace_rays(rays, precision=64)
    st = compare_hits(ta, pa, ia, tb, pb, ib)
    assert st["hits"] > 2000 and st["agreement"] >= 0.999 and st["p9999_rel_t"] <= 1e-6, st
