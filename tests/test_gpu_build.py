"""Device BVH build vs the CPU oracle: every integer and FP32 stage bit for bit.

Geometry processing (GenerateCurves, DOTS vertices, LSS radii, the quantised strand vertex stream),
primitive boxes, Morton codes, the stable sort, the Karras hierarchy, the refit, the BVH8
collapse (topology, child boxes, leaf order) and the 8-bit node quantisation.
"""
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import (DOTS, LSS, MESH, PHANTOM, P, lines_from_strands, mesh_oracle_data, oracle_geometry, oracle_voxels,
                       ref_boxes, sphere_mesh, strand_stream)

pytestmark = pytest.mark.gpu

NODEF = np.dtype([("lo_x", "<f4", 8), ("hi_x", "<f4", 8), ("lo_y", "<f4", 8), ("hi_y", "<f4", 8),
                  ("lo_z", "<f4", 8), ("hi_z", "<f4", 8), ("child_base", "<u4"), ("prim_base", "<u4"),
                  ("imask", "<u4"), ("pad0", "<u4"), ("meta", "u1", 8), ("pad", "<u4", 2)])
NODEQ = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"), ("prim_base", "<u4"),
                  ("meta", "u1", 8), ("qlo_x", "u1", 8), ("qhi_x", "u1", 8), ("qlo_y", "u1", 8), ("qhi_y", "u1", 8),
                  ("qlo_z", "u1", 8), ("qhi_z", "u1", 8)])
assert NODEF.itemsize == 224 and NODEQ.itemsize == 80


def oracle_bvh(orc, boxes, max_leaf, width=8):
    n = len(boxes)
    out = dict(codes=np.zeros(n, np.uint64), srt=np.zeros(n, np.uint32), L=np.zeros(max(n - 1, 0), np.uint32),
               R=np.zeros(max(n - 1, 0), np.uint32), F=np.zeros(max(n - 1, 0), np.uint32),
               La=np.zeros(max(n - 1, 0), np.uint32), pi=np.zeros(max(n - 1, 0), np.uint32),
               pl=np.zeros(n, np.uint32), nb=np.zeros((max(n - 1, 0), 6), np.float32))
    orc.orc_lbvh(P(boxes), n, *[P(out[k]) for k in ("codes", "srt", "L", "R", "F", "La", "pi", "pl", "nb")])
    mx = max(n, 1)
    w = dict(cb=np.zeros(mx, np.uint32), pb=np.zeros(mx, np.uint32), meta=np.zeros((mx, 8), np.uint8),
             cbox=np.zeros((mx, 8, 6), np.float32), order=np.zeros(n, np.uint32), qp=np.zeros((mx, 3), np.float32),
             qe=np.zeros((mx, 3), np.uint8), qlo=np.zeros((mx, 3, 8), np.uint8), qhi=np.zeros((mx, 3, 8), np.uint8))
    nn = orc.orc_bvh8(P(boxes), n, max_leaf | (width << 8), mx, *[P(w[k]) for k in ("cb", "pb", "meta", "cbox", "order", "qp", "qe",
                                                                    "qlo", "qhi")])
    out.update(w)
    out["nn"] = nn
    return out


def rebuild_curves(ent, first):
    """The control points a quantised Phantom leaf rebuilds from stream entries first .. first + 3
    (GenerateCurves, tension 1, every float32 operation rounded separately)."""
    k = np.float32(1.0) / np.float32(6.0)
    p0, p1, p2, p3 = (ent[first + j, :3] for j in range(4))
    return np.ascontiguousarray(np.concatenate([p1, p1 + (p2 - p0) * k, p2 - (p3 - p1) * k, p2], axis=1), np.float32)


def check_blas(ctx, orc, gtype, precision, v, r, off, max_leaf=1, line_indices=None, const_radius=0.02, width=0):
    inp = H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r, strand_offsets=None if line_indices is not None else off,
                      line_indices=line_indices, precision=H.Precision(precision), max_leaf=max_leaf,
                      const_radius=const_radius, keep_intermediate=True, width=width)
    blas = H.BottomLevelAccelerationStructure(inp, ctx)
    if line_indices is None:
        lines, lrad = lines_from_strands(v, r, off, const_radius)
    else:
        li = np.asarray(line_indices).reshape(-1, 2)
        lines = np.ascontiguousarray(np.concatenate([v[li[:, 0]], v[li[:, 1]]], axis=1), np.float32)
        lrad = np.ascontiguousarray(np.stack([r[li[:, 0]], r[li[:, 1]]], axis=1) if r is not None
                                    else np.full((len(li), 2), const_radius, np.float32), np.float32)
    n = len(lines)
    assert blas.info["nprims"] == n
    quant_prims = precision == 1 and gtype == PHANTOM
    data, rad = oracle_geometry(orc, gtype, lines, lrad)
    if n == 0:
        assert blas.info["nnodes"] == 0
        return blas
    if gtype == PHANTOM:
        ref_curves = np.zeros((n, 12), np.float32)
        orc.orc_generate_curves(P(lines), n, P(ref_curves))
        assert blas.get(H.Part.CURVES, np.float32, (n, 12)).tobytes() == ref_curves.tobytes()
    elif gtype == LSS:
        g = blas.get(H.Part.LSS, np.float32, (n, 8))
        assert g[:, :6].tobytes() == np.ascontiguousarray(data).tobytes()
        assert np.ascontiguousarray(g[:, 6:]).tobytes() == rad.tobytes()
    else:
        assert blas.get(H.Part.DOTS_VERTICES, np.float32, (n, 36)).tobytes() == data.tobytes()
    o = check_tree(blas, orc, ref_boxes(orc, gtype, data, rad, n), max_leaf, precision, width or 8)
    if quant_prims:
        # the strand vertex stream and each slot's first entry equal the oracle's, and the control
        # points and radii rebuilt from them are the FP32 curves bit for bit
        ent, first = strand_stream(orc, lines, lrad)
        assert blas.get(H.Part.STRAND_VERTICES, np.float32, ent.shape).tobytes() == ent.tobytes()
        recs = blas.get(H.Part.PRIMS, np.uint32, n)
        order = o["order"]
        assert np.array_equal(recs, first[order])
        assert rebuild_curves(ent, recs).tobytes() == np.ascontiguousarray(data[order]).tobytes()
        assert np.ascontiguousarray(ent[recs + 1, 3]).tobytes() == np.ascontiguousarray(rad[order, 0]).tobytes()
        assert np.ascontiguousarray(ent[recs + 2, 3]).tobytes() == np.ascontiguousarray(rad[order, 1]).tobytes()
    return blas


def check_tree(blas, orc, ref_boxes, max_leaf, precision, width=8):
    """Primitive boxes, Morton codes, sort, binary tree, BVH8 nodes (both encodings) and leaf
    order of a BLAS against the oracle built from the same boxes; returns the oracle's tree."""
    n = len(ref_boxes)
    assert blas.get(H.Part.PRIM_BOXES, np.float32, (n, 6)).tobytes() == ref_boxes.tobytes()
    o = oracle_bvh(orc, ref_boxes, max_leaf, width)
    assert np.array_equal(blas.get(H.Part.MORTON_SORTED, np.uint64, n), o["codes"])
    assert np.array_equal(blas.get(H.Part.SORTED_INDEX, np.uint32, n), o["srt"])
    if n >= 2:
        assert np.array_equal(blas.get(H.Part.BIN_LEFT, np.uint32, n - 1), o["L"])
        assert np.array_equal(blas.get(H.Part.BIN_RIGHT, np.uint32, n - 1), o["R"])
        assert blas.get(H.Part.BIN_BOXES, np.float32, (n - 1, 6)).tobytes() == o["nb"].tobytes()
    nn = o["nn"]
    assert blas.info["nnodes"] == nn
    assert np.array_equal(blas.get(H.Part.PRIM_ORDER, np.uint32, n), o["order"])
    qn = blas.get(H.Part.QNODES, np.uint8, nn * 80).view(NODEQ)
    assert np.array_equal(qn["child_base"], o["cb"][:nn]) and np.array_equal(qn["prim_base"], o["pb"][:nn])
    assert np.array_equal(qn["meta"], o["meta"][:nn])
    imask = (((o["meta"][:nn] & 0x80) != 0).astype(np.uint32) << np.arange(8, dtype=np.uint32)).sum(axis=1)
    assert np.array_equal(qn["imask"], imask.astype(np.uint8))
    assert qn["p"].tobytes() == o["qp"][:nn].tobytes() and np.array_equal(qn["e"], o["qe"][:nn])
    for k, ax in enumerate("xyz"):
        assert np.array_equal(qn["qlo_" + ax], o["qlo"][:nn, k]) and np.array_equal(qn["qhi_" + ax], o["qhi"][:nn, k])
    if precision == 0:
        fn = blas.get(H.Part.NODES, np.uint8, nn * 224).view(NODEF)
        for k, ax in enumerate("xyz"):
            assert fn["lo_" + ax].tobytes() == np.ascontiguousarray(o["cbox"][:nn, :, k]).tobytes()
            assert fn["hi_" + ax].tobytes() == np.ascontiguousarray(o["cbox"][:nn, :, 3 + k]).tobytes()
        assert np.array_equal(fn["meta"], o["meta"][:nn])
        assert np.array_equal(fn["imask"], imask)
    return o


@pytest.mark.parametrize("gtype", [PHANTOM, LSS, DOTS])
@pytest.mark.parametrize("precision", [0, 1])
def test_build_bit_exact(ctx, orc, gtype, precision):
    v, r, off = H.generate_strands(H.StrandParams(seed=5, nstrands=400, nverts=17))
    check_blas(ctx, orc, gtype, precision, v, r, off)


@pytest.mark.parametrize("width", [2, 4, 6])
def test_build_narrower_nodes_bit_exact(ctx, orc, width):
    # a node fan-out below 8 (the collapse fills `width` of the 8 slots): same bit-exact pipeline
    v, r, off = H.generate_strands(H.StrandParams(seed=6, nstrands=300, nverts=17))
    check_blas(ctx, orc, PHANTOM, 1, v, r, off, width=width)
    check_blas(ctx, orc, LSS, 0, v, r, off, width=width)


@pytest.mark.parametrize("max_leaf", [2, 3])
def test_build_multi_primitive_leaves(ctx, orc, max_leaf):
    v, r, off = H.generate_strands(H.StrandParams(seed=6, nstrands=300, nverts=9))
    check_blas(ctx, orc, PHANTOM, 0, v, r, off, max_leaf=max_leaf)


def test_build_large_bit_exact(ctx, orc):
    # 20,000 strands x 32 vertices = 620,000 segments: several radix-sort tiles and scan levels
    v, r, off = H.generate_strands(H.StrandParams(seed=9, nstrands=20000, nverts=32))
    check_blas(ctx, orc, PHANTOM, 1, v, r, off)


def test_build_reference_literal_radius(ctx, orc):
    # no per-vertex radii: the reference's constant 0.02 (geometry_processor.cpp:635)
    v, _, off = H.generate_strands(H.StrandParams(seed=8, nstrands=100, nverts=12))
    check_blas(ctx, orc, PHANTOM, 0, v, None, off, const_radius=0.02)
    check_blas(ctx, orc, DOTS, 0, v, None, off, const_radius=0.02)


def test_build_line_indices_and_runs(ctx, orc):
    # explicit index pairs (GenerateLines) in shuffled order: neighbours are only found when
    # consecutive, so the quantised strand stream has a run per joined stretch
    v, r, off = H.generate_strands(H.StrandParams(seed=10, nstrands=50, nverts=20))
    pairs = np.array([(i, i + 1) for s in range(50) for i in range(int(off[s]), int(off[s + 1]) - 1)], np.uint32)
    rng = np.random.default_rng(0)
    sh = pairs.copy()
    rng.shuffle(sh[: len(sh) // 2])
    check_blas(ctx, orc, PHANTOM, 1, v, r, off, line_indices=sh)
    check_blas(ctx, orc, LSS, 0, v, r, off, line_indices=sh)


def test_build_edge_cases(ctx, orc):
    # empty (single-vertex strands), one segment, two segments, a zero-length segment
    v = np.array([[0, 0, 0], [0, 1, 0], [0, 2, 0], [1, 0, 0], [1, 0, 0], [1, 1, 0]], np.float32)
    r = np.full(6, 0.01, np.float32)
    check_blas(ctx, orc, PHANTOM, 0, v, r, np.array([0, 1, 2, 3], np.uint32))      # no lines
    check_blas(ctx, orc, PHANTOM, 0, v, r, np.array([0, 2], np.uint32))            # one line
    check_blas(ctx, orc, LSS, 0, v, r, np.array([0, 3], np.uint32))                # two lines
    check_blas(ctx, orc, PHANTOM, 1, v, r, np.array([0, 3, 6], np.uint32))         # zero-length line
    # a joint whose two lines carry other radii (a duplicated vertex): the quantised strand
    # stream starts a new run there, and the curves still see their geometric neighbours
    v3 = np.array([[0, 0, 0], [0, 1, 0], [0, 1, 0], [0, 2, 0], [0, 3, 0]], np.float32)
    r3 = np.array([0.01, 0.02, 0.03, 0.02, 0.01], np.float32)
    check_blas(ctx, orc, PHANTOM, 1, v3, r3, None, line_indices=np.array([[0, 1], [2, 3], [3, 4]], np.uint32))


@pytest.mark.parametrize("nseg", [7, 8, 9, 16, 17, 63, 64, 65, 513])
def test_build_collapse_sizes_bit_exact(ctx, orc, nseg):
    # one strand of nseg segments: node fan-out boundaries of the collapse by cost
    v, r, off = H.generate_strands(H.StrandParams(seed=nseg, nstrands=1, nverts=nseg + 1))
    check_blas(ctx, orc, PHANTOM, 1, v, r, off)
    check_blas(ctx, orc, LSS, 0, v, r, off)


def test_build_collapse_ties_bit_exact(ctx, orc):
    # 300 identical segments (every split of the collapse costs the same) and 300 segments on
    # 30 distinct positions
    a = np.array([[0.1, 0.2, 0.3], [0.4, 0.9, 0.3]], np.float32)
    v = np.tile(a, (300, 1))
    off = np.arange(0, 601, 2, dtype=np.uint32)
    check_blas(ctx, orc, PHANTOM, 0, v, None, off)
    rng = np.random.default_rng(4)
    pos = rng.uniform(-1, 1, (30, 2, 3)).astype(np.float32)
    v2 = np.ascontiguousarray(pos[rng.integers(0, 30, 300)].reshape(-1, 3))
    check_blas(ctx, orc, DOTS, 0, v2, None, off)
    check_blas(ctx, orc, PHANTOM, 1, v2, np.full(600, 0.01, np.float32), off)


@pytest.mark.parametrize("size", [0.04, 0.1])
def test_voxel_build_bit_exact(ctx, orc, size):
    """Voxel hair: the filled voxels (boxes in grid order), the BVH over them and the records
    (box and grid index per slot) equal the oracle's."""
    v, _, off = H.generate_strands(H.StrandParams(seed=21, nstrands=80, nverts=16))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eVoxels, vertices=v, strand_offsets=off, const_radius=0.02, voxel_size=size,
                    keep_intermediate=True), ctx)
    lines, _ = lines_from_strands(v, None, off)
    m, g, vox = oracle_voxels(orc, lines, 0.02, size)
    assert blas.info["nprims"] == m and m > 100
    o = check_tree(blas, orc, np.ascontiguousarray(vox[:, :6]), 1, 0)
    recs = blas.get(H.Part.PRIMS, np.float32, (m, 8))
    assert np.array_equal(recs[:, 3].view(np.uint32), vox[o["order"], 6].view(np.uint32))
    assert np.ascontiguousarray(recs[:, :3]).tobytes() == np.ascontiguousarray(vox[o["order"], :3]).tobytes()
    with pytest.raises(H.HrtError):
        blas.refit(v)  # moved strands fill other voxels: a voxel BLAS is rebuilt


def test_build_rejects_bad_input(ctx):
    v = np.zeros((4, 3), np.float32)
    with pytest.raises(H.HrtError) as e:
        H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v,
                                                       strand_offsets=np.array([0, 5], np.uint32)), ctx)
    assert e.value.status == 1
    with pytest.raises(H.HrtError) as e:
        H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v,
                                                       line_indices=np.array([[0, 9]], np.uint32)), ctx)
    assert e.value.status == 1
    with pytest.raises(H.HrtError):
        H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.ePhantom, vertices=v, max_leaf=4,
                                                       strand_offsets=np.array([0, 4], np.uint32)), ctx)


def test_blas_keeps_only_what_tracing_reads(ctx):
    """Without HRT_BUILD_KEEP_INTERMEDIATE a BLAS holds nodes, records, the strand vertex stream
    and the slot map only: the quantised Phantom BLAS is 80 B per node + 4 B per segment (record)
    + 4 B per segment (slot map) + 16 B per stream entry (segments + 3 per strand), and inspection
    parts are refused."""
    v, r, off = H.generate_strands(H.StrandParams(seed=5, nstrands=300, nverts=32))
    n = 300 * 31
    # strands of 31 segments: 34 stream entries per strand
    for prec, node_b, prim_b, nent in ((H.Precision.QUANTISED, 80, 4, 300 * 34), (H.Precision.FP32, 224, 64, 0)):
        blas = H.BottomLevelAccelerationStructure(
            H.BLASInput(type=H.BLASType.ePhantom, vertices=v, radius=r, strand_offsets=off, precision=prec), ctx)
        info = blas.info
        assert info["device_bytes"] == info["nnodes"] * node_b + n * prim_b + n * 4 + nent * 16
        with pytest.raises(H.HrtError) as e:
            blas.get(H.Part.CURVES, np.float32, (n, 12))
        assert e.value.status == 6 or "not kept" in str(e.value)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("with_normals", [True, False])
def test_mesh_build_bit_exact(ctx, orc, precision, with_normals):
    """Triangle-mesh BLAS: boxes, tree and nodes bit for bit against the oracle; records hold the
    triangle's vertices, its vertex normals (or none) and its index as the primitive id."""
    rng = np.random.default_rng(41)
    v, tri, nrm = sphere_mesh(rng)
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri, normals=nrm if with_normals else None,
                    precision=H.Precision(precision), keep_intermediate=True), ctx)
    n = len(tri)
    assert blas.info["nprims"] == n and blas.info["prim_bytes"] == 80
    data, nd = mesh_oracle_data(v, tri, nrm)
    ref_boxes = np.zeros((n, 6), np.float32)
    orc.orc_prim_boxes(MESH, P(data), None, n, P(ref_boxes))
    o = check_tree(blas, orc, ref_boxes, 1, precision)
    rec = blas.get(H.Part.PRIMS, np.float32, (n, 20))
    order = o["order"]
    assert rec[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]].tobytes() == np.ascontiguousarray(data[order]).tobytes()
    assert np.array_equal(rec[:, 3].view(np.uint32), order)
    if with_normals:
        assert rec[:, [7, 11, 12, 13, 14, 15, 16, 17, 18]].tobytes() == np.ascontiguousarray(nd[order]).tobytes()
        assert np.all(rec[:, 19].view(np.uint32) == 1)
    else:
        assert np.all(rec[:, 19].view(np.uint32) == 0)
    with pytest.raises(H.HrtError):  # indices past the vertices
        H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.eMesh, vertices=v[:10], tri_indices=tri), ctx)


def _numpy_refit(nodes, prim_order, boxes):
    """Slot boxes of a BVH8 after a refit, from its structure and new primitive boxes: a leaf
    slot is the union of its primitives' boxes, an internal slot its child's union (exact)."""
    nn = len(nodes)
    lo = np.full((nn, 8, 3), np.inf, np.float32)
    hi = np.full((nn, 8, 3), -np.inf, np.float32)
    nb = np.zeros((nn, 6), np.float32)
    for i in range(nn - 1, -1, -1):
        for q in range(8):
            m = int(nodes["meta"][i, q])
            if m & 0x80:
                c = int(nodes["child_base"][i]) + (m & 7)
                lo[i, q], hi[i, q] = nb[c, :3], nb[c, 3:]
            elif m:
                s = [int(prim_order[int(nodes["prim_base"][i]) + (m & 31) + j]) for j in range(m >> 5)]
                lo[i, q], hi[i, q] = boxes[s, :3].min(axis=0), boxes[s, 3:].max(axis=0)
        used = nodes["meta"][i] != 0
        nb[i, :3], nb[i, 3:] = lo[i, used].min(axis=0), hi[i, used].max(axis=0)
    return lo, hi, nb


@pytest.mark.parametrize("gtype", [PHANTOM, LSS, DOTS])
def test_refit_boxes_exact(ctx, orc, gtype):
    """hrt_blas_refit on moved strands: primitive boxes equal the oracle's for the new geometry
    and every node's slot boxes are the exact unions over the kept tree."""
    v, r, off = H.generate_strands(H.StrandParams(seed=8, nstrands=300, nverts=17))
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType(gtype), vertices=v, radius=r, strand_offsets=off, keep_intermediate=True), ctx)
    rng = np.random.default_rng(9)
    v2 = (v + 0.05 * np.sin(3.0 * v[:, [1, 2, 0]] + rng.uniform(0, 6.28, 3))).astype(np.float32)
    blas.refit(v2, r)
    n = blas.info["nprims"]
    lines, lrad = lines_from_strands(v2, r, off)
    data, rad = oracle_geometry(orc, gtype, lines, lrad)
    rb = ref_boxes(orc, gtype, data, rad, n)
    assert blas.get(H.Part.PRIM_BOXES, np.float32, rb.shape).tobytes() == rb.tobytes()
    nn = blas.info["nnodes"]
    fn = blas.get(H.Part.NODES, np.uint8, nn * 224).view(NODEF)
    lo, hi, nb = _numpy_refit(fn, blas.get(H.Part.PRIM_ORDER, np.uint32, len(rb)), rb)
    for k, ax in enumerate("xyz"):
        assert fn["lo_" + ax].tobytes() == np.ascontiguousarray(lo[:, :, k]).tobytes()
        assert fn["hi_" + ax].tobytes() == np.ascontiguousarray(hi[:, :, k]).tobytes()
    assert np.array_equal(np.array(blas.info["bounds"], np.float32), nb[0])
    with pytest.raises(H.HrtError):  # radii were given at the build
        blas.refit(v2, None)
