"""Mesh materials (triangle_closest_hit.rchit:71-81): the albedo factor times the albedo map at
the hit's interpolated texture coordinate, applied by the Lambert shading modes, against the
FP64 oracle; defaults that leave every frame as it was; the material through a serialised image.
"""
import numpy as np
import pytest

import vkhrt_gb300 as H
from hairscene import MESH, PHANTOM, OracleScene, lines_from_strands, mesh_oracle_data, oracle_geometry, sphere_mesh
from test_gpu_trace import AGREE, RGB_ABS, T_REL, frame_checks, render_both

pytestmark = pytest.mark.gpu

NU, NV = 48, 24


def _sphere_uv():
    """Per-vertex texture coordinates of sphere_mesh's (NV + 1) x (NU + 1) grid, wrapping three
    times around and twice from pole to pole, offset so that negative coordinates occur."""
    i, j = np.meshgrid(np.arange(NV + 1), np.arange(NU + 1), indexing="ij")
    return np.stack([3.0 * j / NU - 0.4, 2.0 * i / NV - 0.3], axis=-1).reshape(-1, 2).astype(np.float32)


def _scene(ctx, orc, precision=0, factor=(0.9, 0.7, 0.5, 1.0), textured=True, hair=True, seed=61):
    rng = np.random.default_rng(seed)
    v, tri, nrm = sphere_mesh(rng, nu=NU, nv=NV)
    tc = _sphere_uv()
    amap = rng.uniform(0.05, 1.0, (7, 11, 4)).astype(np.float32)
    kw = dict(texcoords=tc, albedo_map=amap) if textured else {}
    mb = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri, normals=nrm, precision=H.Precision(precision),
                    albedo_factor=factor, **kw), ctx)
    blases, obl = [mb], [(MESH, *mesh_oracle_data(v, tri, nrm))]
    if hair:
        hv, hr, hoff = H.generate_strands(H.StrandParams(seed=seed + 1, nstrands=600, nverts=24))
        hb = H.BottomLevelAccelerationStructure(
            H.BLASInput(type=H.BLASType.ePhantom, vertices=hv, radius=hr, strand_offsets=hoff,
                        precision=H.Precision(precision)), ctx)
        lines, lrad = lines_from_strands(hv, hr, hoff)
        blases.append(hb)
        obl.append((PHANTOM, *oracle_geometry(orc, PHANTOM, lines, lrad)))
    tlas = H.TopLevelAccelerationStructure(blases, ctx)
    osc = OracleScene(orc, obl)
    osc.set_material(0, factor, tc[tri].reshape(-1, 6) if textured else None, amap if textured else None)
    return blases, tlas, osc, (v, tri, tc)


@pytest.mark.parametrize("precision,shading,hair", [(0, 2, True), (1, 2, True), (0, 1, True), (1, 2, False)])
def test_textured_mesh_frame_vs_oracle(ctx, orc, precision, shading, hair):
    """A textured sphere, alone (one node format) or beside Phantom hair in one TLAS (each
    instance's own format): hits at the trace tests' bars, colours of the agreeing pixels within
    1e-4."""
    _, tlas, osc, _ = _scene(ctx, orc, precision, hair=hair)
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 200, 150, spp=1, shading=shading)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    mesh_px = (hits["inst"] == 0) & (hits["t"] >= 0)
    assert mesh_px.sum() > 1500 and (not hair or (hits["inst"] == 1).sum() > 300)
    assert st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL
    assert px_ok.mean() >= 0.999 and diff[px_ok & mesh_px].max() <= RGB_ABS
    # the hair only brings in the mixed-type kernel: its pixels meet the hair frames' bar, where a
    # grazing Phantom hit's normal can move a colour a little past 1e-4 (one pixel of 30,000 here)
    hair_ok = px_ok & ~mesh_px
    assert (diff[hair_ok] <= RGB_ABS).mean() >= 0.9995 and diff[hair_ok].max() <= 1e-3
    # the map shows: without it the mesh pixels' colours move far beyond the bar
    osc.set_material(0, (0.9, 0.7, 0.5, 1.0))
    vi, pi = H.camera_arrays(H.scene_camera(200, 150))
    o2 = osc.render(vi, pi, 200, 150, shading=shading, precision=64)
    moved = np.abs(rgba.reshape(-1, 4) - o2["fb"]).max(axis=1)[mesh_px]
    assert np.median(moved) > 0.02


def test_material_defaults_and_debug_shading_leave_frames_unchanged(ctx, orc):
    """An albedo factor of 1 without a map reproduces the frame of a mesh without a material bit
    for bit; the debug shading (the reference's output, rchit:84) ignores the material."""
    blases_a, tlas_a, _, _ = _scene(ctx, orc, factor=(1.0, 1.0, 1.0, 1.0), textured=False)
    v, tri, nrm = sphere_mesh(np.random.default_rng(61), nu=NU, nv=NV)
    mb = H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri,
                                                        normals=nrm), ctx)
    tlas_b = H.TopLevelAccelerationStructure([mb, blases_a[1]], ctx)
    cam = H.scene_camera(160, 120)
    frames = []
    for t in (tlas_a, tlas_b):
        fr = H.Frame(ctx, 160, 120, 1)
        H.trace(ctx, t, cam, fr, H.trace_params(shading=2))
        frames.append(fr.download())
    assert np.array_equal(frames[0], frames[1])
    _, tlas_c, _, _ = _scene(ctx, orc)  # textured
    dbg = []
    for t in (tlas_b, tlas_c):
        fr = H.Frame(ctx, 160, 120, 1)
        H.trace(ctx, t, cam, fr, H.trace_params(shading=0))
        dbg.append(fr.download())
    assert np.array_equal(dbg[0], dbg[1])


def test_textured_mesh_through_a_serialised_image(ctx, orc):
    """The material travels in the BLAS image: a loaded copy renders the same frame bit for bit,
    and its per-triangle texture coordinates are the input's, gathered by triangle."""
    blases, tlas, _, (v, tri, tc) = _scene(ctx, orc, hair=False)
    got = blases[0].get(H.Part.TRI_TEXCOORDS, np.float32, (len(tri), 6))
    assert np.array_equal(got, tc[tri].reshape(-1, 6))
    img = blases[0].serialize()
    copy = H.BottomLevelAccelerationStructure.load(img, ctx)
    tlas2 = H.TopLevelAccelerationStructure([copy], ctx)
    cam = H.scene_camera(128, 96)
    out = []
    for t in (tlas, tlas2):
        fr = H.Frame(ctx, 128, 96, 1)
        H.trace(ctx, t, cam, fr, H.trace_params(shading=2))
        out.append(fr.download())
    assert np.array_equal(out[0], out[1])
    assert copy.info["device_bytes"] == blases[0].info["device_bytes"]


@pytest.mark.parametrize("shape", [(0, 4, 4), (4, 20000, 4)])
def test_albedo_map_sizes_are_checked(ctx, shape):
    v, tri, nrm = sphere_mesh(np.random.default_rng(3), nu=8, nv=4)
    i, j = np.meshgrid(np.arange(5), np.arange(9), indexing="ij")
    tc = np.stack([j / 8.0, i / 4.0], axis=-1).reshape(-1, 2).astype(np.float32)
    with pytest.raises(H.HrtError) as e:
        H.BottomLevelAccelerationStructure(H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri, texcoords=tc,
                                                       albedo_map=np.zeros(shape, np.float32)), ctx)
    assert e.value.status == 1


def test_textured_mesh_instance_with_a_transform(ctx, orc):
    """The albedo of a scaled, rotated and moved mesh instance: the shading weights come from the
    object-space ray, as the oracle's do."""
    rng = np.random.default_rng(71)
    v, tri, nrm = sphere_mesh(rng, nu=NU, nv=NV)
    tc = _sphere_uv()
    amap = rng.uniform(0.05, 1.0, (9, 5, 4)).astype(np.float32)
    factor = (0.8, 0.9, 0.6, 1.0)
    c, s = np.cos(0.6), np.sin(0.6)
    xf = np.array([[1.3 * c, 0, 1.3 * s, 0.2], [0, 1.3, 0, -0.1], [-1.3 * s, 0, 1.3 * c, 0.3], [0, 0, 0, 1]],
                  np.float32)
    mb = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=H.BLASType.eMesh, vertices=v, tri_indices=tri, normals=nrm, transform=xf,
                    albedo_factor=factor, texcoords=tc, albedo_map=amap), ctx)
    tlas = H.TopLevelAccelerationStructure([mb], ctx)
    osc = OracleScene(orc, [(MESH, *mesh_oracle_data(v, tri, nrm))], [xf])
    osc.set_material(0, factor, tc[tri].reshape(-1, 6), amap)
    fr, rgba, hits, o = render_both(ctx, tlas, osc, 160, 120, spp=1, shading=2)
    st, px_ok, diff = frame_checks(rgba, hits, o, 1)
    assert st["hits"] > 1000 and st["agreement"] >= AGREE and st["p9999_rel_t"] <= T_REL
    assert px_ok.mean() >= 0.999 and diff[px_ok].max() <= RGB_ABS
