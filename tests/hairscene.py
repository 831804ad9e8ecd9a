"""Test helpers: seeded hair scenes for the GPU library and the CPU oracle, and hit comparison.

The oracle (oracle/) checks the GPU results; it receives the same strands and processes them with its
own restatement of the reference's geometry code.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import build as oracle_build  # noqa: E402

PHANTOM, LSS, DOTS = 0, 1, 2


def P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def strand_stream(orc, lines: np.ndarray, lrad: np.ndarray):
    """The oracle's strand vertex stream of quantised Phantom lines: (entries (m, 4), first entry
    of each line)."""
    n = lines.shape[0]
    ent = np.zeros((n + 3 * n, 4), np.float32)
    first = np.zeros(n, np.uint32)
    m = orc.orc_strand_stream(P(np.ascontiguousarray(lines, np.float32)), P(np.ascontiguousarray(lrad, np.float32)),
                              n, P(ent), P(first))
    return np.ascontiguousarray(ent[:m]), first


def lines_from_strands(v: np.ndarray, r: np.ndarray | None, off: np.ndarray, const_r: float = 0.02):
    """Consecutive vertices of each strand form lines (n x 6) with end radii (n x 2)."""
    ls, rs = [], []
    for s in range(len(off) - 1):
        a, b = int(off[s]), int(off[s + 1])
        if b - a < 2:
            continue
        vv = v[a:b]
        ls.append(np.concatenate([vv[:-1], vv[1:]], axis=1))
        if r is None:
            rs.append(np.full((b - a - 1, 2), const_r, np.float32))
        else:
            rr = r[a:b]
            rs.append(np.stack([rr[:-1], rr[1:]], axis=1))
    if not ls:
        return np.zeros((0, 6), np.float32), np.zeros((0, 2), np.float32)
    return (np.ascontiguousarray(np.concatenate(ls), np.float32),
            np.ascontiguousarray(np.concatenate(rs), np.float32))


def oracle_geometry(orc, gtype: int, lines: np.ndarray, lrad: np.ndarray):
    """Geometry as the oracle restates it: (data, radius) in the layout orc_scene_add_blas takes.
    A quantised BLAS holds the same geometry (its Phantom leaves rebuild the FP32 curves from the
    strand vertex stream), so the oracle traces the strands' FP32 curves for either format."""
    n = lines.shape[0]
    if gtype == PHANTOM:
        curves = np.zeros((n, 12), np.float32)
        orc.orc_generate_curves(P(lines), n, P(curves))
        return curves, lrad.copy()
    if gtype == LSS:
        rad = np.where(lrad < np.float32(0.001), np.float32(0.001), lrad).astype(np.float32)
        return lines.copy(), np.ascontiguousarray(rad)
    verts = np.zeros((n, 36), np.float32)
    orc.orc_generate_dots(P(lines), P(lrad), 0.0, n, P(verts))
    return verts, np.zeros((n, 2), np.float32)


class OracleScene:
    def __init__(self, orc, blases, transforms=None):
        """blases: list of (gtype, data, radius); transforms: list of 4x4 row-major or None."""
        self.orc = orc
        self.h = orc.orc_scene_create()
        self._keep = []
        for i, (gt, data, rad) in enumerate(blases):
            d = np.ascontiguousarray(data, np.float32)
            r = None if rad is None else np.ascontiguousarray(rad, np.float32)
            self._keep += [d, r]
            b = orc.orc_scene_add_blas(self.h, gt, d.shape[0], P(d), P(r))
            xf = None if transforms is None or transforms[i] is None else \
                np.ascontiguousarray(np.asarray(transforms[i], np.float32).T.reshape(-1))
            self._keep.append(xf)
            orc.orc_scene_add_instance(self.h, b, P(xf))

    def set_material(self, blas: int, albedo=(1.0, 1.0, 1.0, 1.0), tri_uv=None, albedo_map=None):
        """A mesh BLAS's material: albedo factor, and a map (h, w, 4) sampled at the per-triangle
        texture coordinates tri_uv (ntris, 6)."""
        a = np.ascontiguousarray(albedo, np.float32)
        uv = None if tri_uv is None else np.ascontiguousarray(tri_uv, np.float32)
        m = None if albedo_map is None else np.ascontiguousarray(albedo_map, np.float32)
        self._keep += [a, uv, m]
        h, w = (0, 0) if m is None else m.shape[:2]
        assert self.orc.orc_scene_set_material(self.h, blas, P(a), P(uv), P(m), w, h) == 0

    def trace_rays(self, rays: np.ndarray, precision: int = 64, tmin=0.001, tmax=10000.0, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        t = np.zeros(n)
        prim = np.zeros(n, np.uint32)
        inst = np.zeros(n, np.uint32)
        nrm = np.zeros((n, 3))
        th = threads or max(1, self.orc.orc_hardware_threads())
        self.orc.orc_trace_rays(self.h, P(rays), n, tmin, tmax, precision, th, P(t), P(prim), P(inst), P(nrm))
        return t, prim, inst, nrm

    def render(self, view_inv, proj_inv, w, h, spp=1, jitter=0, seed=0, shading=2, precision=64, tmin=0.001,
               tmax=10000.0, shadow_tmin=1e-4, threads: int = 0, first_pixel=0, npixels=None, pixel_list=None,
               env=None):
        if pixel_list is not None:
            pixel_list = np.ascontiguousarray(pixel_list, np.uint32)
            npixels = len(pixel_list)
        npx = w * h if npixels is None else npixels
        t = np.zeros(npx * spp)
        prim = np.zeros(npx * spp, np.uint32)
        inst = np.zeros(npx * spp, np.uint32)
        sh = np.zeros(npx * spp, np.uint8)
        fb = np.zeros((npx, 4), np.float32)
        th = threads or max(1, self.orc.orc_hardware_threads())
        vi = np.ascontiguousarray(view_inv, np.float32)
        pi = np.ascontiguousarray(proj_inv, np.float32)
        e = None if env is None else np.ascontiguousarray(env, np.float32)
        eh, ew = (0, 0) if e is None else e.shape[:2]
        self.orc.orc_render(self.h, P(vi), P(pi), w, h, spp, jitter, seed, tmin, tmax, shading, shadow_tmin, precision,
                            th, first_pixel, npx, P(pixel_list), P(t), P(prim), P(inst), P(sh), P(fb), P(e), ew, eh)
        return dict(t=t, prim=prim, inst=inst, shadow=sh, fb=fb)

    def __del__(self):
        try:
            self.orc.orc_scene_destroy(self.h)
        except Exception:
            pass


def compare_hits(g_t, g_prim, g_inst, o_t, o_prim, o_inst, tie_rel=1e-5):
    """Closest-hit agreement: ids must match unless both hit within tie_rel * t (a tie)."""
    g_hit = g_t >= 0
    o_hit = o_t >= 0
    same = (g_hit == o_hit) & (~g_hit | ((g_prim == o_prim) & (g_inst == o_inst)))
    both = g_hit & o_hit
    tie = both & ~same & (np.abs(g_t - o_t) <= tie_rel * np.maximum(np.abs(o_t), 1e-30))
    mism = ~same & ~tie
    agree_both = both & same
    rel = np.abs(g_t[agree_both] - o_t[agree_both]) / o_t[agree_both] if agree_both.any() else np.zeros(0)
    n = len(g_t)
    counted = n - tie.sum()
    return dict(n=n, hits=int(o_hit.sum()), mismatches=int(mism.sum()), ties=int(tie.sum()),
                agreement=float(1.0 - mism.sum() / max(counted, 1)),
                max_rel_t=float(rel.max()) if rel.size else 0.0,
                p9999_rel_t=float(np.quantile(rel, 0.9999)) if rel.size else 0.0,
                mism_idx=np.nonzero(mism)[0])


def load_oracle():
    return oracle_build.load()


def aimed_rays(rng, lines: np.ndarray, n: int, spread: float = 0.01, dist: float = 3.0):
    """Rays from random directions aimed at points near random segments (hits and near misses)."""
    idx = rng.integers(0, lines.shape[0], n)
    a, b = lines[idx, :3], lines[idx, 3:]
    tgt = a + (b - a) * rng.random((n, 1)) + rng.normal(size=(n, 3)) * spread
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    org = tgt - d * dist
    return np.concatenate([org, d], axis=1).astype(np.float32)


MESH = 3


def sphere_mesh(rng, nu=48, nv=24, radius=0.35, bump=0.04, centre=(0.0, 0.3, 0.0)):
    """A bumpy UV sphere: vertices (nv+1)*(nu+1), triangles 2*nu*nv, smooth vertex normals
    (normalised offsets from the centre). Returns (vertices, triangle indices, normals)."""
    th = np.linspace(0.0, np.pi, nv + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, nu + 1)
    T, Ph = np.meshgrid(th, ph, indexing="ij")
    rr = radius * (1.0 + bump * rng.standard_normal(T.shape))
    pts = np.stack([rr * np.sin(T) * np.cos(Ph), rr * np.cos(T), rr * np.sin(T) * np.sin(Ph)], axis=-1)
    v = (pts.reshape(-1, 3) + np.asarray(centre)).astype(np.float32)
    n = pts.reshape(-1, 3)
    n = (n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)).astype(np.float32)
    idx = []
    for i in range(nv):
        for j in range(nu):
            a, b = i * (nu + 1) + j, i * (nu + 1) + j + 1
            c, d = (i + 1) * (nu + 1) + j, (i + 1) * (nu + 1) + j + 1
            idx.append((a, c, b))
            idx.append((b, c, d))
    return v, np.asarray(idx, np.uint32), n


def mesh_oracle_data(v, tri, nrm=None):
    """Oracle BLAS data of a mesh: 9 floats per triangle, and 9 vertex-normal floats or None."""
    data = np.ascontiguousarray(v[tri].reshape(-1, 9), np.float32)
    nd = None if nrm is None else np.ascontiguousarray(nrm[tri].reshape(-1, 9), np.float32)
    return data, nd


VOXELS = 4


def ref_boxes(orc, gtype: int, data: np.ndarray, rad: np.ndarray, n: int) -> np.ndarray:
    """The BVH reference boxes of a hair BLAS as the oracle forms them: one per segment, two (the
    segment's halves, reference 2 i + h) for LSS and DOTS."""
    out = np.zeros((n << (1 if gtype in (LSS, DOTS) else 0), 6), np.float32)
    m = orc.orc_ref_boxes(gtype, P(np.ascontiguousarray(data)), P(np.ascontiguousarray(rad)), n, P(out))
    assert m == len(out)
    return out


def oracle_voxels(orc, lines: np.ndarray, r: float, size: float, max_out: int = 1 << 21):
    """The oracle's capsule voxelisation: (count, grid [origin xyz, size, res xyz], voxels (m, 7))."""
    lines = np.ascontiguousarray(lines, np.float32).reshape(-1, 6)
    g = np.zeros(8, np.float32)
    out = np.zeros((max_out, 7), np.float32)
    m = orc.orc_voxelize(P(lines), len(lines), ctypes.c_float(r), ctypes.c_float(size), P(g), P(out), max_out)
    assert 0 <= m <= max_out
    return m, g, np.ascontiguousarray(out[:m])
