"""The CPU oracle against the reference's own code (golden vectors from oracle/_ref).

tests/golden/ref_vectors.npz holds inputs and outputs of the reference's shader math and host
geometry processing compiled as C++ (tests/golden/gen_golden.py). The oracle's FP32 and FP64
restatements must reproduce them bit for bit.
"""
import os

import numpy as np
import pytest

from hairscene import P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_prhi_fp32_bit_exact(orc, gold):
    rays, curves = gold["prhi_rays"], gold["prhi_curves"]
    import ctypes
    st = ctypes.c_int()
    bad = 0
    for i in range(len(rays)):
        nrm = np.zeros(3, np.float32)
        t = orc.orc_prhi_f32(P(rays[i]), P(curves[i]), 0.02, 0.02, P(nrm), ctypes.byref(st))
        if np.float32(t).tobytes() != gold["prhi_t32"][i].tobytes() or \
                (t > 0 and nrm.tobytes() != gold["prhi_n32"][i].tobytes()):
            bad += 1
    assert bad == 0
    assert (gold["prhi_t32"] > 0).sum() > 1000  # the vectors exercise hits as well as misses


def test_prhi_fp64_bit_exact(orc, gold):
    import ctypes
    st = ctypes.c_int()
    rays = gold["prhi_rays"].astype(np.float64)
    curves = gold["prhi_curves"].astype(np.float64)
    bad = 0
    for i in range(len(rays)):
        nrm = np.zeros(3)
        t = orc.orc_prhi_f64(P(rays[i]), P(curves[i]), 0.02, 0.02, P(nrm), ctypes.byref(st))
        if t != gold["prhi_t64"][i] or (t > 0 and not np.array_equal(nrm, gold["prhi_n64"][i])):
            bad += 1
    assert bad == 0


def test_shader_math_bit_exact(orc, gold):
    m = len(gold["cones"])
    for i in range(m):
        out = np.zeros(6, np.float32)
        orc.orc_cone_f32(P(gold["cones"][i]), P(out))
        assert out.tobytes() == gold["cone_out"][i].tobytes(), f"cone {i}"
        assert orc.orc_cylinder_f32(P(gold["cyl_rays"][i]), P(gold["cyls"][i])) == gold["cyl_out"][i], f"cyl {i}"
        out6 = np.zeros(6, np.float32)
        orc.orc_curve_sample_f32(P(gold["samp_curves"][i]), float(gold["samp_t"][i]), P(out6))
        assert out6.tobytes() == gold["samp_out"][i].tobytes(), f"curve sample {i}"
        m16 = np.zeros(16, np.float32)
        orc.orc_rcc_matrix_f32(P(gold["cyl_rays"][i]), P(m16))
        assert m16.tobytes() == gold["rcc_out"][i].tobytes(), f"rcc {i}"
        rgb = np.zeros(3, np.float32)
        orc.orc_shade_f32(P(gold["normals"][i]), P(rgb))
        assert rgb.tobytes() == gold["shade_out"][i].tobytes(), f"shade {i}"


def test_raygen_bit_exact(orc, gold):
    W, H = (int(x) for x in gold["rg_size"])
    for py in range(H):
        for px in range(W):
            o = np.zeros(3, np.float32)
            d = np.zeros(3, np.float32)
            orc.orc_raygen_f32(P(gold["rg_view_inv"]), P(gold["rg_proj_inv"]), px, py, W, H, 0.5, 0.5, P(o), P(d))
            assert o.tobytes() == gold["rg_o"][py, px].tobytes()
            assert d.tobytes() == gold["rg_d"][py, px].tobytes()


def test_geometry_processing_bit_exact(orc, gold):
    lines = gold["geo_lines"]
    n = len(lines)
    curves = np.zeros((n, 12), np.float32)
    orc.orc_generate_curves(P(lines), n, P(curves))
    assert curves.tobytes() == gold["geo_curves"].tobytes()
    aabbs = np.zeros((n, 6), np.float32)
    orc.orc_generate_aabbs(P(curves), n, 0.02, P(aabbs))
    assert aabbs.tobytes() == gold["geo_aabbs"].tobytes()
    dl = gold["geo_dots_lines"]
    dots = np.zeros((len(dl), 36), np.float32)
    orc.orc_generate_dots(P(dl), None, 0.02, len(dl), P(dots))
    assert dots.tobytes() == gold["geo_dots"].reshape(len(dl), 36).tobytes()
    assert np.array_equal(gold["geo_dots_idx"], np.arange(12 * len(dl)))
    pos = np.zeros((2 * n, 3), np.float32)
    rad = np.zeros(2 * n, np.float32)
    orc.orc_generate_lss(P(lines), n, 0.0005, P(pos), P(rad))
    assert pos.tobytes() == gold["geo_lss_p"].tobytes()
    assert rad.tobytes() == gold["geo_lss_r"].tobytes()


def test_live_reference_random(orc):
    """Where oracle/_ref is built (reference checkout present), fresh random cases too."""
    from oracle import build
    ref = build.load_ref()
    if ref is None:
        pytest.skip("oracle/_ref not built here")
    import ctypes
    rng = np.random.default_rng(7)
    st = ctypes.c_int()
    for _ in range(3000):
        c = (rng.normal(size=(4, 3)) * 0.05).astype(np.float32)
        c[1:] += c[0]
        org = (rng.normal(size=3) * 2).astype(np.float32)
        tgt = c[0] + (c[3] - c[0]) * rng.random() + rng.normal(size=3) * 0.02
        d = (tgt - org) / np.linalg.norm(tgt - org)
        ray = np.concatenate([org, d]).astype(np.float32)
        cv = c.reshape(-1).astype(np.float32)
        n1 = np.zeros(3, np.float32)
        n2 = np.zeros(3, np.float32)
        t1 = ref.ref_prhi_f32(P(ray), P(cv), P(n1))
        t2 = orc.orc_prhi_f32(P(ray), P(cv), 0.02, 0.02, P(n2), ctypes.byref(st))
        assert np.float32(t1).tobytes() == np.float32(t2).tobytes()
        assert t1 <= 0 or n1.tobytes() == n2.tobytes()
