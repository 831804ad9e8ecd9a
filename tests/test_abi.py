"""The C-ABI library: builds for sm_103a, loads without a GPU and exports every declared symbol;
host-side helpers (strand generator, checksum) are deterministic."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hrt.h")

# FNV-1a 64 checksum of the default Phantom FP32 configuration's strands (2,000 x 32 vertices,
# seed 1001): fixed by the generator's definition; identical on x86-64 and aarch64.
C1_CHECKSUM = 0x5BCFA8DB0563635E


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\*]+\s+)+\**(hrt_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    import vkhrt_gb300 as H
    lib = H.load()
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
        assert name in H.SIGNATURES, f"{name} has no Python binding"


def test_abi_version_and_status_strings():
    import vkhrt_gb300 as H
    lib = H.load()
    assert lib.hrt_abi_version() == 10 == H.ABI_VERSION
    assert lib.hrt_status_string(0) == b"ok"
    assert lib.hrt_status_string(4) == b"traversal stack overflow"
    assert lib.hrt_status_string(7) == b"device index check failed"


def test_strand_generator_is_deterministic():
    import vkhrt_gb300 as H
    v, r, off = H.generate_strands(H.StrandParams())
    assert v.shape == (64000, 3) and r.shape == (64000,) and off[-1] == 64000
    assert H.checksum(v, r) == C1_CHECKSUM
    v2, r2, _ = H.generate_strands(H.StrandParams())
    assert np.array_equal(v, v2) and np.array_equal(r, r2)
    # roots on the unit-sphere cap, polar angle < 60 degrees about +y
    roots = v[off[:-1]]
    assert np.allclose(np.linalg.norm(roots, axis=1), 1.0, atol=1e-6)
    assert (roots[:, 1] >= 0.5 - 1e-6).all()
    # taper 0.004 -> 0.001
    assert abs(r[0] - 0.004) < 1e-9 and abs(r[31] - 0.001) < 1e-9
    # step length ~0.05 plus curl
    d = np.linalg.norm(np.diff(v[:32], axis=0), axis=1)
    assert (d > 0.03).all() and (d < 0.07).all()


def test_camera_matches_glm_conventions():
    import vkhrt_gb300 as H
    cam = H.look_at((0, 0, 3), (0, 0, 0), (0, 1, 0), 40.0, 1.0)
    vi, pi = H.camera_arrays(cam)
    V = vi.reshape(4, 4).T  # row-major
    assert np.allclose(V @ np.array([0, 0, 0, 1]), [0, 0, 3, 1], atol=1e-6)  # eye
    Pm = np.linalg.inv(pi.reshape(4, 4).T.astype(np.float64))
    f = 1 / np.tan(np.radians(20))
    assert np.isclose(Pm[0, 0], f, rtol=1e-6) and np.isclose(Pm[1, 1], -f, rtol=1e-6)  # Y flipped
    assert np.isclose(Pm[3, 2], -1.0)


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes mirror of an hrt.h structure has the C compiler's size and field offsets."""
    import ctypes
    import subprocess
    import vkhrt_gb300 as H
    mirrors = {"hrt_blas_input": H.BLASInputC, "hrt_blas_info": H.BLASInfoC, "hrt_camera": H.CameraC,
               "hrt_trace_params": H.TraceParamsC, "hrt_frame_stats": H.FrameStatsC,
               "hrt_scene_desc": H.SceneDescC, "hrt_strand_params": H.StrandParamsC}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "hrt.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            cf = "async" if f == "async_" else f
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {cf}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = str(tmp_path / "layout")
    r = subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, f, v = line.split()
        got[(cname, f)] = int(v)
    for cname, cls in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
