"""The benchmark workloads are deterministic and have the stated shapes (no GPU needed)."""
import math

import vkhrt_gb300 as H


def test_batch_workload_shape_and_determinism():
    a = H.batch_workload()
    assert a == H.batch_workload()
    assert len(a) == 16
    assert {int(m["type"]) for m in a} == {0, 1, 2}
    for m in a:
        assert 2000 <= m["nstrands"] <= 200000
        assert m["nverts"] in (16, 32, 64, 128)
        assert 256 <= m["width"] <= 1920 and 256 <= m["height"] <= 1080
        assert 1 <= m["spp"] <= 4
        # width and height sit at the same fraction of their log ranges
        fw = math.log(m["width"] / 256) / math.log(1920 / 256)
        fh = math.log(m["height"] / 256) / math.log(1080 / 256)
        assert abs(fw - fh) < 0.01
    assert len({m["seed"] for m in a}) == 16


def test_orbit_camera_at_zero_angles_is_the_scene_camera():
    a = H.orbit_camera(320, 200, 0.0, 0.0)
    b = H.scene_camera(320, 200)
    assert bytes(a) == bytes(b)


def test_oracle_library_generates_the_same_workload(orc):
    """The CPU oracle's library compiles the GPU library's workload source (strands, cameras), so
    a CPU-only run traces the same inputs without loading libhrt.so: the two agree bit for bit."""
    import numpy as np
    lib = H.bind_workload(orc)
    for p in (H.StrandParams(seed=1001, nstrands=300, nverts=32),
              H.StrandParams(seed=77, nstrands=40, nverts=128, r_root=0.003, r_tip=0.0008)):
        a, b = H.generate_strands(p), H.generate_strands(p, lib=lib)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        assert H.checksum(a[0], a[1]) == H.checksum(b[0], b[1], lib=lib)
    for az, el, w, h in ((0.0, 0.0, 1920, 1080), (0.7, -0.3, 333, 257), (2.9, 0.45, 256, 256)):
        assert bytes(H.orbit_camera(w, h, az, el)) == bytes(H.orbit_camera(w, h, az, el, lib=lib))


def test_c1_strand_checksum():
    # the C1 checksum stated with the generator's definition
    v, r, _ = H.generate_strands(H.StrandParams(seed=1001, nstrands=2000, nverts=32))
    assert H.checksum(v, r) == 0x5BCFA8DB0563635E
