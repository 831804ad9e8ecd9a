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
