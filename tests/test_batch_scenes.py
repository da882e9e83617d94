"""Host side of the batched workload: the seeded scene list is deterministic
and inside the stated ranges (triangles, lights, map sides, light placement)."""
import math

from globalillumination_gb300 import scenes


def test_batched_scenes_deterministic_and_in_range():
    a = scenes.batched_720p(scenes=12)
    b = scenes.batched_720p(scenes=12)
    assert [f.triangles for f in a] == [f.triangles for f in b]
    for f, g in zip(a, b):
        assert [l.eye for l in f.lights] == [l.eye for l in g.lights]
        assert 1 <= len(f.lights) <= 8 and len(f.maps) == len(f.lights)
        assert 500 <= f.triangles <= 520_000
        assert (f.camera.width, f.camera.height) == (1280, 720)
        assert f.params.kernel_order == 5
        for l, m in zip(f.lights, f.maps):
            assert m.width == m.height == l.width and m.width in (512, 1024, 2048, 4096)
            r = math.sqrt(sum(c * c for c in l.eye))
            assert abs(r - 10.0) < 1e-9
            assert l.eye[1] >= 10.0 * math.sin(math.radians(15.0)) - 1e-9


def test_batched_triangle_counts_span_the_range():
    fr = scenes.batched_720p(scenes=64)
    t = sorted(f.triangles for f in fr)
    assert t[0] < 5_000 and t[-1] > 100_000
