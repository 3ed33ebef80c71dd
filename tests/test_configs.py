"""The benchmark workloads (medimage_gb300/configs.py) hold the sizes, ranges
and seeds they are documented with, so every measured number refers to the
same inputs."""
from collections import Counter


def test_fan_slices():
    from medimage_gb300 import configs

    s1, s2 = configs.c1(), configs.c2()
    assert (s1.geom.n, s1.geom.pixel_mm, s1.geom.nviews, s1.geom.ndets, s1.i0, s1.iters) == (256, 1.0, 360, 512, 1e4, 20)
    assert (s2.geom.n, s2.geom.pixel_mm, s2.geom.nviews, s2.geom.ndets, s2.i0, s2.iters) == (512, 0.75, 720, 888, 5e3, 50)
    assert s2.n_random == 20
    for s in (s1, s2):
        assert (s.geom.sod_mm, s.geom.sdd_mm) == (541.0, 949.0)
        assert abs(s.geom.view_step_deg * s.geom.nviews - 360.0) < 1e-9


def test_uneven_batch_is_seeded_and_in_range():
    from medimage_gb300 import configs

    a, b = configs.c3(), configs.c3()
    assert len(a) == 64
    assert [(s.geom.n, s.geom.nviews, s.geom.ndets, s.i0, s.seed) for s in a] == \
           [(s.geom.n, s.geom.nviews, s.geom.ndets, s.i0, s.seed) for s in b]
    for s in a:
        assert s.geom.n in (256, 384, 512)
        assert s.geom.nviews in (360, 540, 720)
        assert s.geom.ndets in (512, 768, 888)
        assert 2e3 <= s.i0 <= 2e4
        assert s.iters == 30
        assert abs(s.geom.n * s.geom.pixel_mm - 384.0) < 1e-9  # one field of view for every grid
    # how many slices share a plan bounds what grouped projection can share
    shares = Counter((s.geom.n, s.geom.nviews, s.geom.ndets) for s in a)
    assert len(shares) == 27 and max(shares.values()) == 7


def test_cone_volume():
    from medimage_gb300 import configs

    v = configs.c4()
    g = v.geom
    assert (g.nx, g.ny, g.nz, g.voxel_mm) == (512, 512, 512, 0.2)
    assert (g.nproj, g.ndx, g.ndy, g.pitch_mm, g.sod_mm, g.sdd_mm) == (720, 768, 1024, 0.4, 600.0, 1000.0)
    assert (v.i0, v.iters) == (2e4, 10)
    small = configs.c4(n=256, nz=256).geom
    assert abs(small.nx * small.voxel_mm - g.nx * g.voxel_mm) < 1e-9  # smaller volumes keep the field of view
