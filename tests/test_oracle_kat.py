"""The reference's own known-answer test: test_intersection_point.f90:8-38
calls find_intersection_point for a rectilinear face and for the same face
plane given by three skewed points; both must give (1.0, 0.5, 0.5).  The
oracle's restatement (find_intersection_point.f90:39-56) is pinned here; the
same vectors are checked on the GPU in test_gpu_geometry.py."""
import numpy as np
import pytest

# (plane points p1,p2,p3, line points p4,p5) of test_intersection_point.f90:8-20 and :24-36
KAT = [
    ([1.0, 1.0, 1.0, 1.0, 0.0, 1.0, 1.0, 1.0, 0.0, 0.5, 0.5, 0.5, 1.5, 0.5, 0.5], [1.0, 0.5, 0.5]),
    ([1.0, 1.25, 1.0, 1.0, 0.25, 1.0, 1.0, 1.25, 0.0, 0.5, 0.5, 0.5, 1.5, 0.5, 0.5], [1.0, 0.5, 0.5]),
]


@pytest.mark.parametrize("pts,expected", KAT)
def test_find_intersection_point_kat(oracle_mod, pts, expected):
    got = oracle_mod.find_intersection_point(pts)
    # the determinant formula is exact for these dyadic inputs
    np.testing.assert_array_equal(got, expected)


def test_intersection_general_plane(oracle_mod):
    """A point found on an arbitrary plane/line lies on both."""
    rng = np.random.default_rng(7)
    for _ in range(20):
        p = rng.uniform(-1, 1, 15)
        q = oracle_mod.find_intersection_point(p)
        a, b, c, d, e = p.reshape(5, 3)
        n = np.cross(b - a, c - a)
        assert abs(np.dot(q - a, n)) < 1e-9 * (1 + np.linalg.norm(n) * np.linalg.norm(q - a))
        t = np.cross(q - d, e - d)
        assert np.linalg.norm(t) < 1e-8 * (1 + np.linalg.norm(e - d) * np.linalg.norm(q - d))
