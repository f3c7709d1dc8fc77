"""The normal-estimation oracle against analytic answers (CPU)."""
import numpy as np

import normals_oracle


def test_sphere_normals_are_radial_towards_the_viewpoint():
    rng = np.random.default_rng(7)
    p = rng.standard_normal((5000, 3))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    nrm, cond = normals_oracle.estimate_normals(p.astype(np.float32))
    # viewpoint at the centre: every normal points inwards
    assert np.all((nrm * -p).sum(axis=1) > 0.995)


def test_plane_normals():
    rng = np.random.default_rng(8)
    p = np.column_stack([rng.uniform(-1, 1, 2000), rng.uniform(-1, 1, 2000), np.full(2000, 0.5)])
    nrm, _ = normals_oracle.estimate_normals(p)
    # (viewpoint - p) . (0, 0, -1) = 0.5 > 0: all flipped towards the origin
    np.testing.assert_allclose(nrm, np.tile([0.0, 0.0, -1.0], (2000, 1)), atol=1e-9)


def test_fewer_than_three_points_have_no_normal():
    nrm, _ = normals_oracle.estimate_normals(np.zeros((2, 3)))
    assert np.all(np.isnan(nrm))
