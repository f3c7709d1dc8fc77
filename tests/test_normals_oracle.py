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


def test_oracle_matches_brute_force_neighbours():
    """The kd-tree query equals a brute-force search of the 10 nearest (the point itself
    included) wherever the 10th and 11th distances are not tied, and the normal equals the
    smallest eigenvector of those neighbours' covariance computed directly."""
    rng = np.random.default_rng(11)
    p = rng.standard_normal((400, 3)).astype(np.float32)
    p[:, 2] *= 0.05                                    # a noisy slab: well-defined normals
    o, cond = normals_oracle.estimate_normals(p)
    d2 = ((p[:, None, :].astype(np.float64) - p[None, :, :]) ** 2).sum(-1)
    order = np.argsort(d2, axis=1, kind="stable")[:, :10]
    for i in range(0, 400, 7):
        if cond["tie"][i]:
            continue
        nb = p[order[i]].astype(np.float64)
        c = np.cov(nb.T, bias=True)
        w, v = np.linalg.eigh(c)
        n = v[:, 0] if np.dot(-p[i], v[:, 0]) >= 0 else -v[:, 0]
        assert abs(abs(np.dot(n, o[i])) - 1.0) < 1e-9
        assert np.allclose(n, o[i], atol=1e-6) or cond["cos"][i] < 1e-6
