"""Normal estimation of unoriented clouds (psr_estimate_normals) against the FP64 oracle
restating PCL's NormalEstimation (k = 10, viewpoint at the origin).

Compared where the answer is well defined: the 10th and 11th neighbour distances are not
tied (the neighbour set is unique), the two smallest covariance eigenvalues are apart
(relative gap > 0.05: the normal is well conditioned) and the viewpoint ray is not
perpendicular to the normal (the flip is decided).  There the directions agree to 1e-4.
"""
import time

import numpy as np
import pytest

import normals_oracle
import synthetic as syn

pytestmark = pytest.mark.gpu


def clouds():
    out = []
    p, _, _, _ = syn.workload("sphere20k")
    out.append(("sphere20k", p))
    p, _, _, _ = syn.workload("torus_ellipsoid200k", n=50000)
    out.append(("torus_ellipsoid50k", p))
    p, _, _, _ = syn.workload("mix", cloud=1, n=30000)
    out.append(("mix1", p))
    return out


@pytest.mark.parametrize("name,p", clouds())
def test_normals_match_oracle(name, p):
    import psr
    with psr.PoissonReconstruction(max_depth=7, max_points=60000) as r:
        g = r.CalculatePointCloudNormal(p)
    o, cond = normals_oracle.estimate_normals(p)
    m = (cond["gap"] > 0.05) & ~cond["tie"] & (cond["cos"] > 1e-3)
    assert m.mean() > 0.8, m.mean()
    assert np.all(np.isfinite(g))
    dots = (g[m].astype(np.float64) * o[m]).sum(axis=1)
    assert dots.min() > 1.0 - 1e-4, (name, dots.min())
    np.testing.assert_allclose(np.linalg.norm(g, axis=1), 1.0, atol=1e-5)


def test_host_and_device_paths_and_scale():
    import torch
    import psr
    p, _, _, _ = syn.workload("sphere20k")
    with psr.PoissonReconstruction(max_depth=7, max_points=30000) as r:
        a = r.CalculatePointCloudNormal(p)
        dev = torch.device("cuda", 0)
        x = torch.from_numpy(p).to(dev)
        out = torch.empty_like(x)
        r.estimate_normals_device(x.data_ptr(), x.shape[0], out.data_ptr())
        b = out.cpu().numpy()
        c = r.CalculatePointCloudNormal(p * 100.0)
    np.testing.assert_array_equal(a, b)
    assert ((a.astype(np.float64) * c).sum(axis=1) > 0.9999).mean() > 0.99


def test_tiny_clouds():
    import psr
    with psr.PoissonReconstruction(max_depth=7, max_points=100) as r:
        two = r.CalculatePointCloudNormal(np.array([[0, 0, 0], [1, 0, 0]], np.float32))
        assert np.all(np.isnan(two))
        rng = np.random.default_rng(3)
        five = np.column_stack([rng.uniform(-1, 1, 5), rng.uniform(-1, 1, 5), np.full(5, 2.0)]).astype(np.float32)
        n5 = r.CalculatePointCloudNormal(five)
        np.testing.assert_allclose(np.abs(n5[:, 2]), 1.0, atol=1e-5)   # a plane: all 5 points
        assert np.all(n5[:, 2] < 0)                                      # towards the origin


def test_normals_of_the_200k_cloud_feed_the_reconstruction():
    import psr
    p, nr, _, d = syn.workload("torus_ellipsoid200k")
    with psr.PoissonReconstruction(max_depth=7, max_points=200000) as r:
        r.CalculatePointCloudNormal(p)   # warm-up
        t0 = time.perf_counter()
        est = r.CalculatePointCloudNormal(p)
        dt = time.perf_counter() - t0
        print(f"normal estimation, 200k points: {1e3 * dt:.2f} ms (host arrays, copies included)")
        # the synthetic normals point outwards, the estimated ones towards the origin: the
        # directions agree up to the sign
        agree = np.abs((est * nr).sum(axis=1))
        assert np.median(agree) > 0.95
        # the reference feeds such normals to the reconstruction as they are
        mesh = r.SolvePoissionReconstructionMesh(p, est, depth=d)
        assert mesh.triangles.shape[0] > 0
