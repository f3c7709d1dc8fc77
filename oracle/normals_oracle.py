"""Test oracle for the normal estimation stage (test infrastructure only; nothing in the
product path imports it).

The reference estimates normals of unoriented clouds with PCL before the path
(mesh/PoissonReconstruction.cpp:137-161, CalculatePointCloudNormal):
pcl::NormalEstimationOMP with a kd-tree, setKSearch(10), the default viewpoint (0, 0, 0).
PCL (1.12.1 in the reference's build notes, README.md:23) is a third-party dependency
absent from the reference tree; its published algorithm
(pcl::computePointNormal / flipNormalTowardsViewpoint) is restated here in FP64:

* the k nearest samples of a point, the point itself included;
* their centroid and covariance;
* the eigenvector of the covariance's smallest eigenvalue as the normal;
* flipped when (viewpoint - point) . normal < 0;
* fewer than 3 points: no normal (NaN).

Parity pinned on analytic shapes (tests/test_normals_oracle.py: a sphere's normals are
radial, a plane's are its normal), not on PCL's own output (not runnable here).
"""
import numpy as np


def estimate_normals(xyz, k=10, viewpoint=(0.0, 0.0, 0.0)):
    """Returns (normals float64 N x 3, conditioning dict).  conditioning["gap"]: relative gap
    between the two smallest eigenvalues; conditioning["tie"]: the k-th and (k+1)-th
    neighbour distances nearly equal (the neighbour set is then ambiguous)."""
    from scipy.spatial import cKDTree
    p = np.asarray(xyz, np.float64).reshape(-1, 3)
    n = p.shape[0]
    out = np.full((n, 3), np.nan)
    cond = {"gap": np.zeros(n), "tie": np.zeros(n, bool), "cos": np.zeros(n)}
    if n < 3:
        return out, cond
    kk = min(k, n)
    kq = min(k + 1, n)
    tree = cKDTree(p)
    d, idx = tree.query(p, k=kq)
    d = d.reshape(n, kq)
    idx = idx.reshape(n, kq)
    if kq > kk:
        cond["tie"] = np.abs(d[:, kk] - d[:, kk - 1]) <= 1e-5 * np.maximum(d[:, kk], 1e-30)
    nb = p[idx[:, :kk]]
    mu = nb.mean(axis=1, keepdims=True)
    q = nb - mu
    cov = np.einsum("nki,nkj->nij", q, q) / kk
    w, v = np.linalg.eigh(cov)
    nrm = v[:, :, 0]
    vp = np.asarray(viewpoint, np.float64)
    cosv = ((vp - p) * nrm).sum(axis=1)
    nrm = np.where((cosv < 0.0)[:, None], -nrm, nrm)
    cond["gap"] = (w[:, 1] - w[:, 0]) / np.maximum(w[:, 2], 1e-300)
    cond["cos"] = np.abs(cosv) / np.maximum(np.linalg.norm(vp - p, axis=1), 1e-300)
    return nrm, cond
