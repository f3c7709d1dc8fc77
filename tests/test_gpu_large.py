"""The 2M-point, depth-9 superquadric (the precision-study workload) at full size.

Too large for the CPU oracle inside a test run, so it is checked through properties that
do not depend on size: the octree's full-sibling structure, per-depth CG residuals below
the tolerance, a mesh with valid indices inside the unit cube, determinism (two runs are
bit-identical), and the iso-value equal to the mean implicit value at the samples.

With the reference's Laplacian drop threshold (1e-6) the depth-9 stencil loses its edge
and corner entries and the system is indefinite, so CG runs to its iteration cap there;
the run below keeps every entry (laplacian_epsilon = 0), which leaves depths 0-8 unchanged.
114k coarse leaves carry surface; with the cells of certain sign left out, subdivision
builds about 4.9M nodes (the full subtrees would be 92M), hence the capacities.
"""
import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu


def test_superquadric_2m_depth9_properties():
    import psr
    p, nr, _, D = syn.workload("superquadric2m")
    assert D == 9 and p.shape[0] == 2000000
    with psr.PoissonReconstruction(max_depth=9, max_points=2000000, max_triangles=12000000,
                                   max_mesh_vertices=6000000, max_subdivision_nodes=8000000,
                                   compute_normals=True, laplacian_epsilon=0.0) as r:
        a = r.SolvePoissionReconstructionMesh(p, nr, depth=D)
        st = r.stats()
        assert st.error_bits == 0
        assert 0 < st.subdivision_nodes <= 8000000
        # octree: every level below the root is made of whole sibling groups
        lc = np.array(st.level_count[:D + 1])
        assert lc[0] == 1 and np.all(lc[1:] % 8 == 0)
        assert st.nodes == lc.sum()
        # CG: every depth that iterated stopped at the tolerance, not at the iteration cap
        for d in range(D + 1):
            if st.cg_iterations[d] > 0:
                assert st.cg_iterations[d] < 10000, d
                assert st.cg_residual[d] <= 1e-5 * 1.0001, (d, st.cg_residual[d])
        # mesh
        v, t = a.vertices, a.triangles
        assert t.shape[0] > 100000
        assert np.all(np.isfinite(v)) and v.min() > 0.0 and v.max() < 1.0
        assert t.min() >= 0 and t.max() < v.shape[0]
        assert np.all(np.isfinite(a.normals))
        b = r.SolvePoissionReconstructionMesh(p, nr, depth=D)
        np.testing.assert_array_equal(a.vertices, b.vertices)
        np.testing.assert_array_equal(a.triangles, b.triangles)
        # the iso-value is the mean implicit value at the samples
        pv = r.debug("point_val", np.float32)
        assert pv.shape[0] == p.shape[0]
        assert abs(float(pv.astype(np.float64).mean()) - st.iso_value) <= 1e-5 * abs(st.iso_value)
