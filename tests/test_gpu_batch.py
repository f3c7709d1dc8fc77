"""Multi-cloud launches (psr_config.batch_clouds, psr_reconstruct_batch): each cloud's mesh,
colours and normals are bit-identical to the one-cloud call on the same cloud, whatever the
batch holds beside it; clouds of uneven size share one launch per kernel; a cloud that
fails (a non-finite coordinate) fails alone."""
import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu

CAPS = dict(max_depth=7, max_points=160000, compute_colors=True, compute_normals=True)


def mix_clouds(k):
    """The first k clouds of the multi-cloud mix (sizes log-uniform in [5k, 150k]; spheres,
    tori and superquadrics, randomly scaled and rotated), with colour."""
    return [syn.workload("mix", cloud=i, colour=True)[:3] for i in range(k)]


def alone(clouds, depth):
    import psr
    with psr.PoissonReconstruction(**CAPS) as r:
        return [r.SolvePoissionReconstructionMesh(p, nr, rgb, depth=depth) for p, nr, rgb in clouds]


def same(a, b):
    np.testing.assert_array_equal(a.vertices, b.vertices)
    np.testing.assert_array_equal(a.triangles, b.triangles)
    np.testing.assert_array_equal(a.colors, b.colors)
    np.testing.assert_array_equal(a.normals, b.normals)
    np.testing.assert_array_equal(a.center, b.center)
    assert a.scale == b.scale


@pytest.mark.parametrize("k,depth", [(8, 7), (3, 6)])
def test_batch_equals_alone(k, depth):
    import psr
    clouds = mix_clouds(k)
    ref = alone(clouds, depth)
    with psr.PoissonReconstruction(batch_clouds=8, **CAPS) as r:
        got = r.reconstruct_batch(clouds, depth=depth)
        for i in range(k):
            st, s = r.batch_result(i)
            assert st == psr.PSR_OK and s.points == clouds[i][0].shape[0], (i, st, s.points)
        # again, in reverse order: results follow the clouds, not the slots
        again = r.reconstruct_batch(clouds[::-1], depth=depth)
    for a, b in zip(ref, got):
        same(a, b)
    for a, b in zip(ref[::-1], again):
        same(a, b)


def test_batch_isolates_a_failing_cloud():
    import psr
    clouds = mix_clouds(4)
    bad = clouds[1][0].copy()
    bad[17, 1] = np.nan
    clouds[1] = (bad, clouds[1][1], clouds[1][2])
    ref = alone([clouds[0], clouds[2], clouds[3]], 7)
    with psr.PoissonReconstruction(batch_clouds=4, **CAPS) as r:
        got = r.reconstruct_batch(clouds, depth=7)
        assert r.batch_result(1)[0] == psr.PSR_INVALID_INPUT
        assert isinstance(got[1], psr.PsrError)
        for a, b in zip(ref, [got[0], got[2], got[3]]):
            same(a, b)
        # a one-cloud call on a batch handle runs in its first slot
        one = r.SolvePoissionReconstructionMesh(*clouds[0], depth=7)
    same(ref[0], one)


def test_batch_depth8_device_loop_equals_alone():
    """Depth 8: the finest depths of the larger clouds outgrow their clusters' shared memory
    and are solved by the device loop (a CUDA-graph while node); one loop serves every
    cloud of the pass, each cloud's depths ending on their own iteration counts.  Each mesh
    is bit-identical to the one-cloud call's, and the per-depth CG results too."""
    import psr
    # the four largest of the first 16 (the reference's algorithm cannot mesh the sparsest
    # clouds at depth 8: it reads unset vertex records, which both paths reject)
    clouds = sorted(mix_clouds(16), key=lambda c: -c[0].shape[0])[:4]
    caps = dict(CAPS, max_depth=8, max_points=160000, max_mesh_vertices=1000000, max_triangles=2000000,
                max_subdivision_nodes=4000000)
    ref, ref_st = [], []
    with psr.PoissonReconstruction(**caps) as r:
        for p, nr, rgb in clouds:
            ref.append(r.SolvePoissionReconstructionMesh(p, nr, rgb, depth=8))
            ref_st.append(r.stats())
    # the largest cloud's depth 8 has more rows than a 16-CTA cluster holds
    assert ref_st[0].level_count[8] > 16 * 7168
    with psr.PoissonReconstruction(batch_clouds=4, **caps) as r:
        got = r.reconstruct_batch(clouds, depth=8)
        for i in range(len(clouds)):
            st, s = r.batch_result(i)
            assert st == psr.PSR_OK
            assert list(s.cg_iterations) == list(ref_st[i].cg_iterations)
            assert list(s.cg_residual) == list(ref_st[i].cg_residual)
    for a, b in zip(ref, got):
        same(a, b)
