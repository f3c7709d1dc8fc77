"""Served form: every request's result is the same alone and in the mix.

A Server with fewer slots than requests runs clouds of different shapes, sizes and depths
concurrently (continuous batching through psr_submit / psr_poll); each result must equal,
bit for bit, the mesh the blocking psr_reconstruct produces for that cloud on its own.
"""
import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu


def clouds():
    out = []
    for k in range(4):   # the "mix" workload: sphere / torus / superquadric, random pose
        p, nr, rgb, d = syn.workload("mix", cloud=k, n=[12000, 30000, 8000, 45000][k], colour=(k % 2 == 0))
        out.append((p, nr, rgb, min(d, 7)))
    p, nr, rgb, d = syn.workload("sphere20k", cloud=3, colour=True)
    out.append((p, nr, rgb, d))
    return out


def test_served_matches_alone():
    import torch
    import psr
    from serve import Request, Server, latency_summary

    dev = torch.device("cuda", 0)
    cl = clouds()
    caps = dict(max_depth=7, max_points=60000, max_triangles=400000, max_mesh_vertices=200000,
                max_subdivision_nodes=4000000)
    srv = Server(slots=3, out_sets=10, **caps)   # results kept until the end: no set is reused
    try:
        reqs = [Request(xyz=torch.from_numpy(p).to(dev), normals=torch.from_numpy(nr).to(dev),
                        rgb=torch.from_numpy(rgb).to(dev) if rgb is not None else None, depth=d, tag=i)
                for i, (p, nr, rgb, d) in enumerate(cl)]
        done = srv.run(reqs + [Request(xyz=r.xyz, normals=r.normals, rgb=r.rgb, depth=r.depth, tag=("again", r.tag))
                               for r in reqs])
    finally:
        srv.close()
    assert len(done) == 2 * len(cl)
    assert all(not r.error for r in done), [r.error for r in done]
    assert latency_summary(done)["p99_ms"] > 0
    by_tag = {r.tag: r for r in done}
    with psr.PoissonReconstruction(compute_colors=True, compute_normals=True, **caps) as alone:
        for i, (p, nr, rgb, d) in enumerate(cl):
            m = alone.SolvePoissionReconstructionMesh(p, nr, rgb, depth=d)
            for r in (by_tag[i], by_tag[("again", i)]):
                np.testing.assert_array_equal(r.vertices.cpu().numpy(), m.vertices)
                np.testing.assert_array_equal(r.triangles.cpu().numpy(), m.triangles)
                np.testing.assert_array_equal(r.normals_out.cpu().numpy(), m.normals)
                if rgb is not None:
                    np.testing.assert_array_equal(r.colors.cpu().numpy(), m.colors)
                assert r.scale == pytest.approx(m.scale, rel=0, abs=0)


def test_served_host_io_matches_alone():
    """Host-resident inputs (pinned) and outputs: the GPU reads the clouds and writes the
    meshes in pinned memory; each finished request holds views of its slot's output set,
    valid until the slot starts the out_sets-th request after it (here four sets for four
    requests, whichever slots take them)."""
    import torch
    import psr
    from serve import Request, Server

    cl = clouds()[:4]
    caps = dict(max_depth=7, max_points=60000, max_triangles=400000, max_mesh_vertices=200000,
                max_subdivision_nodes=4000000)
    srv = Server(slots=2, host_outputs=True, out_sets=4, **caps)
    try:
        reqs = [Request(xyz=torch.from_numpy(p).pin_memory(), normals=torch.from_numpy(nr).pin_memory(),
                        rgb=torch.from_numpy(rgb).pin_memory() if rgb is not None else None, depth=d, tag=i)
                for i, (p, nr, rgb, d) in enumerate(cl)]
        done = srv.run(reqs)
        assert all(not r.error for r in done), [r.error for r in done]
        by_tag = {r.tag: r for r in done}
        with psr.PoissonReconstruction(compute_colors=True, compute_normals=True, **caps) as alone:
            for i, (p, nr, rgb, d) in enumerate(cl):
                m = alone.SolvePoissionReconstructionMesh(p, nr, rgb, depth=d)
                r = by_tag[i]
                assert not r.vertices.is_cuda and r.vertices.is_pinned()
                np.testing.assert_array_equal(r.vertices.numpy(), m.vertices)
                np.testing.assert_array_equal(r.triangles.numpy(), m.triangles)
                np.testing.assert_array_equal(r.normals_out.numpy(), m.normals)
                if rgb is not None:
                    np.testing.assert_array_equal(r.colors.numpy(), m.colors)
    finally:
        srv.close()


def test_submit_poll_wait_states():
    import torch
    import psr

    dev = torch.device("cuda", 0)
    p, nr, _, d = syn.workload("sphere20k", cloud=5)
    xyz, nrm = torch.from_numpy(p).to(dev), torch.from_numpy(nr).to(dev)
    vcap, tcap = 100000, 300000
    out = [torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((tcap, 3), dtype=torch.int32, device=dev)]
    with psr.PoissonReconstruction(max_depth=6, max_points=30000, max_triangles=tcap, max_mesh_vertices=vcap,
                                   compute_colors=False, compute_normals=False) as r:
        assert r.memory_bytes() > 0
        with pytest.raises(psr.PsrError):
            r.wait()   # nothing in flight
        m = psr.PsrMesh(out[0].data_ptr(), out[1].data_ptr(), None, None, vcap, tcap, psr.PSR_DEVICE, 0, 0)
        r.submit_device(xyz.data_ptr(), nrm.data_ptr(), None, xyz.shape[0], m, depth=d)
        with pytest.raises(psr.PsrError):   # one reconstruction in flight per handle
            r.submit_device(xyz.data_ptr(), nrm.data_ptr(), None, xyz.shape[0], m, depth=d)
        while not r.poll():
            pass
        assert m.vertex_count > 0 and m.triangle_count > 0
        ref = r.SolvePoissionReconstructionMesh(p, nr, None, depth=d)
        np.testing.assert_array_equal(out[0][:m.vertex_count].cpu().numpy(), ref.vertices)
        np.testing.assert_array_equal(out[1][:m.triangle_count].cpu().numpy(), ref.triangles)
