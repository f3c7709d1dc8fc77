"""GPU parity: every stage of the CUDA path against the CPU oracle on the same inputs.

Integer / index stages (sorted points, node arrays, neighbour tables, vertex / edge /
face records) must be bit-exact.  Floating-point stages are compared with the FP64
oracle of the same discretisation:
  vector field, divergence, CG solution : relative L2 <= 1e-5
  iso-value                             : relative error <= 1e-5
The marching-cubes stage is then checked bit for bit against the oracle's float mirror
fed with the GPU's own solution vector and iso-value (same evaluation order).
"""
import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu

REL_L2 = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def recon():
    import psr
    r = psr.PoissonReconstruction(max_depth=8, max_points=300000, compute_colors=True, compute_normals=True)
    yield r
    r.close()


def run_both(recon, oracle_mod, xyz, nrm, rgb, depth, cg_iters=0):
    rgbf = None if rgb is None else rgb.astype(np.float32) / np.float32(255.0)
    mesh = recon.SolvePoissionReconstructionMesh(xyz, nrm, rgb, depth=depth, cg_iterations=cg_iters)
    o = oracle_mod.Oracle()
    rc = o.run(xyz, nrm, rgbf, depth=depth, cg_iters=cg_iters)
    assert rc == 0
    return mesh, o


def check_octree(recon, o):
    s = o.scalars()
    M, N = s["M"], s["N"]
    st = recon.stats()
    assert st.nodes == M and st.points == N
    pos = o.get("pos").reshape(-1, 3)
    for a, nm in enumerate(("px", "py", "pz")):
        np.testing.assert_array_equal(recon.debug(nm, np.float32), pos[:, a])
    np.testing.assert_array_equal(recon.debug("point2node"), o.get("point2node"))
    for nm in ("key", "pidx", "pnum", "parent", "didx", "dnum", "depth", "enc"):
        np.testing.assert_array_equal(recon.debug(nm), o.get(nm), err_msg=nm)
    ch = o.get("children").reshape(M, 8)
    fc = np.where(ch[:, 0] >= 0, ch[:, 0], -1)
    np.testing.assert_array_equal(recon.debug("first_child"), fc)
    ctr = o.get("center").reshape(M, 3)
    for a, nm in enumerate(("ctr_x", "ctr_y", "ctr_z")):
        np.testing.assert_array_equal(recon.debug(nm, np.float32), ctr[:, a])
    nb = recon.debug("neigh", rows=27)
    np.testing.assert_array_equal(nb, o.get("neighs").reshape(M, 27).T)


def check_field_and_solve(recon, o, tol=REL_L2):
    D = recon.stats().depth
    md = o.get("count")[D]
    vf = recon.debug("vfield", np.float32, rows=3)
    assert vf.shape[1] == md
    assert rel_l2(vf.T, o.get("vfield").reshape(md, 3)) <= tol
    assert rel_l2(recon.debug("divg", np.float32), o.get("div")) <= tol
    x_gpu = recon.debug("x", np.float32)
    x_ref = o.get("x")
    assert rel_l2(x_gpu, x_ref) <= tol, rel_l2(x_gpu, x_ref)
    iso_gpu = recon.stats().iso_value
    iso_ref = o.scalars()["iso"]
    assert abs(iso_gpu - iso_ref) <= tol * abs(iso_ref)
    return x_gpu, iso_gpu


def check_geometry(recon, o):
    vr = o.get("vertex_rec").reshape(-1, 3)
    np.testing.assert_array_equal(recon.debug("v_owner"), vr[:, 0])
    np.testing.assert_array_equal(recon.debug("v_kind"), vr[:, 1])
    np.testing.assert_array_equal(recon.debug("v_depth"), vr[:, 2])
    vp = o.get("vertex_pos").reshape(-1, 3)
    for a, nm in enumerate(("v_x", "v_y", "v_z")):
        np.testing.assert_array_equal(recon.debug(nm, np.float32), vp[:, a])
    M = o.scalars()["M"]
    np.testing.assert_array_equal(recon.debug("node_vtx", rows=8), o.get("node_vertices").reshape(M, 8).T)
    er = o.get("edge_rec").reshape(-1, 2)
    np.testing.assert_array_equal(recon.debug("e_owner"), er[:, 0])
    np.testing.assert_array_equal(recon.debug("e_kind"), er[:, 1])
    np.testing.assert_array_equal(recon.debug("node_edge", rows=12), o.get("node_edges").reshape(M, 12).T)
    fr = o.get("face_rec").reshape(-1, 3)
    np.testing.assert_array_equal(recon.debug("f_owner"), fr[:, 0])
    np.testing.assert_array_equal(recon.debug("f_kind"), fr[:, 1])
    np.testing.assert_array_equal(recon.debug("f_hasparent"), fr[:, 2])
    np.testing.assert_array_equal(recon.debug("node_face", rows=6), o.get("node_faces").reshape(M, 6).T)


def check_mesh_mirror(recon, o, mesh, x_gpu, iso_gpu):
    rc = o.run_mesh32(x_gpu, iso_gpu)
    assert rc == 0
    np.testing.assert_array_equal(recon.debug("vvalue", np.float32), o.get("vvalue32"))
    ov = o.get("mesh_v").reshape(-1, 3)
    ot = o.get("mesh_t").reshape(-1, 3)
    assert mesh.vertices.shape == ov.shape, (mesh.vertices.shape, ov.shape)
    assert mesh.triangles.shape == ot.shape, (mesh.triangles.shape, ot.shape)
    np.testing.assert_array_equal(mesh.vertices, ov)
    np.testing.assert_array_equal(mesh.triangles, ot)
    if mesh.colors is not None:
        oc = o.get("vcolor").reshape(-1, 3)
        np.testing.assert_allclose(mesh.colors, oc, atol=2e-6, rtol=0)
    if mesh.normals is not None:
        on = o.get("vnormal").reshape(-1, 3)
        np.testing.assert_allclose(mesh.normals, on, atol=1e-5, rtol=0)


def full_check(recon, oracle_mod, name, n=None, cg_iters=0, depth=None):
    p, nr, rgb, D = syn.workload(name, n=n)
    if depth:
        D = depth
    mesh, o = run_both(recon, oracle_mod, p, nr, rgb, D, cg_iters)
    check_octree(recon, o)
    x_gpu, iso_gpu = check_field_and_solve(recon, o)
    check_geometry(recon, o)
    check_mesh_mirror(recon, o, mesh, x_gpu, iso_gpu)
    return mesh, o


def full_check_arrays(recon, oracle_mod, p, nr, rgb, D, cg_iters=0):
    mesh, o = run_both(recon, oracle_mod, p, nr, rgb, D, cg_iters)
    check_octree(recon, o)
    x_gpu, iso_gpu = check_field_and_solve(recon, o)
    check_geometry(recon, o)
    check_mesh_mirror(recon, o, mesh, x_gpu, iso_gpu)
    return mesh, o


@pytest.mark.parametrize("cloud", [0, 1])
def test_mix_rotated_scaled_clouds_depth7(recon, oracle_mod, cloud):
    # the batched / served workloads' clouds: random shape, rotation and scale, with colour
    p, nr, rgb, _ = syn.workload("mix", cloud=cloud, n=25000, colour=True)
    mesh, o = full_check_arrays(recon, oracle_mod, p, nr, rgb, 7)
    assert o.scalars()["ub_events"] == 0
    assert len(mesh.triangles) > 1000


@pytest.mark.parametrize("cloud", [38, 0])
def test_colour_of_vertices_far_from_every_sample(oracle_mod, cloud):
    """Serving-mix clouds whose meshes hold many vertices far from every sample: cloud 38
    (405k points, depth 7) has about 5,900 mesh vertices whose 4th nearest sample lies
    0.19-0.23 away in the unit cube, cloud 0 (12k points) about 37,000 beyond one colour-grid
    cell.  Their colours come from the far pass's descent of the cell hierarchy; the whole
    pipeline, colours included, against the oracle (exact 4 nearest by brute force)."""
    import psr
    p, nr, rgb, D = syn.workload("serve", cloud=cloud)
    assert D == 7
    caps = dict(max_depth=7, max_points=410000, compute_colors=True, compute_normals=True, laplacian_epsilon=1e-6)
    with psr.PoissonReconstruction(**caps) as r:
        mesh, o = full_check_arrays(r, oracle_mod, p, nr, rgb, D)
    assert len(mesh.vertices) > 30000


def test_laplacian_epsilon_is_applied(oracle_mod):
    # a drop threshold between the depth-6 stencil's edge (2.10e-5) and corner (2.48e-5)
    # entries: GPU and oracle drop the same entries (8 fixed CG iterations per depth)
    import psr
    p, nr, _, D = syn.workload("sphere20k", n=8000)
    eps = 2.2e-5
    x = {}
    for e in (1e-6, eps):
        with psr.PoissonReconstruction(max_depth=6, max_points=10000, laplacian_epsilon=e) as r:
            r.SolvePoissionReconstructionMesh(p, nr, None, depth=D, cg_iterations=8)
            x[e] = r.debug("x", np.float32)
    o = oracle_mod.Oracle(laplacian_epsilon=eps)
    assert o.run(p, nr, None, depth=D, cg_iters=8, stop_after=3) == 0
    assert rel_l2(x[eps], o.get("x")) <= REL_L2
    assert rel_l2(x[eps], x[1e-6]) > 10 * REL_L2   # the threshold changed the system


def test_sphere20k_depth6_eight_iterations(recon, oracle_mod):
    full_check(recon, oracle_mod, "sphere20k", cg_iters=8)


def test_small_sphere_depth5_converged(recon, oracle_mod):
    full_check(recon, oracle_mod, "sphere20k", n=4000, depth=5)


def test_torus_ellipsoid_200k_depth7(recon, oracle_mod):
    mesh, o = full_check(recon, oracle_mod, "torus_ellipsoid200k")
    assert len(mesh.triangles) > 10000


def test_two_points(recon, oracle_mod):
    p = np.array([[0, 0, 0], [1, 1, 1]], np.float32)
    n = np.array([[-1, -1, -1], [1, 1, 1]], np.float32)
    mesh, o = run_both(recon, oracle_mod, p, n, None, 4)
    check_octree(recon, o)


def test_duplicate_points(recon, oracle_mod):
    p, nr, _, _ = syn.workload("sphere20k", n=3000)
    p = np.concatenate([p, p[:500]])
    nr = np.concatenate([nr, nr[:500]])
    mesh, o = run_both(recon, oracle_mod, p, nr, None, 6)
    check_octree(recon, o)
    check_geometry(recon, o)


def test_invalid_inputs(recon):
    import psr
    p, nr, _, _ = syn.workload("sphere20k", n=1000)
    bad = p.copy()
    bad[10, 1] = np.nan
    with pytest.raises(psr.PsrError) as e:
        recon.SolvePoissionReconstructionMesh(bad, nr, depth=6)
    assert e.value.status == psr.PSR_INVALID_INPUT
    with pytest.raises(psr.PsrError) as e:
        recon.SolvePoissionReconstructionMesh(p[:0], nr[:0], depth=6)
    assert e.value.status == psr.PSR_INVALID_INPUT
    with pytest.raises(psr.PsrError) as e:
        recon.SolvePoissionReconstructionMesh(p, nr, depth=9)
    assert e.value.status == psr.PSR_INVALID_INPUT
    # the handle still works afterwards
    recon.SolvePoissionReconstructionMesh(p, nr, depth=6)


def test_capacity_exceeded():
    import psr
    p, nr, _, _ = syn.workload("sphere20k", n=5000)
    r = psr.PoissonReconstruction(max_depth=6, max_points=4000)
    with pytest.raises(psr.PsrError) as e:
        r.SolvePoissionReconstructionMesh(p, nr, depth=6)
    assert e.value.status == psr.PSR_OUT_OF_CAPACITY
    r.close()
    r = psr.PoissonReconstruction(max_depth=6, max_points=5000, max_triangles=100)
    with pytest.raises(psr.PsrError) as e:
        r.SolvePoissionReconstructionMesh(p, nr, depth=6)
    assert e.value.status == psr.PSR_OUT_OF_CAPACITY
    r.close()


def test_deterministic(recon):
    p, nr, rgb, D = syn.workload("sphere20k")
    a = recon.SolvePoissionReconstructionMesh(p, nr, rgb, depth=D)
    b = recon.SolvePoissionReconstructionMesh(p, nr, rgb, depth=D)
    np.testing.assert_array_equal(a.vertices, b.vertices)
    np.testing.assert_array_equal(a.triangles, b.triangles)


def test_root_polynomial_fallback_same_mesh():
    # subdivision roots beyond the root-polynomial capacity sum their octree chain in the
    # level scan itself: with a capacity of one root that path runs for nearly every root
    import psr
    p, nr, rgb, D = syn.workload("mix", cloud=0, n=25000, colour=True)
    caps = dict(max_depth=7, max_points=30000, compute_colors=True, compute_normals=True)
    with psr.PoissonReconstruction(**caps) as r:
        a = r.SolvePoissionReconstructionMesh(p, nr, rgb, depth=7)
        roots = r.stats().subdivision_roots
    with psr.PoissonReconstruction(root_poly_capacity=1, **caps) as r:
        b = r.SolvePoissionReconstructionMesh(p, nr, rgb, depth=7)
    assert roots > 1
    np.testing.assert_array_equal(a.vertices, b.vertices)
    np.testing.assert_array_equal(a.triangles, b.triangles)
    np.testing.assert_array_equal(a.colors, b.colors)
