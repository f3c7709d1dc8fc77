"""Precision study on the superquadric workload (exponents 0.5 / 0.5, sinusoidal radial
displacement 0.05 at frequency 8, normals jittered by 2 degrees): the CUDA solve (FP32
operator and updates, FP64 dot products and residual norms, true-residual refinement)
against the FP64 oracle of the same octree and discretisation, relative L2 of the
solution reported per depth.

* depth 8, 300k points, with the reference's Laplacian drop threshold (1e-6) and with
  every entry kept (0): all depths of depth <= 8 are unaffected by the threshold;
* depth 9, 600k points, every entry kept.  With the 1e-6 threshold the depth-9 stencil
  loses its edge and corner entries and the system is indefinite: the reference's CG
  does not converge there (it runs to its 10,000-iteration cap), so that case is not
  compared.
* the same solve with the true residual never evaluated (cg_residual_period = -1, the
  reference's recursive residual alone) for the A/B of the refinement.

Each depth's true residual ||b - A x|| is also checked: it must end within the refinement
target, the tolerance or the floor of an FP32 solution (2^-20 ||b||), whichever is larger.

Bound: relative L2 <= 1e-5 per depth with at least 1,000 rows (smaller systems are
dominated by a handful of entries and are checked in the whole-vector norm).
"""
import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu

REL_L2 = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def solve_pair(oracle_mod, n, depth, eps, period=0):
    import psr
    p, nr, _, _ = syn.workload("superquadric2m", n=n)
    with psr.PoissonReconstruction(max_depth=depth, max_points=n, max_triangles=6000000, max_mesh_vertices=3000000,
                                   max_subdivision_nodes=8000000, laplacian_epsilon=eps,
                                   cg_residual_period=period) as r:
        r.SolvePoissionReconstructionMesh(p, nr, depth=depth)
        st = r.stats()
        x = r.debug("x", np.float32)
        b = r.debug("divg", np.float32)
        key = r.debug("key")
    o = oracle_mod.Oracle(laplacian_epsilon=eps)
    assert o.run(p, nr, depth=depth, stop_after=3) == 0
    np.testing.assert_array_equal(key, o.get("key"))   # same octree, so the same systems
    return st, (x, b), o


def per_depth(st, xb, o, depth):
    x, bvec = xb
    xr = o.get("x")
    base, count = o.get("base"), o.get("count")
    rows = []
    for d in range(depth + 1):
        b, m = int(base[d]), int(count[d])
        rows.append(dict(d=d, rows=m, err=rel_l2(x[b:b + m], xr[b:b + m]), it=int(st.cg_iterations[d]),
                         it64=int(o.get("cg_iters")[d]), r=float(st.cg_residual[d]),
                         rtrue=float(st.cg_true_residual[d]), checks=int(st.cg_residual_checks[d]),
                         restarts=int(st.cg_restarts[d]),
                         floor=2.0 ** -20 * float(np.linalg.norm(bvec[b:b + m].astype(np.float64)))))
    return rows


def report(title, rows, whole):
    print(f"\n{title}: whole-vector rel L2 {whole:.2e}")
    print(" depth    rows    rel L2   iters(gpu/fp64)  ||r|| recursive  ||b-Ax||  FP32 floor  checks restarts")
    for q in rows:
        print(f"  {q['d']:3d} {q['rows']:8d}  {q['err']:9.2e}   {q['it']:5d} / {q['it64']:5d}   {q['r']:10.2e}"
              f"  {q['rtrue']:9.2e}  {q['floor']:9.2e}   {q['checks']:3d} {q['restarts']:3d}")


@pytest.mark.parametrize("n,depth,eps", [(300000, 8, 1e-6), (300000, 8, 0.0), (600000, 9, 0.0)])
def test_solution_per_depth_against_fp64(oracle_mod, n, depth, eps):
    st, xb, o = solve_pair(oracle_mod, n, depth, eps)
    rows = per_depth(st, xb, o, depth)
    whole = rel_l2(xb[0], o.get("x"))
    report(f"superquadric {n} points, depth {depth}, laplacian_epsilon {eps}", rows, whole)
    assert whole <= REL_L2
    for q in rows:
        if q["rows"] >= 1000:
            assert q["err"] <= REL_L2, q
        if q["it"] > 0:
            assert q["it"] < 10000 and q["r"] <= 1e-5 * 1.0001, q
            # every converged depth evaluated its true residual, which ends within the
            # refinement target: the tolerance or the floor of an FP32 solution
            assert q["checks"] >= 1, q
            assert q["rtrue"] <= 2.0 * max(1e-5, q["floor"]), q


def test_refinement_ab(oracle_mod):
    """The same depth-8 solve with and without the true residual: both within the bound,
    the refined one no farther from the FP64 solution at any large depth."""
    st_a, xb_a, o = solve_pair(oracle_mod, 300000, 8, 1e-6, period=0)
    st_b, xb_b, _ = solve_pair(oracle_mod, 300000, 8, 1e-6, period=-1)
    ra, rb = per_depth(st_a, xb_a, o, 8), per_depth(st_b, xb_b, o, 8)
    report("refined (true residual every 32 iterations and at convergence)", ra, rel_l2(xb_a[0], o.get("x")))
    report("recursive residual only", rb, rel_l2(xb_b[0], o.get("x")))
    assert all(q["checks"] == 0 and q["rtrue"] <= 0 for q in rb)
    for qa, qb in zip(ra, rb):
        if qa["rows"] >= 1000:
            assert qa["err"] <= REL_L2 and qb["err"] <= REL_L2, (qa, qb)
            assert qa["err"] <= qb["err"] * 1.5 + 1e-7, (qa, qb)
