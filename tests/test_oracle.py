"""CPU tests of the oracle: pinned against the reference's own table code and its
hard-coded look-up tables (tests/golden), plus known-answer and invariant checks."""
import json
from pathlib import Path

import numpy as np
import pytest

import synthetic as syn

GOLDEN = Path(__file__).resolve().parent / "golden"


def _run(oracle_mod, xyz, nrm, depth, **kw):
    o = oracle_mod.Oracle()
    rc = o.run(xyz, nrm, depth=depth, **kw)
    return o, rc


@pytest.mark.parametrize("depth", [3, 6])
def test_tables_match_reference_host_code(oracle_mod, depth):
    """<F,F>, <F',F>, <F',F'> of the oracle vs the reference's FunctionData (float arithmetic,
    ~4e-6 relative error in the reference, exact integrals in the oracle)."""
    ref = np.load(GOLDEN / f"ref_tables_d{depth}.npz")
    rng = np.random.default_rng(0)
    p = rng.uniform(-1, 1, (64, 3)).astype(np.float32)
    o, rc = _run(oracle_mod, p, p, depth, stop_after=2)
    assert rc == 0
    res = int(ref["res"])
    ff = o.get("ff").reshape(res, res).T   # oracle stores i + res*j
    dff = o.get("dff").reshape(res, res).T
    d2 = o.get("d2").reshape(res, res).T
    i, j = ref["i"], ref["j"]
    # The reference evaluates these integrals with float polynomial arithmetic; its error is
    # bounded relative to the Cauchy-Schwarz scale of each entry (measured <= 3.7e-5).
    fd, dd = np.diag(ff), np.diag(d2)
    scales = {"ff": np.sqrt(fd[i] * fd[j]), "dff": np.sqrt(dd[i] * fd[j]), "d2": np.sqrt(dd[i] * dd[j])}
    for name, mine, theirs in (("ff", ff[i, j], ref["ff"]), ("dff", dff[i, j], ref["dff"]), ("d2", d2[i, j], ref["d2"])):
        err = (np.abs(mine - theirs) / scales[name]).max()
        assert err < 5e-5, (name, err)
    # same sparsity: every entry the reference leaves empty is zero in the oracle
    mask = np.zeros((res, res), bool)
    mask[i, j] = True
    assert np.abs(ff[~mask]).max(initial=0) < 1e-12
    # base function pieces: F = GaussianApproximation / F(0)
    pieces = ref["pieces"]
    assert pieces.shape == (4, 4)
    np.testing.assert_allclose(pieces[:, 0], [-1.5, -0.5, 0.5, 1.5])


def test_luts_match_reference_constants(oracle_mod):
    ref = json.loads((GOLDEN / "ref_luts.json").read_text())
    mine = oracle_mod.luts()
    for k, v in ref.items():
        if k.startswith("mc_"):
            continue   # the case table: test_mc_table_matches_reference_case_table
        assert mine[k] == v, k


def test_mc_table_matches_reference_case_table(oracle_mod):
    """The case table the kernels and the oracle decode (csrc/mc_tables.inc) equals the
    reference's trianglesCount[256] / triangles[256][16] (mesh/ComputeTriangleIndices.cu:
    41-315), parsed from the reference source: same triangle count, same edges, same order
    and so the same winding, for every cube class."""
    ref = json.loads((GOLDEN / "ref_luts.json").read_text())
    counts, edges = oracle_mod.mc_tables()
    tri = np.array(ref["mc_triangles"]).reshape(256, 16)
    assert counts == ref["mc_count"]
    for c in range(256):
        row = list(tri[c])
        want = row[:row.index(-1)] if -1 in row else row
        assert len(want) == 3 * ref["mc_count"][c], c
        assert edges[c] == want, c


def test_mc_table_uses_exactly_the_crossing_edges(oracle_mod):
    """For every cube class, the triangle list touches exactly the edges whose two corners
    differ in sign (corner numbering of edge_vertex vs the case table)."""
    counts, edges = oracle_mod.mc_tables()
    ev = np.array(json.loads((GOLDEN / "ref_luts.json").read_text())["edge_vertex"]).reshape(12, 2)
    for c in range(256):
        crossing = {e for e in range(12) if ((c >> ev[e, 0]) & 1) != ((c >> ev[e, 1]) & 1)}
        used = set(edges[c][:3 * counts[c]])
        assert used == crossing, c


def test_morton_codes_at_cell_boundaries(oracle_mod):
    # bbox [0,1]^3 -> edge 1.25, centre -0.125: x = 0.5 maps to exactly 0.5 in the unit cube,
    # which the reference assigns to the lower cell (strict '>' against the centre)
    pts = np.array([[0, 0, 0], [1, 1, 1], [0.5, 0.5, 0.5], [0.5000001, 0.5, 0.5]], np.float32)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (4, 1))
    o, rc = _run(oracle_mod, pts, nrm, 4, stop_after=1)
    assert rc == 0
    keys = o.get("sorted_keys")
    codes = (keys >> 32).astype(np.int64)
    idx = keys & 0xFFFFFFFF
    pos = o.get("pos").reshape(-1, 3)
    # the centre point (normalised 0.5) gets all-low bits at level 1 (0.5 > 0.5 is false)
    by_orig = {}
    for k, c in zip(idx, codes):
        by_orig[int(k)] = int(c)
    order = np.argsort(keys)
    assert np.all(np.diff(keys) > 0)
    assert (codes[np.argmin(np.abs(pos[:, 0] - 0.5) + np.abs(pos[:, 1] - 0.5))] >> 9) & 7 == 0


def _invariants(o, D):
    s = o.scalars()
    base = o.get("base")
    count = o.get("count")
    M = s["M"]
    pnum = o.get("pnum")
    parent = o.get("parent")
    children = o.get("children").reshape(M, 8)
    neighs = o.get("neighs").reshape(M, 27)
    dnum = o.get("dnum")
    didx = o.get("didx")
    depth = o.get("depth")
    assert base[0] == 0 and count[0] == 1
    assert np.all(count[1:] % 8 == 0)
    for d in range(D + 1):
        assert pnum[base[d]:base[d] + count[d]].sum() == s["N"]
        assert np.all(depth[base[d]:base[d] + count[d]] == d)
    # dnum of every node equals the D-level slots below it; didx is the first of them
    assert dnum[0] == count[D]
    # every node is its own centre neighbour unless the reference's parent quirk applies
    assert parent[0] == -1
    for i in range(1, M):
        fc = children[i, 0]
        if fc >= 0:
            assert np.all(children[i] == fc + np.arange(8))
            assert np.all(depth[fc:fc + 8] == depth[i] + 1)
    return base, count


@pytest.mark.parametrize("D", [4, 6])
def test_octree_invariants_sphere(oracle_mod, D):
    p, n, _, _ = syn.workload("sphere20k", n=3000)
    o, rc = _run(oracle_mod, p, n, D, stop_after=1)
    assert rc == 0
    _invariants(o, D)


def test_two_points_known_tree(oracle_mod):
    """Opposite corners of the bounding box: one occupied leaf per corner at every level."""
    pts = np.array([[0, 0, 0], [1, 1, 1]], np.float32)
    nrm = np.array([[-1, -1, -1], [1, 1, 1]], np.float32)
    D = 3
    o, rc = _run(oracle_mod, pts, nrm, D, stop_after=1)
    assert rc == 0
    count = o.get("count")
    assert count.tolist() == [1, 8, 16, 16]
    key = o.get("key")
    pnum = o.get("pnum")
    base = o.get("base")
    # level 1: octants 0 and 7 hold one point each
    assert pnum[1:9].tolist() == [1, 0, 0, 0, 0, 0, 0, 1]
    # level 2 groups: children of octant 0 then of octant 7, each child 0 / child 7 occupied
    lvl2 = pnum[base[2]:base[2] + 16]
    assert lvl2.tolist() == [1, 0, 0, 0, 0, 0, 0, 0] + [0, 0, 0, 0, 0, 0, 0, 1]
    # keys of the empty siblings follow the slot order
    sh = 3 * (D - 1)
    assert [(k >> sh) & 7 for k in key[1:9]] == list(range(8))


def test_single_point_rejected(oracle_mod):
    # zero bounding box: the reference divides by a zero edge; the build rejects it
    p = np.array([[0.5, 0.5, 0.5]], np.float32)
    o = oracle_mod.Oracle()
    rc = o.run(p, p, depth=3, stop_after=1)
    pos = o.get("pos")
    assert not np.all(np.isfinite(pos)) or rc != 0


def test_sphere_reconstruction_radius(oracle_mod):
    """Known answer: the mesh of a noisy unit sphere lies on the sphere."""
    p, n, _, D = syn.workload("sphere20k")
    o, rc = _run(oracle_mod, p, n, D, cg_iters=0)
    assert rc == 0
    s = o.scalars()
    v = o.get("mesh_v").reshape(-1, 3).astype(np.float64)
    t = o.get("mesh_t").reshape(-1, 3)
    assert len(v) > 1000 and len(t) > 2000
    w = s["bbox_center"][None, :] + v * s["bbox_edge"]
    r = np.linalg.norm(w, axis=1)
    cell = s["bbox_edge"] / (1 << D)
    main = o.get("mesh_stage_v")[0]
    rm = r[:main]
    assert abs(np.median(rm) - 1.0) < 0.5 * cell
    assert np.percentile(np.abs(rm - 1.0), 95) < 1.5 * cell


def test_cg_converges_to_tolerance(oracle_mod):
    p, n, _, D = syn.workload("sphere20k", n=5000)
    o, rc = _run(oracle_mod, p, n, D, stop_after=3)
    assert rc == 0
    it = o.get("cg_iters")
    res = o.get("cg_resid")
    assert np.all(it < 10000)
    assert np.all(res <= 1.0000001e-5)
