"""The allocation-free point-ordering entry point (psr_morton_sort_noalloc).

It exists for callers that cannot call cudaMalloc (a caller-owned memory pool or arena,
a host process whose allocator must see every byte, real-time loops); its scratch is a
fixed device array inside the library.  Checked through the C ABI against the ordering
that psr_reconstruct produces for the same cloud, on two calls in a row, so the second
call also shows that the shared scratch left by the first is cleared correctly.  This
file is collected last so that a failure here cannot hide any other test.
"""
import ctypes

import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu


def _reference_order(xyz, nrm, depth):
    """Sorted normalised positions and per-point codes from psr_reconstruct.  Only its
    octree is compared, so a few CG iterations do; a sparse cloud at depth 9 can then
    overflow a mesh capacity, which leaves the octree arrays (built before the mesh)
    intact."""
    import psr
    with psr.PoissonReconstruction(max_depth=depth, max_points=max(len(xyz), 300000),
                                   laplacian_epsilon=0.0) as r:
        try:
            r.SolvePoissionReconstructionMesh(xyz, nrm, depth=depth, cg_iterations=4)
        except psr.PsrError as e:
            if e.status != psr.PSR_OUT_OF_CAPACITY:
                raise
        st = r.stats()
        bbox = r.debug("bbox", np.float32)
        px, py, pz = (r.debug(n, np.float32) for n in ("px", "py", "pz"))
        key = r.debug("key")
        p2n = r.debug("point2node")
        bD = sum(st.level_count[d] for d in range(depth))
        codes = key[bD + p2n].astype(np.uint32)
    return np.stack([px, py, pz], 1), codes, bbox[:3], float(bbox[3])


def _noalloc(xyz, depth):
    import torch
    import psr
    lib = psr.load_library()
    dev = torch.device("cuda", 0)
    d_xyz = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).to(dev)
    d_codes = torch.empty(len(xyz), dtype=torch.int32, device=dev)
    d_order = torch.empty(len(xyz), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = lib.psr_morton_sort_noalloc(d_xyz.data_ptr(), len(xyz), depth, ctypes.c_float(1.25), d_codes.data_ptr(),
                                     d_order.data_ptr(), stream)
    assert st == psr.PSR_OK, lib.psr_status_string(st)
    return d_codes.cpu().numpy().view(np.uint32), d_order.cpu().numpy()


def _far_cloud(n):
    """A sphere of radius 1e5 centred near (1e7, -2e7, 3e7): every coordinate of every
    axis lies beyond 1e6 in magnitude (a georeferenced scan)."""
    xyz, nrm, _, _ = syn.workload("sphere20k", n=n)
    far = xyz.astype(np.float64) * 1e5 + np.array([1e7, -2e7, 3e7])
    return far.astype(np.float32), nrm


# depths 7 and 6 take three radix passes (the result lands in the scratch and is copied
# back), depths 5 and 9 an even number (sorted in place)
@pytest.mark.parametrize("calls", [[("torus_ellipsoid200k", None, 7), ("sphere20k", 5000, 6)],
                                   [("sphere20k", 20000, 5), ("sphere20k", 20000, 9)],
                                   [("far", 20000, 6), ("far", 20000, 6)]])
def test_noalloc_sort_matches_pipeline_twice(calls):
    for name, n, depth in calls:
        if name == "far":
            xyz, nrm = _far_cloud(n)
        else:
            xyz, nrm, _, _ = syn.workload(name, n=n)
        sorted_pos, codes_ref, center, scale = _reference_order(xyz, nrm, depth)
        codes, order = _noalloc(xyz, depth)
        np.testing.assert_array_equal(codes, codes_ref)
        assert np.array_equal(np.sort(order), np.arange(len(xyz)))
        # stable: equal codes keep the input order
        same = codes[1:] == codes[:-1]
        assert np.all(order[1:][same] > order[:-1][same])
        # the order reproduces the pipeline's sorted, normalised points bit for bit
        p = (xyz[order] - center[None, :].astype(np.float32)) * np.float32(1.0) / np.float32(scale)
        np.testing.assert_array_equal(p.astype(np.float32), sorted_pos)


def test_noalloc_rejects_oversized_and_bad_input():
    import torch
    import psr
    lib = psr.load_library()
    dev = torch.device("cuda", 0)
    buf = torch.empty(16, dtype=torch.float32, device=dev)
    assert lib.psr_morton_sort_noalloc(buf.data_ptr(), (1 << 20) + 1, 7, ctypes.c_float(1.25), buf.data_ptr(),
                                       buf.data_ptr(), None) == psr.PSR_OUT_OF_CAPACITY
    assert lib.psr_morton_sort_noalloc(None, 10, 7, ctypes.c_float(1.25), buf.data_ptr(), buf.data_ptr(),
                                       None) == psr.PSR_INVALID_INPUT
