"""Input adaptor: the reference's 64-byte DepthSurfel records converted on the device."""
import ctypes

import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu

# row, col, then three float4 fields on 16-byte boundaries (8 bytes of padding)
SURFEL = np.dtype({"names": ["row", "col", "vc", "nr", "ct"],
                   "formats": ["<u4", "<u4", ("<f4", (4,)), ("<f4", (4,)), ("<f4", (4,))],
                   "offsets": [0, 4, 16, 32, 48], "itemsize": 64})


def test_surfels_to_points_and_reconstruction():
    import torch
    import psr
    assert SURFEL.itemsize == 64
    p, nr, _, D = syn.workload("sphere20k", n=12000)
    rng = np.random.default_rng(5)
    s = np.zeros(len(p), SURFEL)
    s["vc"][:, :3] = p
    s["vc"][:, 3] = rng.random(len(p))          # confidence: ignored
    s["nr"][:, :3] = nr
    s["nr"][:, 3] = rng.random(len(p))          # radius: ignored
    s["ct"][:, :3] = rng.random((len(p), 3))    # colour in [0, 1]
    s["ct"][:, 3] = 7.0                         # time: ignored
    dev = torch.device("cuda", 0)
    d_s = torch.from_numpy(s.view(np.uint8)).to(dev)
    xyz = torch.empty((len(p), 3), dtype=torch.float32, device=dev)
    nrm = torch.empty_like(xyz)
    rgb = torch.empty((len(p), 3), dtype=torch.uint8, device=dev)
    lib = psr.load_library()
    st = lib.psr_surfels_to_points(d_s.data_ptr(), len(p), xyz.data_ptr(), nrm.data_ptr(), rgb.data_ptr(), None)
    assert st == psr.PSR_OK
    torch.cuda.synchronize()
    np.testing.assert_array_equal(xyz.cpu().numpy(), p)
    np.testing.assert_array_equal(nrm.cpu().numpy(), nr)
    want = np.clip(np.rint(s["ct"][:, :3] * np.float32(255)), 0, 255).astype(np.uint8)
    np.testing.assert_array_equal(rgb.cpu().numpy(), want)
    with psr.PoissonReconstruction(max_depth=6, max_points=20000, compute_colors=True) as r:
        a = r.SolvePoissionReconstructionMesh(p, nr, want, depth=D)
        vcap, tcap = r.config.max_mesh_vertices, r.config.max_triangles
        out = [torch.empty((vcap, 3), dtype=torch.float32, device=dev),
               torch.empty((tcap, 3), dtype=torch.int32, device=dev),
               torch.empty((vcap, 3), dtype=torch.float32, device=dev)]
        m = psr.PsrMesh(out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), None, vcap, tcap, psr.PSR_DEVICE,
                        0, 0)
        r.reconstruct_device(xyz.data_ptr(), nrm.data_ptr(), rgb.data_ptr(), len(p), depth=D, out=m)
        np.testing.assert_array_equal(out[0][:m.vertex_count].cpu().numpy(), a.vertices)
        np.testing.assert_array_equal(out[1][:m.triangle_count].cpu().numpy(), a.triangles)
        np.testing.assert_array_equal(out[2][:m.vertex_count].cpu().numpy(), a.colors)
    # invalid arguments are rejected before any launch
    assert lib.psr_surfels_to_points(None, 5, xyz.data_ptr(), nrm.data_ptr(), None, None) == psr.PSR_INVALID_INPUT
