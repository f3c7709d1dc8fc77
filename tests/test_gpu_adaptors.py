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


def test_unoriented_pcd_and_txt_files_reconstruct(tmp_path):
    """The reference's unoriented inputs (readPCDFile, readTXTFile): positions only, normals
    estimated on the GPU, then the reconstruction.  The normals point towards the viewpoint
    at the centre (inwards), which negates the indicator function and its iso value: the
    surface still lies on the sphere."""
    import psr
    p, _, _, D = syn.workload("sphere20k")
    pcd = tmp_path / "sphere.pcd"
    head = ("VERSION 0.7\nFIELDS x y z _\nSIZE 4 4 4 1\nTYPE F F F U\nCOUNT 1 1 1 4\n"
            f"WIDTH {len(p)}\nHEIGHT 1\nVIEWPOINT 0 0 0 1 0 0 0\nPOINTS {len(p)}\nDATA binary\n")
    rec = np.zeros(len(p), dtype=[("xyz", "<f4", (3,)), ("pad", "u1", (4,))])
    rec["xyz"] = p
    pcd.write_bytes(head.encode() + rec.tobytes())
    txt = tmp_path / "sphere.txt"
    np.savetxt(txt, p, fmt="%.9g", delimiter="\t")
    with psr.PoissonReconstruction(max_depth=D, max_points=30000) as r:
        for path, read in ((pcd, r.readPCDFile), (txt, r.readTXTFile)):
            xyz, nrm, rgb = read(str(path))
            assert rgb is None and np.all(np.isfinite(nrm))
            radial = (nrm.astype(np.float64) * p).sum(axis=1) / np.linalg.norm(p, axis=1)
            assert np.median(radial) < -0.99                       # inwards, towards the origin
            mesh = r.SolvePoissionReconstructionMesh(*r.getDenseSurfel(), depth=D)
            w = mesh.world_vertices().astype(np.float64)
            rad = np.linalg.norm(w, axis=1)
            cell = mesh.scale / (1 << D)
            assert len(w) > 1000
            assert abs(np.median(rad) - 1.0) < 0.5 * cell
