"""Point-cloud readers and the mesh writer (host only)."""
import numpy as np

import plyio
import synthetic as syn


def _write_points_ply(path, xyz, nrm, rgb, fmt):
    head = ["ply", f"format {fmt} 1.0", "comment test", f"element vertex {len(xyz)}"]
    head += ["property float x", "property float y", "property float z",
             "property float nx", "property float ny", "property float nz"]
    if rgb is not None:
        head += ["property uchar red", "property uchar green", "property uchar blue"]
    head += ["element face 0", "property list uchar int vertex_indices", "end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if fmt == "ascii":
            for i in range(len(xyz)):
                row = list(map(repr, map(float, xyz[i]))) + list(map(repr, map(float, nrm[i])))
                if rgb is not None:
                    row += list(map(str, rgb[i]))
                f.write((" ".join(row) + "\n").encode())
        else:
            end = "<" if fmt == "binary_little_endian" else ">"
            fields = [(k, end + "f4") for k in ("x", "y", "z", "nx", "ny", "nz")]
            if rgb is not None:
                fields += [(k, "u1") for k in ("red", "green", "blue")]
            rec = np.zeros(len(xyz), dtype=fields)
            for a, k in enumerate("xyz"):
                rec[k] = xyz[:, a]
            for a, k in enumerate(("nx", "ny", "nz")):
                rec[k] = nrm[:, a]
            if rgb is not None:
                for a, k in enumerate(("red", "green", "blue")):
                    rec[k] = rgb[:, a]
            f.write(rec.tobytes())


def test_ply_points_all_formats(tmp_path):
    p, nr, rgb, _ = syn.workload("sphere20k", n=500, colour=True)
    for fmt in ("ascii", "binary_little_endian", "binary_big_endian"):
        for colour in (rgb, None):
            path = tmp_path / f"pts_{fmt}_{colour is None}.ply"
            _write_points_ply(path, p, nr, colour, fmt)
            x, n, c = plyio.read_points(path)
            np.testing.assert_array_equal(x, p)
            np.testing.assert_array_equal(n, nr)
            if colour is None:
                assert c is None
            else:
                np.testing.assert_array_equal(c, colour)


def test_txt_points(tmp_path):
    p, nr, rgb, _ = syn.workload("sphere20k", n=200, colour=True)
    path = tmp_path / "pts.txt"
    np.savetxt(path, np.concatenate([p, nr, rgb], 1), fmt="%.9g")
    x, n, c = plyio.read_points(path)
    np.testing.assert_array_equal(x, p)
    np.testing.assert_array_equal(n, nr)
    np.testing.assert_array_equal(c, rgb)


def test_mesh_round_trip_world_coordinates(tmp_path):
    rng = np.random.default_rng(3)
    v = rng.random((50, 3), dtype=np.float32)
    t = rng.integers(0, 50, (80, 3), dtype=np.int32)
    col = rng.random((50, 3), dtype=np.float32)
    nrm = rng.standard_normal((50, 3)).astype(np.float32)
    path = tmp_path / "mesh.ply"
    center, scale = (1.0, -2.0, 0.5), 3.0
    plyio.write_mesh_ply(path, v, t, colors=col, normals=nrm, center=center, scale=scale)
    xyz, tri, rec = plyio.read_mesh_ply(path)
    np.testing.assert_array_equal(tri, t)
    np.testing.assert_allclose(xyz, np.float32(center) + v * np.float32(scale), rtol=0, atol=1e-6)
    np.testing.assert_array_equal(rec["red"], np.clip(np.rint(col[:, 0] * 255), 0, 255).astype(np.uint8))
