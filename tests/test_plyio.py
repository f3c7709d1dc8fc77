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


def _write_pcd(path, fields, sizes, types, counts, cols, kind):
    """A PCD v0.7 file; cols maps each field to an (N,) or (N, count) array."""
    n = len(next(iter(cols.values())))
    head = ["# .PCD v0.7 - Point Cloud Data file format", "VERSION 0.7", "FIELDS " + " ".join(fields),
            "SIZE " + " ".join(map(str, sizes)), "TYPE " + " ".join(types),
            "COUNT " + " ".join(map(str, counts)), f"WIDTH {n}", "HEIGHT 1", "VIEWPOINT 0 0 0 1 0 0 0",
            f"POINTS {n}", f"DATA {kind}"]
    code = {("F", 4): "f4", ("U", 1): "u1", ("U", 4): "u4"}
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if kind == "ascii":
            for i in range(n):
                row = []
                for name in fields:
                    v = np.atleast_1d(cols[name][i])
                    row += [repr(float(x)) if np.issubdtype(v.dtype, np.floating) else str(int(x)) for x in v]
                f.write((" ".join(row) + "\n").encode())
        else:
            dt = np.dtype([(f"{nm}{k}", "<" + code[(t, s)], (c,) if c > 1 else ())
                           for k, (nm, t, s, c) in enumerate(zip(fields, types, sizes, counts))])
            rec = np.zeros(n, dtype=dt)
            for k, nm in enumerate(fields):
                rec[f"{nm}{k}"] = cols[nm]
            f.write(rec.tobytes())


def test_pcd_points_layouts(tmp_path):
    """The field layouts of unoriented PCD clouds: x y z with a 4-byte pad, intensity
    first, packed colour; ascii and binary; and one with normals."""
    p, nr, rgb, _ = syn.workload("sphere20k", n=300, colour=True)
    n = len(p)
    pad = np.zeros((n, 4), np.uint8)
    packed = (rgb[:, 0].astype(np.uint32) << 16) | (rgb[:, 1].astype(np.uint32) << 8) | rgb[:, 2]
    xyz = {"x": p[:, 0], "y": p[:, 1], "z": p[:, 2]}
    cases = [
        (["x", "y", "z", "_"], [4, 4, 4, 1], ["F", "F", "F", "U"], [1, 1, 1, 4], dict(xyz, _=pad), None, None),
        (["intensity", "x", "y", "z", "_"], [4, 4, 4, 4, 1], ["F", "F", "F", "F", "U"], [1, 1, 1, 1, 4],
         dict(xyz, intensity=np.ones(n, np.float32), _=pad), None, None),
        (["x", "y", "z", "confidence", "rgb"], [4, 4, 4, 4, 4], ["F", "F", "F", "F", "U"], [1] * 5,
         dict(xyz, confidence=np.ones(n, np.float32), rgb=packed), None, rgb),
        (["x", "y", "z", "normal_x", "normal_y", "normal_z"], [4] * 6, ["F"] * 6, [1] * 6,
         dict(xyz, normal_x=nr[:, 0], normal_y=nr[:, 1], normal_z=nr[:, 2]), nr, None),
    ]
    for k, (fields, sizes, types, counts, cols, want_n, want_c) in enumerate(cases):
        for kind in ("ascii", "binary"):
            if kind == "ascii" and "_" in fields:
                continue   # padding fields appear in binary files only
            path = tmp_path / f"c{k}_{kind}.pcd"
            _write_pcd(path, fields, sizes, types, counts, cols, kind)
            x, nn, c = plyio.read_points(path)
            np.testing.assert_array_equal(x, p)
            if want_n is None:
                assert nn is None
            else:
                np.testing.assert_array_equal(nn, want_n)
            if want_c is None:
                assert c is None
            else:
                np.testing.assert_array_equal(c, want_c)


def test_pcd_rejects_compressed_and_short(tmp_path):
    import pytest
    path = tmp_path / "c.pcd"
    path.write_bytes(b"VERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\nCOUNT 1 1 1\nWIDTH 2\nHEIGHT 1\n"
                     b"POINTS 2\nDATA binary_compressed\n\x00\x00")
    with pytest.raises(ValueError, match="binary_compressed"):
        plyio.read_points(path)
    path.write_bytes(b"VERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\nCOUNT 1 1 1\nWIDTH 2\nHEIGHT 1\n"
                     b"POINTS 2\nDATA binary\n\x00\x00\x00\x00")
    with pytest.raises(ValueError, match="shorter"):
        plyio.read_points(path)


def test_txt_positions_only(tmp_path):
    """Three columns (the reference's .txt fixtures): positions, no normals."""
    p, _, _, _ = syn.workload("sphere20k", n=100)
    path = tmp_path / "xyz.txt"
    np.savetxt(path, p, fmt="%.9g", delimiter="\t")
    x, n, c = plyio.read_points(path)
    np.testing.assert_array_equal(x, p)
    assert n is None and c is None


def test_organised_pcd_with_invalid_pixels(tmp_path):
    """An organised cloud (HEIGHT > 1) with NaN pixels: dropped by default, kept on request."""
    p, _, _, _ = syn.workload("sphere20k", n=64)
    q = p.copy()
    q[[3, 10, 40]] = np.nan
    path = tmp_path / "org.pcd"
    head = ("VERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\nCOUNT 1 1 1\nWIDTH 8\nHEIGHT 8\n"
            "VIEWPOINT 0 0 0 1 0 0 0\nPOINTS 64\nDATA binary\n")
    path.write_bytes(head.encode() + q.astype("<f4").tobytes())
    x, n, c = plyio.read_points(path)
    keep = np.ones(64, bool)
    keep[[3, 10, 40]] = False
    np.testing.assert_array_equal(x, p[keep])
    x2, _, _ = plyio.read_points(path, finite_only=False)
    assert x2.shape == (64, 3) and np.isnan(x2[3]).all()
