"""Point-cloud input and mesh output files (host side, numpy).

The reference reads its inputs through PCL (mesh/PoissonReconstruction.cpp:63-188:
`.pcd`, `.ply`, `.txt`) and only draws its mesh.  These readers cover the oriented
point formats of its `PointCloudData/` fixtures without PCL:

* PLY (ascii, binary_little_endian, binary_big_endian) with vertex properties x, y, z,
  nx, ny, nz and optionally red, green, blue (any numeric types);
* whitespace-separated text, one point per line: x y z [nx ny nz [r g b]];
* PCD v0.7 (`DATA ascii` or `binary`) with fields x, y, z, optionally normal_x,
  normal_y, normal_z and a packed rgb, other fields (intensity, padding `_`) skipped.

Files without normals (the reference's `.txt` and `.pcd` fixtures) return normals None;
the caller estimates them on the GPU (`PoissonReconstruction.CalculatePointCloudNormal`,
the reference's PCL step of readPCDFile, mesh/PoissonReconstruction.cpp:80-101).

`write_mesh_ply` writes a reconstructed mesh (binary little endian; optional per-vertex
normals and colours), in world coordinates when given the call's center / scale.
"""
import numpy as np

_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def _read_header(f):
    if f.readline().strip() != b"ply":
        raise ValueError("not a PLY file")
    fmt, elements = None, []
    while True:
        line = f.readline()
        if not line:
            raise ValueError("PLY header without end_header")
        w = line.decode("ascii", "replace").split()
        if not w or w[0] in ("comment", "obj_info"):
            continue
        if w[0] == "format":
            fmt = w[1]
        elif w[0] == "element":
            elements.append([w[1], int(w[2]), []])
        elif w[0] == "property":
            if w[1] == "list":
                elements[-1][2].append((w[4], ("list", w[2], w[3])))
            else:
                elements[-1][2].append((w[2], w[1]))
        elif w[0] == "end_header":
            return fmt, elements


def read_ply_points(path):
    """Returns (xyz float32 N x 3, normals float32 N x 3, rgb uint8 N x 3 or None)."""
    with open(path, "rb") as f:
        fmt, elements = _read_header(f)
        if fmt not in ("ascii", "binary_little_endian", "binary_big_endian"):
            raise ValueError(f"PLY format {fmt!r} not supported")
        end = "<" if fmt == "binary_little_endian" else ">"
        vertex = None
        for name, count, props in elements:
            if any(isinstance(t, tuple) for _, t in props):
                if name == "vertex":
                    raise ValueError("list properties in the vertex element are not supported")
                if vertex is None:
                    raise ValueError("elements with lists before the vertex element are not supported")
                break
            if fmt == "ascii":
                data = np.loadtxt(f, max_rows=count, ndmin=2) if count else np.zeros((0, len(props)))
                cols = {p: data[:, i] for i, (p, _) in enumerate(props)}
            else:
                dt = np.dtype([(p, end + _PLY_TYPES[t]) for p, t in props])
                arr = np.frombuffer(f.read(dt.itemsize * count), dtype=dt, count=count)
                cols = {p: arr[p] for p, _ in props}
            if name == "vertex":
                vertex = cols
                break
        if vertex is None:
            raise ValueError("PLY file without a vertex element")
    for k in ("x", "y", "z", "nx", "ny", "nz"):
        if k not in vertex:
            raise ValueError(f"PLY vertex element lacks '{k}' (oriented points are required)")
    xyz = np.stack([vertex["x"], vertex["y"], vertex["z"]], 1).astype(np.float32)
    nrm = np.stack([vertex["nx"], vertex["ny"], vertex["nz"]], 1).astype(np.float32)
    rgb = None
    if all(k in vertex for k in ("red", "green", "blue")):
        rgb = np.clip(np.stack([vertex["red"], vertex["green"], vertex["blue"]], 1), 0, 255).astype(np.uint8)
    return xyz, nrm, rgb


def read_txt_points(path):
    """x y z [nx ny nz [r g b]] per line (r g b in 0..255); normals None for 3 columns
    (the reference's readTXTFile, mesh/PoissonReconstruction.cpp:63-78, reads positions)."""
    data = np.loadtxt(path, ndmin=2)
    if data.shape[1] < 3 or 3 < data.shape[1] < 6:
        raise ValueError("text points need 3 columns (x y z) or at least 6 (x y z nx ny nz)")
    nrm = data[:, 3:6].astype(np.float32) if data.shape[1] >= 6 else None
    rgb = np.clip(data[:, 6:9], 0, 255).astype(np.uint8) if data.shape[1] >= 9 else None
    return data[:, :3].astype(np.float32), nrm, rgb


_PCD_TYPES = {("F", 4): "f4", ("F", 8): "f8", ("U", 1): "u1", ("U", 2): "u2", ("U", 4): "u4", ("U", 8): "u8",
              ("I", 1): "i1", ("I", 2): "i2", ("I", 4): "i4", ("I", 8): "i8"}


def read_pcd_points(path):
    """PCD v0.7 (the reference's readPCDFile input, pcl::io::loadPCDFile): returns (xyz
    float32 N x 3, normals float32 N x 3 or None, rgb uint8 N x 3 or None)."""
    with open(path, "rb") as f:
        hdr = {}
        while True:
            line = f.readline()
            if not line:
                raise ValueError("PCD header without DATA")
            w = line.decode("ascii", "replace").split()
            if not w or w[0].startswith("#"):
                continue
            hdr[w[0].upper()] = w[1:]
            if w[0].upper() == "DATA":
                break
        fields = hdr.get("FIELDS")
        if not fields:
            raise ValueError("PCD header without FIELDS")
        nf = len(fields)
        sizes = [int(x) for x in hdr.get("SIZE", ["4"] * nf)]
        types = hdr.get("TYPE", ["F"] * nf)
        counts = [int(x) for x in hdr.get("COUNT", ["1"] * nf)]
        if not (len(sizes) == len(types) == len(counts) == nf):
            raise ValueError("PCD FIELDS / SIZE / TYPE / COUNT lengths differ")
        n = int(hdr["POINTS"][0]) if "POINTS" in hdr else int(hdr["WIDTH"][0]) * int(hdr.get("HEIGHT", ["1"])[0])
        data_kind = hdr["DATA"][0].lower()
        cols = {}
        if data_kind == "ascii":
            arr = np.loadtxt(f, max_rows=n, ndmin=2) if n else np.zeros((0, sum(counts)))
            if arr.shape[0] != n:
                raise ValueError(f"PCD declares {n} points, holds {arr.shape[0]}")
            at = 0
            for name, t, sz, c in zip(fields, types, sizes, counts):
                col = arr[:, at]
                if (t.upper(), sz) in (("U", 4), ("F", 4)) and name == "rgb":
                    col = col.astype(np.float32 if t.upper() == "F" else np.uint32)
                cols[name] = col
                at += c
        elif data_kind == "binary":
            dt = []
            for k, (name, t, sz, c) in enumerate(zip(fields, types, sizes, counts)):
                key = (t.upper(), sz)
                if key not in _PCD_TYPES:
                    raise ValueError(f"PCD field {name!r}: type {t} size {sz} not supported")
                dt.append((f"{name}#{k}", "<" + _PCD_TYPES[key], (c,) if c > 1 else ()))
            dt = np.dtype(dt)
            buf = f.read(dt.itemsize * n)
            if len(buf) != dt.itemsize * n:
                raise ValueError("PCD binary data shorter than declared")
            arr = np.frombuffer(buf, dtype=dt, count=n)
            for k, name in enumerate(fields):
                cols.setdefault(name, arr[f"{name}#{k}"])
        else:
            raise ValueError(f"PCD DATA {data_kind!r} not supported (ascii or binary)")
    for k in ("x", "y", "z"):
        if k not in cols:
            raise ValueError(f"PCD file lacks field '{k}'")
    xyz = np.stack([cols["x"], cols["y"], cols["z"]], 1).astype(np.float32)
    nrm = None
    if all(k in cols for k in ("normal_x", "normal_y", "normal_z")):
        nrm = np.stack([cols["normal_x"], cols["normal_y"], cols["normal_z"]], 1).astype(np.float32)
    rgb = None
    if "rgb" in cols or "rgba" in cols:
        packed = np.asarray(cols.get("rgb", cols.get("rgba")))
        packed = packed.view(np.uint32) if packed.dtype == np.float32 else packed.astype(np.uint32)
        rgb = np.stack([(packed >> 16) & 255, (packed >> 8) & 255, packed & 255], 1).astype(np.uint8)
    return xyz, nrm, rgb


def read_points(path, finite_only=True):
    """(xyz, normals or None, rgb or None) of a .ply, .pcd or text point file.  With
    finite_only, points whose position (or normal, when present) is not finite are
    dropped, order kept: organised PCD clouds mark invalid pixels with NaN, and the
    reconstruction rejects non-finite input."""
    p = str(path).lower()
    if p.endswith(".ply"):
        xyz, nrm, rgb = read_ply_points(path)
    elif p.endswith(".pcd"):
        xyz, nrm, rgb = read_pcd_points(path)
    elif p.endswith((".txt", ".xyz", ".xyzn")):
        xyz, nrm, rgb = read_txt_points(path)
    else:
        raise ValueError(f"unsupported point file {path}")
    if finite_only:
        keep = np.isfinite(xyz).all(axis=1)
        if nrm is not None:
            keep &= np.isfinite(nrm).all(axis=1)
        if not keep.all():
            xyz = xyz[keep]
            nrm = None if nrm is None else nrm[keep]
            rgb = None if rgb is None else rgb[keep]
    return xyz, nrm, rgb


def write_mesh_ply(path, vertices, triangles, colors=None, normals=None, center=None, scale=None):
    """Binary little-endian PLY.  vertices in the unit cube of the reconstruction are mapped
    to world coordinates (center + v * scale) when center and scale are given; colours are
    floats in [0, 1] (written as uchar)."""
    v = np.asarray(vertices, np.float32).reshape(-1, 3)
    if center is not None and scale is not None:
        v = (np.asarray(center, np.float32) + v * np.float32(scale)).astype(np.float32)
    t = np.asarray(triangles, np.int32).reshape(-1, 3)
    fields = [("x", "<f4"), ("y", "<f4"), ("z", "<f4")]
    if normals is not None:
        fields += [("nx", "<f4"), ("ny", "<f4"), ("nz", "<f4")]
    if colors is not None:
        fields += [("red", "u1"), ("green", "u1"), ("blue", "u1")]
    rec = np.zeros(v.shape[0], dtype=np.dtype(fields))
    rec["x"], rec["y"], rec["z"] = v[:, 0], v[:, 1], v[:, 2]
    if normals is not None:
        n = np.asarray(normals, np.float32).reshape(-1, 3)
        rec["nx"], rec["ny"], rec["nz"] = n[:, 0], n[:, 1], n[:, 2]
    if colors is not None:
        c = np.clip(np.rint(np.asarray(colors, np.float32).reshape(-1, 3) * 255.0), 0, 255).astype(np.uint8)
        rec["red"], rec["green"], rec["blue"] = c[:, 0], c[:, 1], c[:, 2]
    faces = np.zeros(t.shape[0], dtype=np.dtype([("n", "u1"), ("i", "<i4", (3,))]))
    faces["n"] = 3
    faces["i"] = t
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {v.shape[0]}"]
    head += [f"property float {k}" for k in ("x", "y", "z")]
    if normals is not None:
        head += [f"property float {k}" for k in ("nx", "ny", "nz")]
    if colors is not None:
        head += [f"property uchar {k}" for k in ("red", "green", "blue")]
    head += [f"element face {t.shape[0]}", "property list uchar int vertex_indices", "end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode("ascii"))
        f.write(rec.tobytes())
        f.write(faces.tobytes())


def read_mesh_ply(path):
    """Reads back a triangle mesh written by write_mesh_ply (binary little endian)."""
    with open(path, "rb") as f:
        fmt, elements = _read_header(f)
        if fmt != "binary_little_endian":
            raise ValueError("only binary_little_endian meshes are read back")
        (vn, vc, vp), (fn, fc, fp) = elements[0], elements[1]
        dt = np.dtype([(p, "<" + _PLY_TYPES[t]) for p, t in vp])
        v = np.frombuffer(f.read(dt.itemsize * vc), dtype=dt, count=vc)
        faces = np.frombuffer(f.read(13 * fc), dtype=np.dtype([("n", "u1"), ("i", "<i4", (3,))]), count=fc)
    xyz = np.stack([v["x"], v["y"], v["z"]], 1)
    return xyz, faces["i"].copy(), v
