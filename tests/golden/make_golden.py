#!/usr/bin/env python3
"""Generates the golden fixtures that pin the oracle to the reference.

1. B-spline inner-product tables: runs oracle/_ref/ref_tables, i.e. the reference's own
   host code (mesh/FunctionData.h setDotTables with PPolynomial<2>::GaussianApproximation,
   compiled in place from the reference tree by oracle/build_ref.sh), for max depths 3 and
   6, and stores every non-zero (i, j, <F,F>, <F',F>, <F',F'>) entry plus the base
   function's polynomial pieces -> ref_tables_d3.npz, ref_tables_d6.npz.
2. Look-up tables the reference hard-codes (neighbour LUTs base/Constants.h:5-24 and
   mesh/BuildOctree.cu:20-42, edge / face / parent-face / child-vertex tables
   mesh/ComputeTriangleIndices.cu:31-38,317-322, mesh/BuildMeshGeometry.cu:19-26), parsed
   from the source text -> ref_luts.json.

   It also holds the marching-cubes case table (mesh/ComputeTriangleIndices.cu:41-315).

Usage: python3 tests/golden/make_golden.py REFERENCE_ROOT (or with $PSR_REFERENCE_ROOT set)
"""
import json
import re
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent


def tables(depth):
    exe = ROOT / "oracle" / "_ref" / "ref_tables"
    if not exe.exists():
        subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh"), str(reference_root())], check=True)
    out = subprocess.run([str(exe), str(depth)], check=True, capture_output=True, text=True).stdout
    pieces, rows = [], []
    res = None
    for line in out.splitlines():
        f = line.split()
        if f[0] == "res":
            res = int(f[1])
        elif f[0] == "piece":
            pieces.append([float(x) for x in f[1:]])
        elif f[0] == "t":
            rows.append([float(x) for x in f[1:]])
    rows = np.array(rows)
    np.savez_compressed(HERE / f"ref_tables_d{depth}.npz", res=res, pieces=np.array(pieces),
                        i=rows[:, 0].astype(np.int32), j=rows[:, 1].astype(np.int32),
                        ff=rows[:, 2], dff=rows[:, 3], d2=rows[:, 4])


def _array(text, name, count):
    start = text.index(name)
    brace = text.index("{", start)
    depth = 0
    for k in range(brace, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                body = text[brace:k + 1]
                break
    nums = [int(x) for x in re.findall(r"-?\d+", body)]
    assert len(nums) == count, (name, len(nums))
    return nums


def luts(ref):
    def rd(p):
        return (ref / p).read_bytes().decode("gbk", errors="replace")
    oct_src = rd("mesh/BuildOctree.cu")
    tri_src = rd("mesh/ComputeTriangleIndices.cu")
    geo_src = rd("mesh/BuildMeshGeometry.cu")
    out = {
        "lut_parent": _array(oct_src, "LUTparent[8][27]", 216),
        "lut_child": _array(oct_src, "LUTchild[8][27]", 216),
        "edge_vertex": _array(tri_src, "edgeVertex[12][2]", 24),
        "face_edges": _array(tri_src, "faceEdges[6][4]", 24),
        "children_vertex_kind": _array(tri_src, "childrenVertexKind[8]", 8),
        "parent_face_kind": _array(geo_src, "parentFaceKind[8][6]", 48),
        # marching-cubes case table (mesh/ComputeTriangleIndices.cu:41-315): triangle count
        # and the 16-entry edge list (-1 terminated) of every cube class
        "mc_count": _array(tri_src, "trianglesCount[256]", 256),
        "mc_triangles": _array(tri_src, "triangles[256][16]", 256 * 16),
    }
    (HERE / "ref_luts.json").write_text(json.dumps(out))


def reference_root():
    """The reference tree: first argument, else $PSR_REFERENCE_ROOT."""
    import os
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PSR_REFERENCE_ROOT")
    if not arg:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT (or set PSR_REFERENCE_ROOT)")
    return Path(arg)


if __name__ == "__main__":
    ref = reference_root()
    tables(3)
    tables(6)
    luts(ref)
    print("golden fixtures written to", HERE)
