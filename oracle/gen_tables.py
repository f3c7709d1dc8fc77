#!/usr/bin/env python3
"""Generate the marching-cubes case table used by both the CUDA kernels and the oracle.

The triangle list of every cube case has to be identical to the reference's so that
triangle topology and the vertex order inside each triangle match bit for bit.  That
table is data, not something that can be derived, so this recipe reads it from the
reference source (mesh/ComputeTriangleIndices.cu:41-315, the `trianglesCount[256]` and
`triangles[256][16]` constants) and re-encodes it in this project's own compact form:

    kMcTriangles[case] : uint64, one 4-bit edge index per nibble (low nibble first),
                         terminated by the nibble 0xF.
    kMcTriangleCount[case] : the per-case triangle count, taken verbatim because the
                         reference indexes its triangle list by that count.

The output is committed (poisson-surface-reconstruction-gpu_gb300/csrc/mc_tables.inc);
re-running this script against the reference must reproduce it byte for byte.

Usage:  python3 oracle/gen_tables.py REFERENCE_ROOT [output_path]   (or $PSR_REFERENCE_ROOT)
"""
import re
import subprocess
import sys
from pathlib import Path


def _read_gbk(path: Path) -> str:
    raw = path.read_bytes()
    try:
        return raw.decode("gbk")
    except UnicodeDecodeError:
        return raw.decode("utf-8", errors="replace")


def _int_block(text: str, name: str, count: int):
    start = text.index(name)
    brace = text.index("{", start)
    # find matching closing brace of the outer initializer
    depth = 0
    for i in range(brace, len(text)):
        ch = text[i]
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth == 0:
                end = i
                break
    body = text[brace:end + 1]
    nums = [int(x) for x in re.findall(r"-?\d+", body)]
    if len(nums) != count:
        raise SystemExit(f"{name}: expected {count} integers, found {len(nums)}")
    return nums


def main():
    import os
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PSR_REFERENCE_ROOT")
    if not arg:
        raise SystemExit("usage: gen_tables.py REFERENCE_ROOT [out] (or set PSR_REFERENCE_ROOT)")
    ref = Path(arg)
    out = Path(sys.argv[2] if len(sys.argv) > 2 else
               Path(__file__).resolve().parent.parent /
               "poisson-surface-reconstruction-gpu_gb300" / "csrc" / "mc_tables.inc")
    text = _read_gbk(ref / "mesh" / "ComputeTriangleIndices.cu")
    counts = _int_block(text, "trianglesCount[256]", 256)
    tris = _int_block(text, "triangles[256][16]", 256 * 16)

    packed = []
    for c in range(256):
        row = tris[16 * c:16 * c + 16]
        edges = []
        for v in row:
            if v < 0:
                break
            if v > 11:
                raise SystemExit(f"case {c}: edge index {v} out of range")
            edges.append(v)
        if len(edges) % 3:
            raise SystemExit(f"case {c}: {len(edges)} edge entries is not a multiple of 3")
        if counts[c] * 3 > len(edges):
            raise SystemExit(f"case {c}: count {counts[c]} exceeds listed triangles")
        word = 0
        for k, e in enumerate(edges):
            word |= e << (4 * k)
        word |= 0xF << (4 * len(edges))
        packed.append(word)

    lines = [
        "// Generated by oracle/gen_tables.py from the reference's marching-cubes case table",
        "// (mesh/ComputeTriangleIndices.cu:41-315).  Do not edit by hand.",
        "// kMcTriangles: 4-bit edge indices, low nibble first, 0xF terminates the list.",
        "// kMcTriangleCount: triangles emitted per cube case.",
        "#pragma once",
        "static const unsigned long long kMcTrianglesInit[256] = {",
    ]
    for i in range(0, 256, 4):
        lines.append("    " + ", ".join(f"0x{w:016X}ULL" for w in packed[i:i + 4]) + ",")
    lines.append("};")
    lines.append("static const int kMcTriangleCountInit[256] = {")
    for i in range(0, 256, 16):
        lines.append("    " + ", ".join(str(v) for v in counts[i:i + 16]) + ",")
    lines.append("};")
    out.write_text("\n".join(lines) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
