"""ctypes binding of the CPU oracle (oracle/psr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU-baseline leg
of bench.py, as the checker.  The product library never loads it.
"""
import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "libpsr_oracle.so"
SRC = HERE / "psr_oracle.cpp"

_ELEM = {0: np.int32, 1: np.float32, 2: np.float64, 3: np.int64}


def build(force=False):
    """Compile the oracle (host C++, OpenMP)."""
    if LIB.exists() and not force and LIB.stat().st_mtime > SRC.stat().st_mtime:
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC",
           "-o", str(LIB), str(SRC)]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        L.oro_create.restype = ctypes.c_void_p
        L.oro_destroy.argtypes = [ctypes.c_void_p]
        L.oro_set_lap_eps.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.oro_set_tables.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5
        L.oro_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oro_run.restype = ctypes.c_int
        L.oro_run_mesh32.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float]
        L.oro_run_mesh32.restype = ctypes.c_int
        L.oro_point_values.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oro_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                              ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)]
        L.oro_get.restype = ctypes.c_int
        L.oro_luts.argtypes = [ctypes.c_void_p]
        L.oro_luts.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def luts():
    out = np.zeros(1024, np.int32)
    n = lib().oro_luts(out.ctypes.data_as(ctypes.c_void_p))
    out = out[:n]
    o = 0
    res = {}
    for name, cnt in (("lut_parent", 216), ("lut_child", 216), ("edge_vertex", 24), ("face_edges", 24),
                      ("children_vertex_kind", 8), ("parent_face_kind", 48)):
        res[name] = out[o:o + cnt].tolist()
        o += cnt
    return res


def mc_tables():
    """The marching-cubes case table as (count[256], edges[256] lists)."""
    src = (HERE.parent / "poisson-surface-reconstruction-gpu_gb300" / "csrc" / "mc_tables.inc").read_text()
    import re
    body = src[src.index("kMcTrianglesInit"):src.index("kMcTriangleCountInit")]
    words = [int(w, 16) for w in re.findall(r"0x([0-9A-F]+)ULL", body)]
    cbody = src[src.index("kMcTriangleCountInit"):]
    counts = [int(x) for x in re.findall(r"-?\d+", cbody[cbody.index("{"):])][:256]
    edges = []
    for w in words:
        lst = []
        while (w & 0xF) != 0xF:
            lst.append(w & 0xF)
            w >>= 4
        edges.append(lst)
    return counts, edges


class Oracle:
    """One oracle run; arrays are copied out on access."""

    def __init__(self, laplacian_epsilon=None):
        self._h = lib().oro_create()
        if laplacian_epsilon is not None:   # default: the reference's 1e-6 drop threshold
            lib().oro_set_lap_eps(self._h, float(laplacian_epsilon))

    def set_tables(self, res, i, j, ff, dff, d2):
        """Solve the following runs (of the depth with this res) on the given table entries
        instead of the exact integrals; res = 0 goes back to the exact tables."""
        arrs = [np.ascontiguousarray(i, np.int32), np.ascontiguousarray(j, np.int32),
                np.ascontiguousarray(ff, np.float64), np.ascontiguousarray(dff, np.float64),
                np.ascontiguousarray(d2, np.float64)]
        self._keept = arrs
        lib().oro_set_tables(self._h, int(res), int(arrs[0].shape[0]), *[_ptr(a) for a in arrs])

    def __del__(self):
        try:
            if self._h:
                lib().oro_destroy(self._h)
        except Exception:
            pass

    def run(self, xyz, nrm, rgb=None, depth=7, cg_iters=0, cg_tol=1e-5, cg_max_iter=10000,
            stop_after=99, vert_cap=0, tri_cap=0):
        xyz = np.ascontiguousarray(xyz, np.float32)
        nrm = np.ascontiguousarray(nrm, np.float32)
        if rgb is not None:
            rgb = np.ascontiguousarray(rgb, np.float32)
            if rgb.dtype != np.float32:
                rgb = rgb.astype(np.float32)
        self._keep = (xyz, nrm, rgb)
        return lib().oro_run(self._h, _ptr(xyz), _ptr(nrm), _ptr(rgb), int(xyz.shape[0]), int(depth),
                             int(cg_iters), float(cg_tol), int(cg_max_iter), int(stop_after),
                             int(vert_cap), int(tri_cap))

    def run_mesh32(self, x, iso):
        x = np.ascontiguousarray(x, np.float32)
        self._keepx = x
        return lib().oro_run_mesh32(self._h, _ptr(x), ctypes.c_float(float(iso)))

    def point_values(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(int(self.scalars()["N"]), np.float64)
        lib().oro_point_values(self._h, _ptr(x), _ptr(out))
        return out

    def get(self, name):
        p = ctypes.c_void_p()
        n = ctypes.c_longlong()
        e = ctypes.c_int()
        rc = lib().oro_get(self._h, name.encode(), ctypes.byref(p), ctypes.byref(n), ctypes.byref(e))
        if rc != 0:
            raise KeyError(name)
        dt = _ELEM[e.value]
        if n.value == 0:
            return np.zeros(0, dt)
        buf = (ctypes.c_char * (n.value * np.dtype(dt).itemsize)).from_address(p.value)
        return np.frombuffer(buf, dtype=dt).copy()

    def scalars(self):
        s = self.get("scalars")
        return dict(iso=s[0], bbox_center=s[1:4], bbox_edge=s[4], ub_events=int(s[5]), M=int(s[6]),
                    N=int(s[7]), status=int(s[8]))
