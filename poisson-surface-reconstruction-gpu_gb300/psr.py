"""Python mirror of the reference's PoissonReconstruction host API over the C ABI.

The reference class (mesh/PoissonReconstruction.h:63-184) owns the pipeline and exposes
``SolvePoissionReconstructionMesh`` (spelling kept) plus mesh getters
(mesh/ComputeTriangleIndices.h:331-342).  This module loads the in-tree libpsr.so built
for sm_103a (include/psr/psr.h) with ctypes.  There is no CPU fallback: if the library
is missing or no GPU is present the calls raise.
"""
import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libpsr.so"

(PSR_OK, PSR_OUT_OF_CAPACITY, PSR_INVALID_INPUT, PSR_NONCONVERGED, PSR_DEVICE_TIMEOUT, PSR_CUDA_ERROR,
 PSR_PENDING) = range(7)
PSR_HOST, PSR_DEVICE = 0, 1

# every function declared in include/psr/psr.h
EXPORTED = ["psr_config_default", "psr_create", "psr_destroy", "psr_reconstruct", "psr_submit", "psr_poll",
            "psr_wait", "psr_memory_bytes", "psr_get_stats", "psr_debug_array", "psr_status_string",
            "psr_last_error", "psr_surfels_to_points", "psr_morton_sort_noalloc", "psr_estimate_normals",
            "psr_submit_batch", "psr_reconstruct_batch", "psr_get_batch_result"]


class PsrConfig(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_int), ("max_points", ctypes.c_int), ("max_triangles", ctypes.c_int),
                ("max_mesh_vertices", ctypes.c_int), ("max_nodes", ctypes.c_int),
                ("max_subdivision_nodes", ctypes.c_int), ("bbox_scale", ctypes.c_float),
                ("cg_max_iterations", ctypes.c_int), ("cg_tolerance", ctypes.c_float),
                ("compute_colors", ctypes.c_int), ("compute_normals", ctypes.c_int), ("device", ctypes.c_int),
                ("laplacian_epsilon", ctypes.c_float), ("concurrent_stages", ctypes.c_int),
                ("weld_vertices", ctypes.c_int), ("disable_graphs", ctypes.c_int),
                ("root_poly_capacity", ctypes.c_int), ("cg_residual_period", ctypes.c_int),
                ("batch_clouds", ctypes.c_int), ("cg_cluster_ctas", ctypes.c_int),
                ("cg_cluster_ctas_fine", ctypes.c_int)]


class PsrPoints(ctypes.Structure):
    _fields_ = [("xyz", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("rgb", ctypes.c_void_p),
                ("count", ctypes.c_int), ("location", ctypes.c_int)]


class PsrOptions(ctypes.Structure):
    _fields_ = [("depth", ctypes.c_int), ("cg_iterations", ctypes.c_int)]


class PsrMesh(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_void_p), ("triangles", ctypes.c_void_p), ("colors", ctypes.c_void_p),
                ("normals", ctypes.c_void_p), ("vertex_capacity", ctypes.c_int),
                ("triangle_capacity", ctypes.c_int), ("location", ctypes.c_int), ("vertex_count", ctypes.c_int),
                ("triangle_count", ctypes.c_int), ("center", ctypes.c_float * 3), ("scale", ctypes.c_float)]


class PsrStats(ctypes.Structure):
    _fields_ = [("points", ctypes.c_int), ("unique_leaves", ctypes.c_int), ("nodes", ctypes.c_int),
                ("depth", ctypes.c_int), ("level_count", ctypes.c_int * 10), ("vertices", ctypes.c_int),
                ("edges", ctypes.c_int), ("faces", ctypes.c_int), ("crossings", ctypes.c_int),
                ("triangles", ctypes.c_int), ("subdivision_roots", ctypes.c_int),
                ("subdivision_nodes", ctypes.c_int), ("mesh_vertices", ctypes.c_int),
                ("mesh_triangles", ctypes.c_int), ("cg_iterations", ctypes.c_int * 10),
                ("cg_residual", ctypes.c_double * 10), ("iso_value", ctypes.c_float),
                ("error_bits", ctypes.c_uint), ("stage_ms", ctypes.c_float * 6),
                ("kernel_launches", ctypes.c_int), ("graph_replay", ctypes.c_int),
                ("cg_kernel_ms", ctypes.c_float), ("cg_depth_ms", ctypes.c_float * 10),
                ("cg_true_residual", ctypes.c_double * 10), ("cg_residual_checks", ctypes.c_int * 10),
                ("cg_restarts", ctypes.c_int * 10)]


_lib = None


def load_library(path=None):
    """Load libpsr.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(str(p))
    L.psr_config_default.argtypes = [ctypes.POINTER(PsrConfig)]
    L.psr_create.argtypes = [ctypes.POINTER(PsrConfig), ctypes.POINTER(ctypes.c_void_p)]
    L.psr_destroy.argtypes = [ctypes.c_void_p]
    L.psr_reconstruct.argtypes = [ctypes.c_void_p, ctypes.POINTER(PsrPoints), ctypes.POINTER(PsrOptions),
                                  ctypes.POINTER(PsrMesh), ctypes.c_void_p]
    L.psr_submit.argtypes = L.psr_reconstruct.argtypes
    L.psr_submit_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(PsrPoints), ctypes.c_int,
                                   ctypes.POINTER(PsrOptions), ctypes.POINTER(PsrMesh), ctypes.c_void_p]
    L.psr_reconstruct_batch.argtypes = L.psr_submit_batch.argtypes
    L.psr_get_batch_result.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.psr_poll.argtypes = [ctypes.c_void_p]
    L.psr_wait.argtypes = [ctypes.c_void_p]
    L.psr_memory_bytes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]
    L.psr_surfels_to_points.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p]
    L.psr_estimate_normals.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]
    L.psr_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(PsrStats)]
    L.psr_debug_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_size_t)]
    L.psr_status_string.argtypes = [ctypes.c_int]
    L.psr_status_string.restype = ctypes.c_char_p
    L.psr_last_error.argtypes = [ctypes.c_void_p]
    L.psr_last_error.restype = ctypes.c_char_p
    L.psr_morton_sort_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    for fn in EXPORTED:
        if fn not in ("psr_status_string", "psr_last_error"):
            getattr(L, fn).restype = ctypes.c_int
    if path is None:
        _lib = L
    return L


class PsrError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


class Mesh:
    """Output of one reconstruction (unit-cube vertices, int32 triangles)."""

    def __init__(self, vertices, triangles, colors, normals, center, scale):
        self.vertices = vertices
        self.triangles = triangles
        self.colors = colors
        self.normals = normals
        self.center = center
        self.scale = scale

    def world_vertices(self):
        return self.center[None, :] + self.vertices * self.scale


def default_config():
    cfg = PsrConfig()
    load_library().psr_config_default(ctypes.byref(cfg))
    return cfg


class PoissonReconstruction:
    """Drop-in mirror of SparseSurfelFusion::PoissonReconstruction for the GPU path."""

    def __init__(self, max_depth=7, max_points=300000, max_triangles=1000000, max_mesh_vertices=300000,
                 compute_colors=False, compute_normals=False, cg_tolerance=1e-5, cg_max_iterations=10000,
                 max_nodes=0, max_subdivision_nodes=0, device=0, laplacian_epsilon=1e-6, concurrent_stages=True, weld_vertices=False,
                 disable_graphs=False, root_poly_capacity=0, cg_residual_period=0, batch_clouds=1,
                 cg_cluster_ctas=0, cg_cluster_ctas_fine=0):
        self._lib = load_library()
        cfg = default_config()
        cfg.max_depth = max_depth
        cfg.max_points = max_points
        cfg.max_triangles = max_triangles
        cfg.max_mesh_vertices = max_mesh_vertices
        cfg.compute_colors = int(compute_colors)
        cfg.compute_normals = int(compute_normals)
        cfg.cg_tolerance = cg_tolerance
        cfg.cg_max_iterations = cg_max_iterations
        cfg.max_nodes = max_nodes
        cfg.max_subdivision_nodes = max_subdivision_nodes
        cfg.device = device
        cfg.laplacian_epsilon = laplacian_epsilon
        cfg.concurrent_stages = int(concurrent_stages)
        cfg.weld_vertices = int(weld_vertices)
        cfg.disable_graphs = int(disable_graphs)
        cfg.root_poly_capacity = int(root_poly_capacity)
        cfg.cg_residual_period = int(cg_residual_period)
        cfg.batch_clouds = int(batch_clouds)
        cfg.cg_cluster_ctas = int(cg_cluster_ctas)
        cfg.cg_cluster_ctas_fine = int(cg_cluster_ctas_fine)
        self.config = cfg
        h = ctypes.c_void_p()
        st = self._lib.psr_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != PSR_OK:
            raise PsrError(st, "psr_create failed")
        self._h = h
        self._mesh = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.psr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _error(self, st, what):
        msg = self._lib.psr_last_error(self._h).decode()
        return PsrError(st, f"{what}: {self._lib.psr_status_string(st).decode()}: {msg}")

    def SolvePoissionReconstructionMesh(self, xyz, normals, rgb=None, depth=0, cg_iterations=0):
        """Reconstruct from host arrays; returns a Mesh (also kept for the getters)."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        normals = np.ascontiguousarray(normals, np.float32)
        if rgb is not None:
            rgb = np.ascontiguousarray(rgb, np.uint8)
        n = int(xyz.shape[0])
        pts = PsrPoints(xyz.ctypes.data, normals.ctypes.data, rgb.ctypes.data if rgb is not None else None, n,
                        PSR_HOST)
        opt = PsrOptions(int(depth), int(cg_iterations))
        vcap = int(self.config.max_mesh_vertices)
        tcap = int(self.config.max_triangles)
        v = np.empty((vcap, 3), np.float32)
        t = np.empty((tcap, 3), np.int32)
        c = np.empty((vcap, 3), np.float32) if self.config.compute_colors else None
        nm = np.empty((vcap, 3), np.float32) if self.config.compute_normals else None
        mesh = PsrMesh(v.ctypes.data, t.ctypes.data, c.ctypes.data if c is not None else None,
                       nm.ctypes.data if nm is not None else None, vcap, tcap, PSR_HOST, 0, 0)
        st = self._lib.psr_reconstruct(self._h, ctypes.byref(pts), ctypes.byref(opt), ctypes.byref(mesh), None)
        if st != PSR_OK:
            raise self._error(st, "psr_reconstruct")
        nv, nt = mesh.vertex_count, mesh.triangle_count
        self._mesh = Mesh(v[:nv].copy(), t[:nt].copy(), None if c is None else c[:nv].copy(),
                          None if nm is None else nm[:nv].copy(), np.array(mesh.center[:], np.float32),
                          float(mesh.scale))
        return self._mesh

    reconstruct = SolvePoissionReconstructionMesh

    def _host_mesh(self):
        vcap = int(self.config.max_mesh_vertices)
        tcap = int(self.config.max_triangles)
        v = np.empty((vcap, 3), np.float32)
        t = np.empty((tcap, 3), np.int32)
        c = np.empty((vcap, 3), np.float32) if self.config.compute_colors else None
        nm = np.empty((vcap, 3), np.float32) if self.config.compute_normals else None
        desc = PsrMesh(v.ctypes.data, t.ctypes.data, c.ctypes.data if c is not None else None,
                       nm.ctypes.data if nm is not None else None, vcap, tcap, PSR_HOST, 0, 0)
        return desc, (v, t, c, nm)

    def reconstruct_batch(self, clouds, depth=0, cg_iterations=0):
        """Reconstruct up to batch_clouds clouds of one depth in one multi-cloud pass
        (psr_reconstruct_batch).  `clouds`: list of (xyz, normals, rgb or None) host arrays.
        Returns one Mesh per cloud, or a PsrError for a cloud that failed."""
        n = len(clouds)
        keep = []
        pts = (PsrPoints * n)()
        meshes = (PsrMesh * n)()
        bufs = []
        for k, (xyz, nrm, rgb) in enumerate(clouds):
            xyz = np.ascontiguousarray(xyz, np.float32)
            nrm = np.ascontiguousarray(nrm, np.float32)
            rgb = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
            keep.append((xyz, nrm, rgb))
            pts[k] = PsrPoints(xyz.ctypes.data, nrm.ctypes.data, rgb.ctypes.data if rgb is not None else None,
                               int(xyz.shape[0]), PSR_HOST)
            meshes[k], b = self._host_mesh()
            bufs.append(b)
        opt = PsrOptions(int(depth), int(cg_iterations))
        st = self._lib.psr_reconstruct_batch(self._h, pts, n, ctypes.byref(opt), meshes, None)
        if st != PSR_OK and self.batch_result(n - 1)[1].points == 0:
            raise self._error(st, "psr_reconstruct_batch")   # the call itself failed: no per-cloud results
        out = []
        for k in range(n):
            sk = self._lib.psr_get_batch_result(self._h, k, None)
            if sk != PSR_OK:
                out.append(PsrError(sk, f"cloud {k}: {self._lib.psr_status_string(sk).decode()}"))
                continue
            v, t, c, nm = bufs[k]
            m = meshes[k]
            nv, nt = m.vertex_count, m.triangle_count
            out.append(Mesh(v[:nv].copy(), t[:nt].copy(), None if c is None else c[:nv].copy(),
                            None if nm is None else nm[:nv].copy(), np.array(m.center[:], np.float32),
                            float(m.scale)))
        return out

    def submit_batch_device(self, points, meshes, depth=0, cg_iterations=0, stream=None):
        """Enqueue a multi-cloud pass: `points` a ctypes array of PsrPoints (device or pinned
        host pointers), `meshes` a ctypes array of PsrMesh of the same length; returns at
        once (collect with poll / wait, then batch_result)."""
        self._pend = (points, PsrOptions(int(depth), int(cg_iterations)), meshes)
        st = self._lib.psr_submit_batch(self._h, points, len(points), ctypes.byref(self._pend[1]), meshes, stream)
        if st != PSR_OK:
            self._pend = None
            raise self._error(st, "psr_submit_batch")

    def batch_result(self, index):
        """(status, PsrStats) of cloud `index` of the last completed call."""
        s = PsrStats()
        st = self._lib.psr_get_batch_result(self._h, int(index), ctypes.byref(s))
        return st, s

    def reconstruct_device(self, xyz_ptr, nrm_ptr, rgb_ptr, n, depth=0, cg_iterations=0, stream=None,
                           out=None):
        """Reconstruct from device pointers (e.g. torch CUDA tensors' data_ptr())."""
        pts = PsrPoints(xyz_ptr, nrm_ptr, rgb_ptr, int(n), PSR_DEVICE)
        opt = PsrOptions(int(depth), int(cg_iterations))
        mesh = out if out is not None else PsrMesh(None, None, None, None, 0, 0, PSR_HOST, 0, 0)
        st = self._lib.psr_reconstruct(self._h, ctypes.byref(pts), ctypes.byref(opt), ctypes.byref(mesh), stream)
        if st != PSR_OK and not (st == PSR_OUT_OF_CAPACITY and out is None):
            raise self._error(st, "psr_reconstruct")
        return mesh

    # ---- served form: submit, then poll / wait (one reconstruction in flight per handle)
    def submit_device(self, xyz_ptr, nrm_ptr, rgb_ptr, n, out, depth=0, cg_iterations=0, stream=None,
                      location=PSR_DEVICE):
        """Enqueue a reconstruction of the points at the given pointers (device memory, or
        pinned host memory with location=PSR_HOST) into the mesh buffers of ``out`` (a
        PsrMesh, device- or host-resident); returns immediately."""
        self._pend = (PsrPoints(xyz_ptr, nrm_ptr, rgb_ptr, int(n), int(location)),
                      PsrOptions(int(depth), int(cg_iterations)), out)
        pts, opt, mesh = self._pend
        st = self._lib.psr_submit(self._h, ctypes.byref(pts), ctypes.byref(opt), ctypes.byref(mesh), stream)
        if st != PSR_OK:
            self._pend = None
            raise self._error(st, "psr_submit")

    def poll(self):
        """True once the submitted reconstruction has completed (its mesh counts are then
        set in the PsrMesh given to submit_device); raises on a failed reconstruction."""
        st = self._lib.psr_poll(self._h)
        if st == PSR_PENDING:
            return False
        self._pend = None
        if st != PSR_OK:
            raise self._error(st, "psr_poll")
        return True

    def wait(self):
        st = self._lib.psr_wait(self._h)
        self._pend = None
        if st != PSR_OK:
            raise self._error(st, "psr_wait")

    # ---- file inputs: the reference's readTXTFile / readPCDFile / readPLYFile and
    # getDenseSurfel (mesh/PoissonReconstruction.cpp:63-135, :176-179)
    def readPointFile(self, path, viewpoint=(0.0, 0.0, 0.0)):
        """Reads a .ply / .pcd / .txt cloud (plyio.read_points); a file without normals gets
        them estimated on the GPU as the reference's readPCDFile does through PCL (k = 10,
        viewpoint at the origin).  Returns (xyz, normals, rgb or None), also kept for
        getDenseSurfel()."""
        import plyio
        xyz, nrm, rgb = plyio.read_points(path)
        if nrm is None:
            nrm = self.CalculatePointCloudNormal(xyz, viewpoint)
            # no normal (fewer than 3 samples, or all neighbours at one position): a zero
            # normal, which adds nothing to the vector field, instead of a NaN that the
            # reconstruction rejects
            nrm[~np.isfinite(nrm).all(axis=1)] = 0.0
        self._surfel = (xyz, nrm, rgb)
        return self._surfel

    def readTXTFile(self, path):
        return self.readPointFile(path)

    def readPCDFile(self, path):
        return self.readPointFile(path)

    def readPLYFile(self, path):
        """Oriented points of a PLY file (the reference only displays the file in a PCL viewer)."""
        return self.readPointFile(path)

    def getDenseSurfel(self):
        """The points of the last file read: (xyz, normals, rgb or None), the arguments of
        SolvePoissionReconstructionMesh."""
        return getattr(self, "_surfel", None)

    def CalculatePointCloudNormal(self, xyz, viewpoint=(0.0, 0.0, 0.0)):
        """Normals of an unoriented cloud (float32 N x 3, host): the smallest-eigenvalue
        eigenvector of each point's 10 nearest neighbours' covariance, flipped towards
        `viewpoint` (mesh/PoissonReconstruction.cpp:137-161).  Returns float32 N x 3."""
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        out = np.empty_like(xyz)
        vp = np.asarray(viewpoint, np.float32)
        st = self._lib.psr_estimate_normals(self._h, xyz.ctypes.data, xyz.shape[0], PSR_HOST, out.ctypes.data,
                                            vp.ctypes.data, None)
        if st != PSR_OK:
            raise self._error(st, "psr_estimate_normals")
        return out

    def estimate_normals_device(self, xyz_ptr, n, out_ptr, viewpoint=(0.0, 0.0, 0.0), stream=None):
        """The same on device buffers (n x 3 floats each); blocks until written."""
        vp = np.asarray(viewpoint, np.float32)
        st = self._lib.psr_estimate_normals(self._h, xyz_ptr, int(n), PSR_DEVICE, out_ptr, vp.ctypes.data, stream)
        if st != PSR_OK:
            raise self._error(st, "psr_estimate_normals")

    def memory_bytes(self):
        b = ctypes.c_size_t(0)
        self._lib.psr_memory_bytes(self._h, ctypes.byref(b))
        return int(b.value)

    def GetRebuildMeshVertices(self):
        return None if self._mesh is None else self._mesh.vertices

    def GetRebuildMeshTriangleIndices(self):
        return None if self._mesh is None else self._mesh.triangles

    def stats(self):
        s = PsrStats()
        self._lib.psr_get_stats(self._h, ctypes.byref(s))
        return s

    def launch_count(self):
        return self.stats().kernel_launches

    def debug(self, name, dtype=np.int32, rows=None):
        """Copy an internal device array of the last reconstruction to host."""
        nb = ctypes.c_size_t()
        st = self._lib.psr_debug_array(self._h, name.encode(), None, 0, ctypes.byref(nb))
        if st != PSR_OK:
            raise self._error(st, f"psr_debug_array({name})")
        buf = np.empty(nb.value // np.dtype(dtype).itemsize, dtype)
        st = self._lib.psr_debug_array(self._h, name.encode(), buf.ctypes.data, buf.nbytes, ctypes.byref(nb))
        if st != PSR_OK:
            raise self._error(st, f"psr_debug_array({name})")
        if rows:
            buf = buf.reshape(rows, -1)
        return buf
