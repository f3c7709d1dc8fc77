"""Served form of the reconstruction: continuous batching over resident slots.

The reference reconstructs one cloud per blocking call (mesh/PoissonReconstruction.cpp:
195-245).  Here a Server owns K slots -- one handle (pre-allocated workspace, CUDA graphs),
one CUDA stream and one device-resident output mesh each -- and one host thread drives
them through the non-blocking C ABI (psr_submit / psr_poll): a request that arrives while
others are on the GPU is admitted as soon as a slot is free, and the slots' work overlaps
on the device.  K is bounded by a device-memory budget (the handles' workspace sizes).
Each slot's pipeline is one chain (concurrent_stages off): with K reconstructions
already overlapping, a second stream per slot only adds contention.
Results are the same as psr_reconstruct alone (the pipeline is deterministic per handle).

Device buffers for the slots' outputs come from PyTorch (plumbing only).
"""
import time
from dataclasses import dataclass

import numpy as np

import psr


@dataclass
class Request:
    """One cloud to reconstruct: xyz / normals (/ rgb) are float32 N x 3 (uint8 N x 3)
    tensors, either on the GPU or in pinned host memory (copied by the reconstruction's
    own stream), alive until the request completes."""
    xyz: object
    normals: object
    rgb: object = None
    depth: int = 0
    tag: object = None
    arrival: float = 0.0          # host clock (time.perf_counter) when it arrived
    # filled on completion
    vertices: object = None       # device tensor V x 3 (unit cube)
    triangles: object = None      # device tensor T x 3
    colors: object = None
    normals_out: object = None
    center: tuple = ()
    scale: float = 0.0
    admitted: float = 0.0
    finished: float = 0.0
    error: str = ""

    @property
    def latency_ms(self):
        return 1000.0 * (self.finished - self.arrival)


@dataclass
class _Slot:
    recon: object
    stream: object
    out: list
    mesh: object = None
    req: Request = None


class Server:
    """K concurrent reconstruction slots on one GPU, driven from one host thread."""

    def __init__(self, slots=8, max_depth=7, max_points=300000, max_triangles=1000000, max_mesh_vertices=300000,
                 compute_colors=True, compute_normals=True, device=0, memory_budget=None, host_outputs=False,
                 **caps):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.vcap, self.tcap = max_mesh_vertices, max_triangles
        self.compute_colors, self.compute_normals = compute_colors, compute_normals
        self.host_outputs = host_outputs
        self.slots = []
        for k in range(slots):
            r = psr.PoissonReconstruction(max_depth=max_depth, max_points=max_points, max_triangles=max_triangles,
                                          max_mesh_vertices=max_mesh_vertices, compute_colors=compute_colors,
                                          compute_normals=compute_normals, device=device,
                                          **{"concurrent_stages": False, **caps})
            if memory_budget is not None and (k + 1) * self.slot_bytes(r) > memory_budget:
                r.close()
                if k == 0:
                    raise ValueError(f"memory_budget {memory_budget} B is below one slot "
                                     f"({self.slot_bytes(r)} B: workspace and output buffers)")
                break
            def buf(shape, dtype):
                if host_outputs:
                    return torch.empty(shape, dtype=dtype).pin_memory()
                return torch.empty(shape, dtype=dtype, device=self.dev)
            out = [buf((self.vcap, 3), torch.float32), buf((self.tcap, 3), torch.int32),
                   buf((self.vcap, 3), torch.float32) if compute_colors else None,
                   buf((self.vcap, 3), torch.float32) if compute_normals else None]
            self.slots.append(_Slot(r, torch.cuda.Stream(self.dev), out))
        self.queue = []
        self.done = []

    def slot_bytes(self, recon):
        """Device bytes of one slot: the handle's workspace plus its output mesh buffers
        (vertices, triangles, and colours / normals when computed; none on the device when
        outputs go to pinned host memory)."""
        out = 0
        if not self.host_outputs:
            per_vertex = 12 * (1 + int(self.compute_colors) + int(self.compute_normals))
            out = per_vertex * self.vcap + 12 * self.tcap
        return recon.memory_bytes() + out

    def close(self):
        for sl in self.slots:
            if sl.req is not None:
                sl.recon.wait()
            sl.recon.close()
        self.slots = []

    def submit(self, req):
        if not req.arrival:
            req.arrival = time.perf_counter()
        self.queue.append(req)

    def _admit(self, sl, req):
        o = sl.out
        sl.mesh = psr.PsrMesh(o[0].data_ptr(), o[1].data_ptr(),
                              o[2].data_ptr() if (o[2] is not None and req.rgb is not None) else None,
                              o[3].data_ptr() if o[3] is not None else None, self.vcap, self.tcap,
                              psr.PSR_HOST if self.host_outputs else psr.PSR_DEVICE, 0, 0)
        req.admitted = time.perf_counter()
        sl.req = req
        try:
            sl.recon.submit_device(req.xyz.data_ptr(), req.normals.data_ptr(),
                                   req.rgb.data_ptr() if req.rgb is not None else None, req.xyz.shape[0],
                                   sl.mesh, depth=req.depth, stream=sl.stream.cuda_stream,
                                   location=psr.PSR_DEVICE if req.xyz.is_cuda else psr.PSR_HOST)
        except psr.PsrError as e:
            self._finish(sl, str(e))

    def _finish(self, sl, error=""):
        req, m = sl.req, sl.mesh
        req.finished = time.perf_counter()
        req.error = error
        if not error:
            with self.torch.cuda.stream(sl.stream):   # device copies stay ordered before the slot's next run
                nv, nt = m.vertex_count, m.triangle_count
                req.vertices = sl.out[0][:nv].clone()
                req.triangles = sl.out[1][:nt].clone()
                req.colors = sl.out[2][:nv].clone() if (sl.out[2] is not None and m.colors) else None
                req.normals_out = sl.out[3][:nv].clone() if sl.out[3] is not None else None
            if not self.host_outputs:
                sl.stream.synchronize()   # only the copies above are left on the slot's stream
            req.center = tuple(m.center)
            req.scale = m.scale
        sl.req = None
        self.done.append(req)

    def step(self):
        """Collects finished slots and admits queued requests; returns the number of busy slots."""
        busy = 0
        for sl in self.slots:
            if sl.req is not None:
                try:
                    fin = sl.recon.poll()
                except psr.PsrError as e:
                    self._finish(sl, str(e))
                    fin = False
                if fin:
                    self._finish(sl)
            if sl.req is None and self.queue:
                self._admit(sl, self.queue.pop(0))
            busy += sl.req is not None
        return busy

    def run(self, requests, arrivals=None, idle_sleep=20e-6):
        """Serves `requests` (arriving at host times `arrivals`, seconds from now, or all at
        once) until every one has completed; returns them in completion order."""
        t0 = time.perf_counter()
        pending = list(zip(arrivals if arrivals is not None else [0.0] * len(requests), requests))
        pending.sort(key=lambda p: p[0])
        self.done = []
        i = 0
        while len(self.done) < len(requests):
            now = time.perf_counter() - t0
            while i < len(pending) and pending[i][0] <= now:
                pending[i][1].arrival = t0 + pending[i][0]
                self.submit(pending[i][1])
                i += 1
            if self.step() == 0 and i < len(pending):
                time.sleep(max(0.0, min(idle_sleep, pending[i][0] - now)))
        return self.done


def latency_summary(done):
    lat = np.array([r.latency_ms for r in done if not r.error])
    if lat.size == 0:
        return {"p50_ms": None, "p99_ms": None}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
