"""Served form of the reconstruction: continuous batching over resident slots.

The reference reconstructs one cloud per blocking call (mesh/PoissonReconstruction.cpp:
195-245).  Here a Server owns K slots -- one handle (pre-allocated workspace, CUDA graphs),
one CUDA stream and one device-resident output mesh each -- and one host thread drives
them through the non-blocking C ABI (psr_submit / psr_poll): a request that arrives while
others are on the GPU is admitted as soon as a slot is free, and the slots' work overlaps
on the device.  K is bounded by a device-memory budget (the handles' workspaces and output buffers); slots
of several sizes admit each cloud by its footprint (point count and depth).
Each slot's pipeline is one chain (concurrent_stages off): with K reconstructions
already overlapping, a second stream per slot only adds contention.
Results are the same as psr_reconstruct alone (the pipeline is deterministic per handle).

Output buffers come from PyTorch (plumbing only): device memory, or pinned host memory
with `host_outputs` (the GPU writes the meshes there directly).  Each slot writes its
meshes into a ring of `out_sets` buffer sets and a finished request holds views of its set,
not copies: they stay valid until its slot starts the out_sets-th request after it (copy
them to keep them longer).
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
    vertices: object = None       # V x 3 (unit cube), T x 3: views of the slot's output
    triangles: object = None      # buffers (device, or pinned host memory; see above)
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
    out: list                     # output buffers [vertices, triangles, colours, normals]
    mesh: object = None
    ring: list = None             # the output buffer sets `out` rotates over
    ring_at: int = 0
    req: Request = None
    max_points: int = 1 << 30     # the largest cloud and depth the slot's workspace takes
    max_depth: int = 9
    vcap: int = 0                 # output capacities (0: the server's)
    tcap: int = 0

    def fits(self, req):
        return req.xyz.shape[0] <= self.max_points and (req.depth or self.max_depth) <= self.max_depth


class Server:
    """Concurrent reconstruction slots on one GPU, driven from one host thread.

    `slots` handles of one size (max_points, max_depth, output capacities), or `classes`:
    a list of dicts, each {"count": n, "max_points": ..., "max_depth": ..., "max_triangles":
    ..., "max_mesh_vertices": ...} (other handle settings as keyword arguments), for clouds
    of uneven size: a request is admitted into the first free slot whose workspace takes its
    point count and depth, so small clouds do not hold a workspace sized for the largest.
    `memory_budget` (bytes) bounds the device memory of all slots: each slot costs its
    handle's workspace plus its output buffers; slots of a class are created while the
    budget allows, classes in the order given, at least one slot per class."""

    def __init__(self, slots=8, max_depth=7, max_points=300000, max_triangles=1000000, max_mesh_vertices=300000,
                 compute_colors=True, compute_normals=True, device=0, memory_budget=None, host_outputs=False,
                 classes=None, out_sets=2, **caps):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.vcap, self.tcap = max_mesh_vertices, max_triangles
        self.compute_colors, self.compute_normals = compute_colors, compute_normals
        self.host_outputs = host_outputs
        self.slots = []
        self.rejected = []
        if classes is None:
            classes = [dict(count=slots, max_points=max_points, max_depth=max_depth, max_triangles=max_triangles,
                            max_mesh_vertices=max_mesh_vertices)]
        used = 0
        for ci, cl in enumerate(classes):
            cl = dict(cl)
            count = cl.pop("count")
            vcap, tcap = cl.get("max_mesh_vertices", max_mesh_vertices), cl.get("max_triangles", max_triangles)
            for k in range(count):
                r = psr.PoissonReconstruction(compute_colors=compute_colors, compute_normals=compute_normals,
                                              device=device, **{"concurrent_stages": False, **caps, **cl})
                cost = self.slot_bytes(r, vcap, tcap, out_sets)
                if memory_budget is not None and used + cost > memory_budget:
                    r.close()
                    if k == 0:
                        self.close()
                        raise ValueError(f"memory_budget {memory_budget} B leaves no slot of class {ci} "
                                         f"({cost} B: workspace and output buffers)")
                    break
                used += cost
                def buf(shape, dtype):
                    if host_outputs:
                        return torch.empty(shape, dtype=dtype).pin_memory()
                    return torch.empty(shape, dtype=dtype, device=self.dev)
                def out_set():
                    return [buf((vcap, 3), torch.float32), buf((tcap, 3), torch.int32),
                            buf((vcap, 3), torch.float32) if compute_colors else None,
                            buf((vcap, 3), torch.float32) if compute_normals else None]
                ring = [out_set() for _ in range(max(2, out_sets))]
                self.slots.append(_Slot(r, torch.cuda.Stream(self.dev), ring[0], ring=ring,
                                        max_points=r.config.max_points, max_depth=r.config.max_depth, vcap=vcap,
                                        tcap=tcap))
        self.memory_bytes = used
        self.queue = []
        self.done = []

    def slot_bytes(self, recon, vcap=None, tcap=None, out_sets=2):
        """Device bytes of one slot: the handle's workspace plus its output mesh buffer sets
        (vertices, triangles, and colours / normals when computed; none on the device when
        outputs go to pinned host memory)."""
        vcap = self.vcap if vcap is None else vcap
        tcap = self.tcap if tcap is None else tcap
        out = 0
        if not self.host_outputs:
            per_vertex = 12 * (1 + int(self.compute_colors) + int(self.compute_normals))
            out = max(2, out_sets) * (per_vertex * vcap + 12 * tcap)
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
        if not any(sl.fits(req) for sl in self.slots):
            # no slot of this server takes the cloud: finished at once with an error
            req.admitted = req.finished = time.perf_counter()
            req.error = "rejected: no slot takes this cloud's point count and depth"
            self.rejected.append(req)
            self.done.append(req)
            return
        self.queue.append(req)

    def _admit(self, sl, req):
        o = sl.out
        vcap, tcap = (sl.vcap or self.vcap), (sl.tcap or self.tcap)
        sl.mesh = psr.PsrMesh(o[0].data_ptr(), o[1].data_ptr(),
                              o[2].data_ptr() if (o[2] is not None and req.rgb is not None) else None,
                              o[3].data_ptr() if o[3] is not None else None, vcap, tcap,
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
            nv, nt = m.vertex_count, m.triangle_count
            # the reconstruction wrote its mesh into this set before its completion event: the
            # request keeps views and the slot's next request writes the next set of the ring
            o = sl.out
            req.vertices = o[0][:nv]
            req.triangles = o[1][:nt]
            req.colors = o[2][:nv] if (o[2] is not None and m.colors) else None
            req.normals_out = o[3][:nv] if o[3] is not None else None
            if sl.ring:
                sl.ring_at = (sl.ring_at + 1) % len(sl.ring)
                sl.out = sl.ring[sl.ring_at]
            req.center = tuple(m.center)
            req.scale = m.scale
        sl.req = None
        self.done.append(req)

    def step(self):
        """Collects finished slots and admits queued requests (the oldest request that fits
        a free slot first); returns the number of busy slots."""
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
                for qi, rq in enumerate(self.queue):
                    if sl.fits(rq):
                        self._admit(sl, self.queue.pop(qi))
                        break
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
