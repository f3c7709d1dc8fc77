#!/usr/bin/env python3
"""Benchmark of the GB300 Poisson reconstruction path.

Workload (default): the depth-7, 200,000-point torus-plus-ellipsoid cloud with colour
(seeded synthetic, see synthetic.py).  A step is one reconstruction of one cloud through
the C ABI (psr_reconstruct): octree, splat, divergence, per-depth CG, marching cubes with
subdivision, colour and normal transfer.

Reported metric: reconstructions per second (higher is better) and p99 latency.
  value : device-resident inputs and outputs, CUDA-event time per step on the launching
          stream, L2 flushed (256 MiB write) between steps outside the timed events
  e2e   : host inputs / host outputs through the same C ABI call (H2D + D2H inside)
Multi-GPU (torchrun): every rank reconstructs its own clouds (no collective on the data
path, weak scaling); the step time is the max over ranks.

--impl reference: the reference path has no CPU implementation and its CUDA code cannot be
built on the benchmark machine, so the reference arm times the CPU restatement of the
same algorithm (oracle/, FP64, OpenMP over all host cores) on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "poisson-surface-reconstruction-gpu_gb300"
sys.path[:0] = [str(PKG), str(ROOT / "oracle")]

METRIC = "depth-7 200k-pt recons/s & p99 ms, served vs plain, at FP64-checked accuracy"
UNIT = "recons/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="torus_ellipsoid200k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--slots", type=int, default=8, help="concurrent reconstructions of the served leg")
    ap.add_argument("--batch", type=int, default=16, help="clouds per multi-cloud launch in the batch leg")
    ap.add_argument("--serve-seconds", type=float, default=15.0,
                    help="open-loop duration of the serving-loop leg (Poisson arrivals, mixed sizes and depths)")
    ap.add_argument("--no-serve-mix", action="store_true", help="skip the serving-loop leg")
    ap.add_argument("--no-mix-batch", action="store_true", help="skip the 256-cloud multi-cloud mix leg")
    ap.add_argument("--no-large", action="store_true", help="skip the 2M-point depth-9 leg")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def rank_clouds(rank, slots):
    """Cloud seeds a rank reconstructs: slot k of the served leg takes rank * slots + k, and
    the plain and host legs take the rank's slot-0 cloud.  Ranks hold disjoint clouds (the
    shards of the job); rank 0 of a 1-GPU run uses clouds 0 .. slots - 1."""
    return [rank * slots + k for k in range(slots)]


def job_rates(world, steps, slots, totals_ms, reduce_max=None):
    """Whole-job reconstructions/s from each rank's timed totals (ms): the plain, plain-e2e,
    served and served-e2e legs.  The job's time is the slowest rank's (`reduce_max` takes
    the element-wise maximum over ranks, e.g. an all_reduce MAX); every rank processed
    `steps` clouds in the plain legs and `slots * steps` in the served legs."""
    t = list(totals_ms)
    if world > 1 and reduce_max is not None:
        t = reduce_max(t)
    t_dev, t_e2e, t_sdev, t_se2e = t
    return {"plain": world * steps / (t_dev / 1000.0),
            "plain_e2e": world * steps / (t_e2e / 1000.0),
            "served": world * slots * steps / (t_sdev / 1000.0),
            "served_e2e": world * slots * steps / (t_se2e / 1000.0),
            "max_totals_ms": t}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        out.update(sm_mhz=float(np.median(sm)) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        return out


def cpu_baseline(xyz, nrm, rgb, depth, budget_s=20.0):
    """The oracle (CPU restatement, FP64, OpenMP) on the same cloud, repeated within a budget."""
    import oracle
    o = oracle.Oracle()
    rgbf = None if rgb is None else rgb.astype(np.float32) / np.float32(255.0)
    times = []
    t_all = time.time()
    while True:
        t = time.time()
        rc = o.run(xyz, nrm, rgbf, depth=depth)
        times.append(time.time() - t)
        if rc != 0 or time.time() - t_all > budget_s * 0.5 or len(times) >= 5:
            break
    per = float(np.median(times))
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": 1.0 / per, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(times)} full reconstruction(s) of the {len(xyz)}-point depth-{depth} cloud, "
                      f"median {per:.2f} s each"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import synthetic as syn
    xyz, nrm, rgb, depth = syn.workload(args.workload)
    import oracle
    oracle.build()
    o = oracle.Oracle()
    rgbf = None if rgb is None else rgb.astype(np.float32) / np.float32(255.0)
    for _ in range(args.warmup):
        o.run(xyz, nrm, rgbf, depth=depth)
    times = []
    for _ in range(args.steps):
        t = time.time()
        o.run(xyz, nrm, rgbf, depth=depth)
        times.append(time.time() - t)
    total = sum(times)
    value = args.steps / total
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"{args.workload} (N={len(xyz)}, depth {depth}, colour)", "l2": "n/a (host)"},
            "p50_ms": 1000 * float(np.median(times)), "p99_ms": 1000 * float(np.percentile(times, 99)),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"full reconstruction of the {len(xyz)}-point cloud per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as ge
    if rank == 0 or world == 1:
        ge.build()
    if world > 1:
        dist.barrier()
    import psr
    import synthetic as syn

    seeds = rank_clouds(rank, args.slots)
    xyz, nrm, rgb, depth = syn.workload(args.workload, cloud=seeds[0])
    n = len(xyz)
    r = psr.PoissonReconstruction(max_depth=depth, max_points=max(300000, n), max_triangles=1000000,
                                  max_mesh_vertices=300000, compute_colors=rgb is not None,
                                  compute_normals=True, device=local)
    dev = torch.device("cuda", local)
    d_xyz = torch.from_numpy(xyz).to(dev)
    d_nrm = torch.from_numpy(nrm).to(dev)
    d_rgb = torch.from_numpy(rgb).to(dev) if rgb is not None else None
    vcap, tcap = 300000, 1000000
    o_v = torch.empty((vcap, 3), dtype=torch.float32, device=dev)
    o_t = torch.empty((tcap, 3), dtype=torch.int32, device=dev)
    o_c = torch.empty((vcap, 3), dtype=torch.float32, device=dev)
    o_n = torch.empty((vcap, 3), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def dev_mesh():
        return psr.PsrMesh(o_v.data_ptr(), o_t.data_ptr(), o_c.data_ptr() if rgb is not None else None,
                           o_n.data_ptr(), vcap, tcap, psr.PSR_DEVICE, 0, 0)

    def step_device():
        m = dev_mesh()
        r.reconstruct_device(d_xyz.data_ptr(), d_nrm.data_ptr(), d_rgb.data_ptr() if d_rgb is not None else None,
                             n, depth=depth, stream=sptr, out=m)
        return m

    # host (pinned) buffers for the end-to-end leg
    h_xyz = torch.from_numpy(xyz).pin_memory()
    h_nrm = torch.from_numpy(nrm).pin_memory()
    h_rgb = torch.from_numpy(rgb).pin_memory() if rgb is not None else None
    h_v = torch.empty((vcap, 3), dtype=torch.float32).pin_memory()
    h_t = torch.empty((tcap, 3), dtype=torch.int32).pin_memory()
    h_c = torch.empty((vcap, 3), dtype=torch.float32).pin_memory()
    h_n = torch.empty((vcap, 3), dtype=torch.float32).pin_memory()

    def step_host():
        pts = psr.PsrPoints(h_xyz.data_ptr(), h_nrm.data_ptr(), h_rgb.data_ptr() if h_rgb is not None else None, n,
                            psr.PSR_HOST)
        m = psr.PsrMesh(h_v.data_ptr(), h_t.data_ptr(), h_c.data_ptr() if h_rgb is not None else None,
                        h_n.data_ptr(), vcap, tcap, psr.PSR_HOST, 0, 0)
        opt = psr.PsrOptions(depth, 0)
        import ctypes
        st = r._lib.psr_reconstruct(r._h, ctypes.byref(pts), ctypes.byref(opt), ctypes.byref(m), sptr)
        if st != 0:
            raise r._error(st, "psr_reconstruct")
        return m

    for _ in range(max(args.warmup, 3)):
        step_device()
        step_host()
    torch.cuda.synchronize(dev)

    cg_samples = []

    def timed(fn, k):
        times = []
        last = None
        for _ in range(k):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            last = fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
            if fn is step_device:
                cg_samples.append(r.stats().cg_kernel_ms)   # CUDA events around the CG kernel
        return np.array(times), last

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    # served slots: distinct seeded clouds of the same workload, staged on the device
    # (value) and in pinned host memory (e2e)
    from serve import Server
    dclouds, hclouds = [], []
    for k in range(args.slots):
        cx, cn, cc, _ = syn.workload(args.workload, cloud=seeds[k]) if k else (xyz, nrm, rgb, depth)
        dclouds.append((torch.from_numpy(cx).to(dev), torch.from_numpy(cn).to(dev),
                        torch.from_numpy(cc).to(dev) if cc is not None else None, depth))
        hclouds.append((torch.from_numpy(cx).pin_memory(), torch.from_numpy(cn).pin_memory(),
                        torch.from_numpy(cc).pin_memory() if cc is not None else None, depth))
    caps = dict(max_depth=depth, max_points=max(300000, n), max_triangles=1000000, max_mesh_vertices=300000,
                compute_colors=rgb is not None, compute_normals=True, device=local)
    # launch shapes of the served slots chosen by the autotuner (CG cluster sizes)
    import autotune
    from serve import Request as _Req
    def tune_requests():
        return [_Req(xyz=c[0], normals=c[1], rgb=c[2], depth=c[3]) for _ in range(2) for c in dclouds]
    tuned, tune_table = autotune.tune_served(lambda **kw: Server(slots=args.slots, **caps, **kw), tune_requests,
                                             torch, dev)
    tuned_kw = dict(cg_cluster_ctas=tuned[0], cg_cluster_ctas_fine=tuned[1])
    server = Server(slots=args.slots, **caps, **tuned_kw)
    server_h = Server(slots=args.slots, host_outputs=True, **caps, **tuned_kw)
    served_leg(server, dclouds, 2, torch, dev)
    served_leg(server_h, hclouds, 2, torch, dev)
    with ClockSampler(local) as clk:
        t_dev, m_dev = timed(step_device, args.steps)
        t_e2e, m_host = timed(step_host, args.steps)
        s_dev, s_lat, s_stages = served_leg(server, dclouds, args.steps, torch, dev)
        s_e2e, s_lat_e2e, _ = served_leg(server_h, hclouds, args.steps, torch, dev)
        # open loop at 70% of the measured served throughput: arrival-to-completion latency
        rate = 0.7 * args.slots * args.steps / (float(s_dev) / 1000.0)
        ol_lat = open_loop_leg(server, dclouds, args.slots * args.steps, rate)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    st = r.stats()
    def all_max(vals):
        tt = torch.tensor(vals, dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        return tt.tolist()

    K = args.slots
    rates = job_rates(world, args.steps, K, [float(t_dev.sum()), float(t_e2e.sum()), float(s_dev), float(s_e2e)],
                      all_max)
    tot_dev, tot_e2e, tot_sdev, tot_se2e = rates["max_totals_ms"]
    plain_value, plain_e2e = rates["plain"], rates["plain_e2e"]
    value, e2e_value = rates["served"], rates["served_e2e"]
    clocks = clk.summary()
    h2d = n * (12 + 12 + (3 if rgb is not None else 0))
    d2h = m_host.vertex_count * 12 * (3 if rgb is not None else 2) + m_host.triangle_count * 12
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    # roofline of the dominant kernel, the per-depth CG (latency bound: its vectors stay
    # in L2), timed by the solve-stage events
    import json as _j
    peaks = {}
    try:
        peaks = _j.load(open(ROOT / "MEASURED_PEAKS.json"))
    except Exception:
        pass
    peak_hbm = float(peaks.get("hbm_gbs", 6800.0))
    M = st.nodes
    # algorithmic bytes of one CG row-iteration of the matrix-free operator: the row's
    # residual and previous direction read (8 B), its new direction and residual written
    # (8 B), x read and written (8 B); the neighbours' values are the same vectors, counted
    # once per row, and the neighbour / descriptor table is built once per solve
    row_bytes = 24
    cg_bytes = 0
    for d in range(depth + 1):
        cg_bytes += st.level_count[d] * row_bytes * st.cg_iterations[d]
    cg_ms = float(np.mean(cg_samples)) if cg_samples else st.cg_kernel_ms
    roofline = {"bound": "hbm", "kernel": "CG of all depths: k_cg_cluster (depth D on 16 CTAs; D-1, D-2 on 8-CTA "
                                          "clusters) and k_cg_cta (coarser depths), concurrent, timed together",
                "achieved": cg_bytes / (cg_ms * 1e-3) / 1e9 if cg_ms > 0 else None, "peak": peak_hbm,
                "unit": "GB/s", "frac": None, "traffic": None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s",
                "algorithmic_bytes": cg_bytes, "launch_ms": cg_ms,
                "note": "vectors resident in shared memory, descriptor table in L2 (DRAM traffic ~3 MB per "
                        "reconstruction): the HBM fraction does not bound it",
                "limiter": "two cluster barriers and the distributed-shared-memory gathers of every iteration",
                "us_per_iteration_depth_d": (1000.0 * st.cg_depth_ms[depth] / st.cg_iterations[depth]
                                             if st.cg_iterations[depth] else None),
                "sm_ms_per_recon": None}
    # DRAM traffic of one launch, from the committed ncu summary of the same kernel and workload
    try:
        for line in open(ROOT / "profiles" / "cg_cluster_torus200k_d7.md"):
            if line.startswith("traffic_bytes_per_launch:") and args.workload == "torus_ellipsoid200k":
                roofline["traffic"] = int(line.split(":")[1])
                roofline["traffic_source"] = "profiles/cg_cluster_torus200k_d7.md (ncu dram__bytes_read+write)"
    except OSError:
        pass
    if roofline["achieved"]:
        roofline["frac"] = roofline["achieved"] / peak_hbm
    # SM time of the CG per reconstruction: every depth's cluster or CTA holds its SMs for
    # its own device time (one 1024-thread CTA per SM)
    cl = 16 if depth >= 2 else 1
    sm_ms = 0.0
    for d in range(depth + 1):
        ctas = cl if d == depth else (8 if d >= depth - 2 and depth >= 5 else 1)
        sm_ms += ctas * st.cg_depth_ms[d]
    roofline["sm_ms_per_recon"] = round(sm_ms, 3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_sdev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (CG dots, norms and iso-value sums in f64 across warps / CTAs)", "data": "synthetic",
            "impl": "gpu",
            "config": {"workload": f"{args.workload} (N={n}, depth {depth}, colour, normals)",
                       "path": f"served: Server with {K} slots (handle + stream + CUDA graphs each), one host "
                               f"thread, psr_submit / psr_poll continuous batching; a step = one cloud per slot",
                       "l2": f"working set of {K} concurrent reconstructions exceeds L2; plain leg flushes 256 MiB "
                             f"between steps"},
            "p50_ms": float(np.median(ol_lat)), "p99_ms": float(np.percentile(ol_lat, 99)),
            "latency": {"kind": "open-loop Poisson arrivals at 70% of the served throughput, arrival to completion",
                        "rate_per_s": round(rate, 1), "requests": int(ol_lat.size),
                        "service_p50_ms": float(np.median(s_lat)), "service_p99_ms": float(np.percentile(s_lat, 99))},
            "plain": {"value": plain_value, "unit": UNIT, "ms_per_step": tot_dev / args.steps,
                      "p50_ms": float(np.median(t_dev)), "p99_ms": float(np.percentile(t_dev, 99)),
                      "e2e_value": plain_e2e},
            "served_vs_plain": value / plain_value,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": K * h2d, "d2h_bytes_per_step": K * d2h,
                    "p50_ms": float(np.median(s_lat_e2e)), "p99_ms": float(np.percentile(s_lat_e2e, 99))},
            "stage_ms": [round(x, 4) for x in st.stage_ms], "served_stage_ms": s_stages,
            "cg_depth_ms": [round(x, 4) for x in st.cg_depth_ms[:depth + 1]], "nodes": M, "cg_iterations": list(st.cg_iterations[:depth + 1]),
            "mesh": {"vertices": m_host.vertex_count, "triangles": m_host.triangle_count},
            # kernels launched in the timed served leg: per reconstruction the graph's kernel
            # nodes + the output copy kernel, K reconstructions per step
            "gpu_launches": (int(st_launches(server.slots[0].recon)) + 1) * K * args.steps,
            "gpu_launches_per_recon": int(st_launches(server.slots[0].recon)) + 1,
            "roofline": roofline, "clocks": clocks,
            "autotune": {"chosen": {"cg_cluster_ctas": tuned[0], "cg_cluster_ctas_fine": tuned[1]},
                         "served_recons_per_s": {f"{a}x{b}": (round(v, 1) if v else None)
                                                 for (a, b), v in tune_table.items()},
                         "plain": "cg_cluster_ctas 16 (the device's widest cluster), fine 8"}}
    line.update(side_legs(psr, r, caps, d_xyz, d_nrm, d_rgb, n, depth, dev_mesh, stream, torch, st))
    try:
        line["batch"] = batch_leg(psr, {**caps, **tuned_kw}, dclouds, args.steps, torch, dev, args.batch)
        line["batch"]["vs_plain"] = line["batch"]["value"] / plain_value
    except Exception as e:   # reported, not fatal: the headline legs are above
        line["batch"] = {"error": str(e)}
    if not args.no_serve_mix:
        try:
            import serve as serve_mod
            line["serve_mix"] = serve_mix_leg(psr, serve_mod, syn, torch, dev, args.serve_seconds)
        except Exception as e:
            line["serve_mix"] = {"error": str(e)}
    if not args.no_mix_batch:
        try:
            line["mix_batch"] = mix_batch_leg(psr, syn, torch, dev)
        except Exception as e:
            line["mix_batch"] = {"error": str(e)}
    if not args.no_large:
        try:
            line["large"] = large_leg(psr, syn, torch, dev)
        except Exception as e:
            line["large"] = {"error": str(e)}
    if not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(xyz, nrm, rgb, depth)
        except Exception as e:
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def side_legs(psr, r, caps, d_xyz, d_nrm, d_rgb, n, depth, dev_mesh, stream, torch, st, reps=10):
    """Stages beside the reconstruction, timed after the headline legs with CUDA events on
    the launching stream (device-resident arrays, median of `reps` after 3 warm-ups):
    normal estimation of the cloud as if unoriented (psr_estimate_normals, k = 10), and the
    plain leg on a handle that welds the vertices repeated by subdivided regions."""
    def median_ms(fn):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))
    out = {}
    d_out = torch.empty_like(d_xyz)
    ms = median_ms(lambda: r.estimate_normals_device(d_xyz.data_ptr(), n, d_out.data_ptr(),
                                                     stream=stream.cuda_stream))
    out["normal_estimation"] = {"points": n, "k": 10, "ms": ms, "points_per_s": n / (ms * 1e-3)}
    with psr.PoissonReconstruction(weld_vertices=True, **caps) as rw:
        def weld_step():
            rw.reconstruct_device(d_xyz.data_ptr(), d_nrm.data_ptr(),
                                  d_rgb.data_ptr() if d_rgb is not None else None, n, depth=depth,
                                  stream=stream.cuda_stream, out=dev_mesh())
        ms = median_ms(weld_step)
        out["weld"] = {"plain_ms": ms, "vertices_before": st.mesh_vertices,
                       "vertices_after": rw.stats().mesh_vertices}
    return out


def open_loop_leg(server, clouds, n_req, rate, seed=7):
    """Open-loop serving: n_req requests (cycling over the staged clouds) arriving as a
    Poisson process at `rate` per second; latency = arrival to completion (queueing
    included)."""
    from serve import Request
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    K = len(clouds)
    reqs = [Request(xyz=clouds[i % K][0], normals=clouds[i % K][1], rgb=clouds[i % K][2], depth=clouds[i % K][3])
            for i in range(n_req)]
    done = server.run(reqs, arrivals=list(arrivals))
    errs = [r.error for r in done if r.error]
    if errs:
        raise RuntimeError(f"open-loop leg: {errs[0]}")
    return np.array([r.latency_ms for r in done])


def served_leg(server, clouds, steps, torch, dev):
    """Continuous serving through the Server (psr_submit / psr_poll from one host thread):
    steps x K requests cycling over the K staged clouds, all arriving at once.  Device
    time = CUDA events from a common start (every slot stream waits on it) to the last
    slot's final completion; per-request latency = host time from arrival to completion."""
    from serve import Request, latency_summary
    K = len(server.slots)
    reqs = [Request(xyz=c[0], normals=c[1], rgb=c[2], depth=c[3]) for _ in range(steps) for c in clouds[:K]]
    torch.cuda.synchronize(dev)
    start = torch.cuda.Event(enable_timing=True)
    start.record(torch.cuda.default_stream(dev))
    for sl in server.slots:
        sl.stream.wait_event(start)
    done = server.run(reqs)
    ends = []
    for sl in server.slots:
        e = torch.cuda.Event(enable_timing=True)
        e.record(sl.stream)
        ends.append(e)
    torch.cuda.synchronize(dev)
    errs = [r.error for r in done if r.error]
    if errs:
        raise RuntimeError(f"served leg: {errs[0]}")
    total_ms = max(start.elapsed_time(e) for e in ends)
    lat = np.array([1000.0 * (r.finished - r.admitted) for r in done])   # service time (no queueing)
    stages = np.mean([list(sl.recon.stats().stage_ms) for sl in server.slots], axis=0)
    return total_ms, lat, [round(float(x), 4) for x in stages]


def batch_leg(psr, caps, clouds, steps, torch, dev, K):
    """Multi-cloud launches (psr_submit_batch): K clouds of the workload per pass, one launch
    of each kernel for all of them, device-resident inputs and outputs.  Device time = CUDA
    events around `steps` passes on the launching stream (3 untimed passes first)."""
    vcap, tcap = caps["max_mesh_vertices"], caps["max_triangles"]
    with psr.PoissonReconstruction(batch_clouds=K, concurrent_stages=False, **caps) as r:
        pts, meshes, outs = (psr.PsrPoints * K)(), (psr.PsrMesh * K)(), []
        for k in range(K):
            x, nrm, rgb, _ = clouds[k % len(clouds)]
            o = [torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((tcap, 3), dtype=torch.int32, device=dev),
                 torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((vcap, 3), dtype=torch.float32, device=dev)]
            outs.append(o)
            pts[k] = psr.PsrPoints(x.data_ptr(), nrm.data_ptr(), rgb.data_ptr() if rgb is not None else None,
                                   x.shape[0], psr.PSR_DEVICE)
            meshes[k] = psr.PsrMesh(o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr() if rgb is not None else None,
                                    o[3].data_ptr(), vcap, tcap, psr.PSR_DEVICE, 0, 0)
        stream = torch.cuda.current_stream(dev)
        for _ in range(3):
            r.submit_batch_device(pts, meshes, depth=clouds[0][3], stream=stream.cuda_stream)
            r.wait()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        a.record(stream)
        for _ in range(steps):
            r.submit_batch_device(pts, meshes, depth=clouds[0][3], stream=stream.cuda_stream)
            r.wait()
        b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b)
        st = [r.batch_result(k) for k in range(K)]
        if any(x[0] != psr.PSR_OK for x in st):
            raise RuntimeError("batch leg: a cloud failed")
        return {"clouds_per_launch": K, "value": K * steps / (ms / 1000.0), "unit": UNIT,
                "ms_per_pass": ms / steps, "kernel_launches_per_pass": int(st[0][1].kernel_launches),
                "stage_ms": [round(float(v), 4) for v in st[0][1].stage_ms],
                "memory_gb": round(r.memory_bytes() / 1e9, 2)}


def mix_batch_leg(psr, syn, torch, dev, n_clouds=256, per_pass=16):
    """The multi-cloud mix: 256 seeded clouds (point counts log-uniform in [5k, 150k];
    spheres, tori and superquadrics randomly scaled and rotated; no colour; depth drawn from
    6, 7, 8), grouped by depth into multi-cloud passes of up to `per_pass` clouds
    (psr_submit_batch: one launch of each kernel per pass), against the plain path (one
    handle, one psr_reconstruct per cloud) on the same clouds and capacities.  Inputs and
    outputs device-resident; each form timed over one whole pass of the 256 clouds after an
    untimed one (host clock, the device synchronised at both ends)."""
    clouds = []
    for i in range(n_clouds):
        p, nr, _, d = syn.workload("mix", cloud=i)
        clouds.append((torch.from_numpy(p).to(dev), torch.from_numpy(nr).to(dev), d))
    caps = dict(max_points=150000, max_depth=8, max_triangles=1500000, max_mesh_vertices=800000,
                max_subdivision_nodes=4000000, compute_colors=False, compute_normals=True)
    vcap, tcap = caps["max_mesh_vertices"], caps["max_triangles"]
    outs = [[torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((tcap, 3), dtype=torch.int32, device=dev),
             torch.empty((vcap, 3), dtype=torch.float32, device=dev)] for _ in range(per_pass)]
    def mesh_of(k):
        o = outs[k]
        return psr.PsrMesh(o[0].data_ptr(), o[1].data_ptr(), None, o[2].data_ptr(), vcap, tcap, psr.PSR_DEVICE, 0, 0)
    depths = sorted({c[2] for c in clouds})
    groups = [[c for c in clouds if c[2] == d] for d in depths]
    stream = torch.cuda.current_stream(dev)
    out = {"clouds": n_clouds, "clouds_per_depth": {str(d): len(g) for d, g in zip(depths, groups)},
           "clouds_per_pass": per_pass}
    with psr.PoissonReconstruction(batch_clouds=per_pass, concurrent_stages=False, **caps) as r:
        def run_all():
            ok = 0
            for g in groups:
                for s0 in range(0, len(g), per_pass):
                    part = g[s0:s0 + per_pass]
                    pts, meshes = (psr.PsrPoints * len(part))(), (psr.PsrMesh * len(part))()
                    for k, (x, nrm, _) in enumerate(part):
                        pts[k] = psr.PsrPoints(x.data_ptr(), nrm.data_ptr(), None, x.shape[0], psr.PSR_DEVICE)
                        meshes[k] = mesh_of(k)
                    r.submit_batch_device(pts, meshes, depth=part[0][2], stream=stream.cuda_stream)
                    try:
                        r.wait()
                    except psr.PsrError:
                        pass
                    for k in range(len(part)):
                        stk = r.batch_result(k)[0]
                        ok += stk == psr.PSR_OK
                        if stk != psr.PSR_OK:
                            name = psr.load_library().psr_status_string(stk).decode()
                            failed[name] = failed.get(name, 0) + 1
            return ok
        failed = {}
        run_all()   # graph capture of every (clouds, depth) shape
        torch.cuda.synchronize(dev)
        failed.clear()
        t = time.perf_counter()
        ok = run_all()
        torch.cuda.synchronize(dev)
        dt = time.perf_counter() - t
        out.update(batched={"recons_per_s": ok / dt, "completed": ok, "seconds": dt, "failed": failed,
                            "memory_gb": round(r.memory_bytes() / 1e9, 2)},
                   failed_note="clouds the reference's algorithm cannot mesh at their depth (it reads unset "
                               "vertex records: sparse clouds at depth 8) are rejected as invalid input by both "
                               "forms")
    with psr.PoissonReconstruction(**caps) as r:
        def one(c):
            try:
                r.reconstruct_device(c[0].data_ptr(), c[1].data_ptr(), None, c[0].shape[0], depth=c[2], out=mesh_of(0))
                return 1
            except psr.PsrError:
                return 0
        for g in groups:
            one(g[0])
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        ok = sum(one(c) for c in clouds)
        torch.cuda.synchronize(dev)
        dt = time.perf_counter() - t
        out["plain"] = {"recons_per_s": ok / dt, "completed": ok, "seconds": dt}
    out["batched_vs_plain"] = out["batched"]["recons_per_s"] / out["plain"]["recons_per_s"]
    return out


def large_leg(psr, syn, torch, dev, reps=3):
    """The precision-study cloud as a throughput case: 2,000,000 points on the superquadric
    (sinusoidal displacement, jittered normals), depth 9, every Laplacian entry kept, one
    cloud per call, inputs and outputs device-resident; median of `reps` timed calls after a
    warm one (CUDA events on the calling stream)."""
    p, nr, _, d = syn.workload("superquadric2m")
    caps = dict(max_depth=9, max_points=p.shape[0], max_triangles=12000000, max_mesh_vertices=6000000,
                max_subdivision_nodes=8000000, compute_colors=False, compute_normals=True, laplacian_epsilon=0.0)
    x, n = torch.from_numpy(p).to(dev), torch.from_numpy(nr).to(dev)
    vcap, tcap = caps["max_mesh_vertices"], caps["max_triangles"]
    o = [torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((tcap, 3), dtype=torch.int32, device=dev),
         torch.empty((vcap, 3), dtype=torch.float32, device=dev)]
    stream = torch.cuda.current_stream(dev)
    with psr.PoissonReconstruction(**caps) as r:
        def one():
            m = psr.PsrMesh(o[0].data_ptr(), o[1].data_ptr(), None, o[2].data_ptr(), vcap, tcap, psr.PSR_DEVICE, 0, 0)
            r.reconstruct_device(x.data_ptr(), n.data_ptr(), None, x.shape[0], depth=d, out=m, stream=stream.cuda_stream)
            return m
        one()
        times = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            m = one()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        st = r.stats()
        ms = float(np.median(times))
        return {"workload": "superquadric2m (N=2,000,000, depth 9, normals, laplacian_epsilon 0)", "ms": ms,
                "recons_per_s": 1000.0 / ms, "points_per_s": p.shape[0] / (ms / 1000.0),
                "stage_ms": [round(float(v), 3) for v in st.stage_ms],
                "cg_depth_ms": [round(float(v), 3) for v in st.cg_depth_ms[:d + 1]],
                "cg_iterations": list(st.cg_iterations[:d + 1]), "nodes": int(st.nodes),
                "mesh": {"vertices": int(m.vertex_count), "triangles": int(m.triangle_count)},
                "memory_gb": round(r.memory_bytes() / 1e9, 2)}


def serve_mix_leg(psr, serve, syn, torch, dev, seconds, rate=200.0, budget=40e9, pool=48, seed=11):
    """The serving loop: Poisson arrivals at `rate` per second of clouds of the serving mix
    (point counts log-uniform in [10k, 500k], depth uniform in 6..9, spheres, tori and
    superquadrics randomly scaled and rotated, colour), admitted by footprint into slots of
    two sizes under a device-memory budget; open loop for `seconds` after a 2 s warm-up.
    Requests cycle over a pool of distinct seeded clouds resident on the device.  Reported:
    completed reconstructions per second, arrival-to-completion p50 / p99, rejected
    requests, and the plain path (one handle, one cloud at a time) on the same pool."""
    from serve import Server, Request
    clouds = []
    for i in range(pool):
        p, nr, rgb, d = syn.workload("serve", cloud=i)
        clouds.append((torch.from_numpy(p).to(dev), torch.from_numpy(nr).to(dev), torch.from_numpy(rgb).to(dev), d))
    big = dict(max_points=500000, max_depth=9, max_triangles=8000000, max_mesh_vertices=4000000,
               max_subdivision_nodes=16000000)
    small = dict(max_points=120000, max_depth=9, max_triangles=4000000, max_mesh_vertices=2000000,
                 max_subdivision_nodes=8000000)
    server = Server(classes=[dict(count=2, **big), dict(count=64, **small)], memory_budget=budget,
                    compute_colors=True, compute_normals=True, laplacian_epsilon=0.0)
    slots = {"large": sum(1 for s in server.slots if s.max_points == big["max_points"]),
             "small": sum(1 for s in server.slots if s.max_points == small["max_points"])}
    def open_loop(rate_s, secs, warm, seed_):
        rng = np.random.default_rng(seed_)
        n_req = int(rate_s * (secs + warm))
        arrivals = np.cumsum(rng.exponential(1.0 / rate_s, n_req))
        reqs = [Request(xyz=clouds[i % pool][0], normals=clouds[i % pool][1], rgb=clouds[i % pool][2],
                        depth=clouds[i % pool][3]) for i in range(n_req)]
        done = server.run(reqs, arrivals=list(arrivals))
        t0 = min(r.arrival for r in done)
        meas = [r for r in done if r.arrival - t0 >= warm]
        ok = [r for r in meas if not r.error]
        lat = np.array([r.latency_ms for r in ok])
        span = max(r.finished for r in meas) - min(r.arrival for r in meas)
        errors = sorted({r.error.split(":")[0] for r in meas if r.error})
        return {"rate_per_s": round(rate_s, 2), "seconds": secs, "requests": len(meas), "completed": len(ok),
                "rejected": sum(1 for r in meas if r.error), "errors": errors[:3],
                "recons_per_s": len(ok) / span, "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99)) if lat.size else None}
    # as configured (200 requests/s): completions per second are the loop's capacity when
    # the arrivals exceed it, and latency is then mostly queueing; then an open loop at 70%
    # of that capacity for latency under a sustainable load
    out = open_loop(rate, seconds, 2.0, seed)
    out.update(slots=slots, memory_gb=round(server.memory_bytes / 1e9, 2), budget_gb=budget / 1e9,
               laplacian_epsilon=0.0)
    if out["recons_per_s"] < 0.95 * rate:
        out["sustainable"] = open_loop(0.7 * out["recons_per_s"], seconds, 2.0, seed + 1)
    server.close()
    # the plain path on the same pool: one handle sized for the largest cloud, one at a time
    with psr.PoissonReconstruction(compute_colors=True, compute_normals=True, laplacian_epsilon=0.0, **big) as r:
        vcap, tcap = big["max_mesh_vertices"], big["max_triangles"]
        o = [torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((tcap, 3), dtype=torch.int32, device=dev),
             torch.empty((vcap, 3), dtype=torch.float32, device=dev), torch.empty((vcap, 3), dtype=torch.float32, device=dev)]
        def one(c):
            m = psr.PsrMesh(o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), o[3].data_ptr(), vcap, tcap,
                            psr.PSR_DEVICE, 0, 0)
            try:
                r.reconstruct_device(c[0].data_ptr(), c[1].data_ptr(), c[2].data_ptr(), c[0].shape[0], depth=c[3],
                                     out=m)
                return True
            except psr.PsrError:
                return False
        for c in clouds[:4]:
            one(c)
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        good = sum(one(c) for c in clouds)
        torch.cuda.synchronize(dev)
        out["plain"] = {"recons_per_s": good / (time.perf_counter() - t), "clouds": pool, "completed": good}
    out["served_vs_plain"] = out["recons_per_s"] / out["plain"]["recons_per_s"]
    return out


def st_launches(r):
    try:
        return r.launch_count()
    except Exception:
        return -1


if __name__ == "__main__":
    main()
