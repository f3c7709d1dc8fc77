"""Launch-shape autotuner for the served forms.

A single call is latency-bound: its depth-D CG runs on the widest thread-block cluster the
device schedules (16 CTAs) and depths D-1, D-2 on 8-CTA clusters, which leaves most SMs to
the other stages.  When many reconstructions share the GPU (the resident slots of
serve.Server, or a multi-cloud pass), the SM time of each one is what bounds throughput,
and a CG cluster with fewer CTAs (more rows each) spends less SM time for a somewhat
longer solve.  The tuner measures the served throughput of a workload for each candidate
pair (psr_config.cg_cluster_ctas, cg_cluster_ctas_fine) and returns the best, with the
table of measurements.  Candidates whose rows do not fit the CG's shared-memory budget run
on its global-memory path and lose on their own.
"""
import time

CANDIDATES = ((16, 8), (16, 4), (12, 8), (12, 4), (10, 4))


def measure_served(server, requests_fn, torch, dev, rounds=3):
    """Recons/s of the server on the requests of requests_fn() (all queued at once), the
    best of `rounds` after one untimed round."""
    server.run(requests_fn())
    best = 0.0
    for _ in range(rounds):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        done = server.run(requests_fn())
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t
        if any(r.error for r in done):
            return None
        best = max(best, len(done) / el)
    return best


def tune_served(make_server, requests_fn, torch, dev, candidates=CANDIDATES):
    """make_server(cg_cluster_ctas=.., cg_cluster_ctas_fine=..) -> Server; returns
    (best (ctas, fine), {candidate: recons/s})."""
    table = {}
    for ctas, fine in candidates:
        srv = make_server(cg_cluster_ctas=ctas, cg_cluster_ctas_fine=fine)
        try:
            table[(ctas, fine)] = measure_served(srv, requests_fn, torch, dev)
        finally:
            srv.close()
    ok = {k: v for k, v in table.items() if v}
    best = max(ok, key=ok.get) if ok else candidates[0]
    return best, table
