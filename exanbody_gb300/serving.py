"""Continuous-batching request loop for LJ MD runs.

Requests (an FCC system size, state point, seed and step count) arrive as a
seeded Poisson process. The server keeps one batch resident on the GPU:
  * admission: an arrived request is admitted as soon as its device footprint
    (xnb_system_bytes, neighbour segment included) fits the HBM budget and a
    system slot is free; its state is built, uploaded and initialised (neighbour
    lists + forces) while the others wait at a chunk boundary;
  * batching: every chunk of steps advances all admitted systems together --
    their work shares the same kernels on the device;
  * retirement: a system that reached its step count is downloaded and
    removed, freeing its slot and memory for the queue.
Latency of a request = completion time - arrival time (host clock, seconds).

The baseline serves the same requests one at a time through the plain FP64
path (a fresh single-system batch per request, in arrival order).

  python -m exanbody_gb300.serving [--requests 10000] [--rate R] [--budget-gb 150] [--baseline-requests 1000]
"""
import argparse
import collections
import ctypes
import json
import time

import numpy as np

from . import replicas, workloads, xnb

BYTES_LIST_PER_ATOM = 160.0  # neighbour slot entries per atom for admission (rho <= 1, x1.25 margin)


def request_system(req):
    return workloads.lj_fcc_system(req["n"], req["rho"], req["T"], req["seed"])


def footprint(w):
    ncell = int(np.prod(w["geom"]["dims"]))
    return int(xnb.load().xnb_system_bytes(w["n_atoms"], ncell, BYTES_LIST_PER_ATOM))


class Server:
    """One resident batch serving requests by continuous batching.

    Each chunk of steps runs as a CUDA graph (xnb_step_graph_create), cached per
    chunk length and captured again only when an admission grew the batch's
    extent (xnb_graph_is_current). While the GPU runs a chunk, the host builds
    the initial states of the requests that arrive next, so that their upload
    and initialisation at the next chunk boundary do not wait for it."""

    def __init__(self, budget_bytes, max_systems=4096, precision=xnb.PREC_MIXED, chunk=50, stream=None,
                 use_graphs=True, lookahead_s=2.0, lookahead_max=64):
        import torch

        self.stream = stream or torch.cuda.Stream()
        per_atom = footprint(workloads.lj_fcc_system(5, 1.0, 1.0, 1)) / 500.0
        cap_atoms = int(budget_bytes / per_atom)
        self.batch = xnb.Batch(cap_atoms, cap_atoms // 8 + 4096, int(cap_atoms * BYTES_LIST_PER_ATOM),
                               max_systems=max_systems)
        self.batch.stream = ctypes.c_void_p(self.stream.cuda_stream)
        self.budget = budget_bytes
        self.used = 0
        self.peak_used = 0
        self.max_systems = max_systems
        self.precision = precision
        self.chunk = chunk
        self.use_graphs = use_graphs
        self.lookahead_s = lookahead_s
        self.lookahead_max = lookahead_max
        self.graphs = {}  # chunk length -> captured graph
        self.captures = 0
        self.chunks = 0

    def close(self):
        for g in self.graphs.values():
            g.close()
        self.graphs = {}
        self.batch.close()

    def _launch_chunk(self, nsteps):
        if not self.use_graphs:
            self.batch.step(nsteps, self.precision, 0)
            return
        g = self.graphs.get(nsteps)
        if g is None or not g.current():
            if g is not None:
                g.close()
            g = self.batch.graph(nsteps, self.precision, 0)
            self.graphs[nsteps] = g
            self.captures += 1
        g.launch()

    def serve(self, requests, prebuilt=None, time_limit=None, keep_results=False):
        """Serve requests in real time; returns (records, wall seconds, atom-steps).
        records[k]: arrival, admit, done, latency (done - arrival), wait (admit - arrival)."""
        order = sorted(range(len(requests)), key=lambda k: requests[k]["arrival"])
        pending = collections.deque(order)
        pending_set = set(order)
        ready = {}  # request -> initial state built on the host ahead of its admission
        upcoming = collections.deque(order)  # requests whose state is not built yet

        def system_of(k):
            if prebuilt is not None:
                return prebuilt[k]
            w = ready.pop(k, None)
            return w if w is not None else request_system(requests[k])

        def prepare(now):
            # host work overlapped with the running chunk: the states of the next arrivals
            if prebuilt is not None:
                return
            while upcoming and len(ready) < self.lookahead_max:
                k = upcoming[0]
                if requests[k]["arrival"] > now + self.lookahead_s:
                    break
                upcoming.popleft()
                if k in pending_set and k not in ready:
                    ready[k] = request_system(requests[k])

        active = {}  # sys id -> [req index, remaining steps, bytes, atoms]
        records = {}
        t0 = time.perf_counter()
        atom_steps = 0
        while pending or active:
            now = time.perf_counter() - t0
            if time_limit and now > time_limit:
                break
            admitted = []
            while pending and requests[pending[0]]["arrival"] <= now and len(active) < self.max_systems:
                k = pending[0]
                w = system_of(k)
                fb = footprint(w)
                if self.used + fb > self.budget:
                    if prebuilt is None:
                        ready[k] = w
                    break
                pending.popleft()
                pending_set.discard(k)
                try:
                    s = self.batch.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=1.25)
                except xnb.XnbError:
                    pending.appendleft(k)  # pool fragmentation: retry after a retirement
                    pending_set.add(k)
                    if prebuilt is None:
                        ready[k] = w
                    break
                self.used += fb
                self.peak_used = max(self.peak_used, self.used)
                active[s] = [k, requests[k]["steps"], fb, w["n_atoms"]]
                t_admit = time.perf_counter() - t0
                records[k] = {"arrival": requests[k]["arrival"], "admit": t_admit,
                              "wait": t_admit - requests[k]["arrival"]}
                admitted.append(s)
            for s in admitted:
                self.batch.init_particles(s, self.precision)
            if not active:
                prepare(time.perf_counter() - t0)
                if pending:
                    wait = requests[pending[0]]["arrival"] - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                continue
            nsteps = min(self.chunk, min(v[1] for v in active.values()))
            self._launch_chunk(nsteps)  # asynchronous on self.stream
            self.chunks += 1
            prepare(time.perf_counter() - t0)
            self.stream.synchronize()
            atom_steps += nsteps * sum(v[3] for v in active.values())
            finished = [s for s, v in active.items() if v[1] - nsteps <= 0]
            for s in active:
                active[s][1] -= nsteps
            if finished:
                self.batch.check_errors()
            for s in finished:
                k, _, fb, _ = active.pop(s)
                result = self.batch.download(s)  # the request's result leaves the device
                if keep_results:
                    records[k]["result"] = result
                self.batch.remove_system(s)
                self.used -= fb
                t = time.perf_counter() - t0
                records[k].update(done=t, latency=t - requests[k]["arrival"])
        wall = time.perf_counter() - t0
        return records, wall, atom_steps


def serve_sequential(requests, prebuilt=None, precision=xnb.PREC_FP64, time_limit=None):
    """Same requests, one at a time in arrival order, one system per batch."""
    import torch

    stream = torch.cuda.Stream()
    records = {}
    t0 = time.perf_counter()
    atom_steps = 0
    for k in sorted(range(len(requests)), key=lambda q: requests[q]["arrival"]):
        req = requests[k]
        now = time.perf_counter() - t0
        if time_limit and now > time_limit:
            break
        if req["arrival"] > now:
            time.sleep(req["arrival"] - now)
        w = prebuilt[k] if prebuilt else request_system(req)
        ncell = int(np.prod(w["geom"]["dims"]))
        b = xnb.Batch(w["n_atoms"] + 64, ncell + 64, int(w["n_atoms"] * BYTES_LIST_PER_ATOM) + 4096)
        b.stream = ctypes.c_void_p(stream.cuda_stream)
        s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=1.25)
        b.init_particles(s, precision)
        b.step(req["steps"], precision, 0)
        _ = b.download(s)
        b.check_errors()
        b.close()
        atom_steps += w["n_atoms"] * req["steps"]
        t = time.perf_counter() - t0
        records[k] = {"done": t, "latency": t - req["arrival"]}
    return records, time.perf_counter() - t0, atom_steps


def summarize(records, wall, atom_steps, device=None):
    """Completion-latency percentiles and throughput (and the admission waits
    where recorded); under torchrun the values of all ranks are gathered and the
    wall time is the slowest rank's."""
    lat = np.array([r["latency"] for r in records.values() if "latency" in r])
    lat = replicas.gather_values(lat, device=device)
    wall = replicas.max_over_ranks(wall, device=device)
    atom_steps = replicas.gather_values([atom_steps], device=device).sum()
    out = {"completed": int(len(lat)), "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
           "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
           "mean_s": float(lat.mean()) if len(lat) else None, "max_s": float(lat.max()) if len(lat) else None,
           "wall_s": wall, "atom_steps_per_s": float(atom_steps) / wall}
    waits = np.array([r["wait"] for r in records.values() if "wait" in r])
    if len(waits):
        waits = replicas.gather_values(waits, device=device)
        out["admission_wait_s"] = {"p50": float(np.percentile(waits, 50)), "p90": float(np.percentile(waits, 90)),
                                   "p99": float(np.percentile(waits, 99)), "max": float(waits.max()),
                                   "mean": float(waits.mean()), "zero_fraction": float(np.mean(waits < 1e-3))}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=10000)
    ap.add_argument("--rate", type=float, default=0.0, help="arrivals per second (0: 0.8 x measured capacity)")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--seed", type=int, default=4242)
    ap.add_argument("--baseline-requests", type=int, default=1000,
                    help="the sequential FP64 baseline serves this prefix of the stream (0: none)")
    ap.add_argument("--no-graphs", action="store_true", help="eager xnb_step chunks instead of captured graphs")
    ap.add_argument("--out", default="", help="also write the JSON result to this file")
    args = ap.parse_args()
    import torch

    rank, world, local = replicas.dist_env()
    dev = None
    if world > 1:
        # replicas: each GPU serves every world-th request of the one stream
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        torch.cuda.set_device(local)
        dev = torch.device("cuda", local)
    torch.cuda.init()
    reqs = replicas.shard(workloads.serving_stream(args.requests, seed=args.seed, rate=1.0), rank, world)
    # FCC n^3 holds 4 n^3 atoms: the work is known without building the systems
    work = sum(4 * r["n"] ** 3 * r["steps"] for r in reqs)
    rate = args.rate
    capacity = None
    if rate <= 0:
        # capacity: a batch of the first requests, all admitted at once
        probe = [dict(r, arrival=0.0) for r in reqs[: min(64, len(reqs))]]
        srv = Server(args.budget_gb * 1e9, precision=xnb.PREC_MIXED, chunk=args.chunk)
        rec, wall, ast = srv.serve(probe, [request_system(r) for r in probe])
        srv.close()
        mean_work = work / len(reqs)
        capacity = ast / wall / mean_work  # requests per second of one GPU
        # the whole stream arrives at 0.8 x the capacity of all GPUs (the slowest one's x world)
        capacity = -replicas.max_over_ranks(-capacity, device=dev) * world
        rate = 0.8 * capacity
    # rescale the unit-rate arrival times of the seeded stream to the chosen rate
    for r in reqs:
        r["arrival"] = r["arrival"] / rate
    srv = Server(args.budget_gb * 1e9, precision=xnb.PREC_MIXED, chunk=args.chunk, use_graphs=not args.no_graphs)
    rec_b, wall, ast = srv.serve(reqs)
    batched = summarize(rec_b, wall, ast, dev)
    batched.update(peak_admitted_gb=srv.peak_used / 1e9, chunks=srv.chunks, graph_captures=srv.captures,
                   chunk_runs="eager xnb_step" if args.no_graphs else "captured CUDA graphs")
    srv.close()
    out = {"workload": "serving_%d_requests_fcc_n5-40_steps200-2000" % args.requests,
           "arrival_rate_per_s": rate, "capacity_req_per_s": capacity, "budget_gb": args.budget_gb,
           "chunk_steps": args.chunk, "total_atom_steps": int(replicas.gather_values([work], device=dev).sum()),
           "gpus": world, "batched_mixed": batched}
    nb = min(args.baseline_requests, len(reqs))
    if nb > 0:
        # the plain FP64 path at its faster traversal (Newton half lists) on one
        # system at a time, over the first nb requests of the same stream
        first = sorted(range(len(reqs)), key=lambda k: reqs[k]["arrival"])[:nb]
        sub = [reqs[k] for k in first]
        rec, wall, ast = serve_sequential(sub, precision=xnb.PREC_FP64 | xnb.PREC_NEWTON)
        out["sequential_fp64"] = dict(summarize(rec, wall, ast, dev), traversal="newton",
                                      requests="the first %d of the stream, same arrival times" % nb)
        # the batched loop's latencies over the same requests, for a like-for-like comparison
        pre = [rec_b[k]["latency"] for k in first if "latency" in rec_b.get(k, {})]
        if pre:
            out["batched_mixed_same_prefix"] = {"completed": len(pre), "p50_s": float(np.percentile(pre, 50)),
                                                "p99_s": float(np.percentile(pre, 99)), "mean_s": float(np.mean(pre))}
    if rank == 0:
        line = json.dumps(out)
        print(line)
        if args.out:
            with open(args.out, "w") as f:
                f.write(line + "\n")


if __name__ == "__main__":
    main()
