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

  python -m exanbody_gb300.serving [--requests 200] [--rate R] [--budget-gb 150]
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
    def __init__(self, budget_bytes, max_systems=4096, precision=xnb.PREC_MIXED, chunk=50, stream=None):
        import torch

        self.stream = stream or torch.cuda.Stream()
        per_atom = footprint(workloads.lj_fcc_system(5, 1.0, 1.0, 1)) / 500.0
        cap_atoms = int(budget_bytes / per_atom)
        self.batch = xnb.Batch(cap_atoms, cap_atoms // 8 + 4096, int(cap_atoms * BYTES_LIST_PER_ATOM),
                               max_systems=max_systems)
        self.batch.stream = ctypes.c_void_p(self.stream.cuda_stream)
        self.budget = budget_bytes
        self.used = 0
        self.max_systems = max_systems
        self.precision = precision
        self.chunk = chunk

    def close(self):
        self.batch.close()

    def serve(self, requests, prebuilt=None, time_limit=None, keep_results=False):
        """Serve requests in real time; returns per-request records."""
        pending = collections.deque(sorted(range(len(requests)), key=lambda k: requests[k]["arrival"]))
        active = {}  # sys id -> [req index, remaining steps, bytes]
        records = {}
        t0 = time.perf_counter()
        steps_done = 0
        atom_steps = 0
        while pending or active:
            now = time.perf_counter() - t0
            if time_limit and now > time_limit:
                break
            admitted = []
            while pending and requests[pending[0]]["arrival"] <= now and len(active) < self.max_systems:
                k = pending[0]
                w = prebuilt[k] if prebuilt else request_system(requests[k])
                fb = footprint(w)
                if self.used + fb > self.budget:
                    break
                pending.popleft()
                try:
                    s = self.batch.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=1.25)
                except xnb.XnbError:
                    pending.appendleft(k)  # pool fragmentation: retry after a retirement
                    break
                self.used += fb
                active[s] = [k, requests[k]["steps"], fb, w["n_atoms"]]
                records[k] = {"admit": time.perf_counter() - t0}
                admitted.append(s)
            for s in admitted:
                self.batch.init_particles(s, self.precision)
            if not active:
                if pending:
                    wait = requests[pending[0]]["arrival"] - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                continue
            nsteps = min(self.chunk, min(v[1] for v in active.values()))
            self.batch.step(nsteps, self.precision, 0)
            self.stream.synchronize()
            steps_done += nsteps
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
    """Completion-latency percentiles and throughput; under torchrun the latencies
    of all ranks are gathered and the wall time is the slowest rank's."""
    lat = np.array([r["latency"] for r in records.values() if "latency" in r])
    lat = replicas.gather_values(lat, device=device)
    wall = replicas.max_over_ranks(wall, device=device)
    atom_steps = replicas.gather_values([atom_steps], device=device).sum()
    return {"completed": int(len(lat)), "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_s": float(lat.mean()) if len(lat) else None, "wall_s": wall,
            "atom_steps_per_s": float(atom_steps) / wall}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=0.0, help="arrivals per second (0: 0.8 x measured capacity)")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--seed", type=int, default=4242)
    ap.add_argument("--no-baseline", action="store_true")
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
    prebuilt = [request_system(r) for r in reqs]
    work = sum(w["n_atoms"] * r["steps"] for w, r in zip(prebuilt, reqs))
    rate = args.rate
    capacity = None
    if rate <= 0:
        # capacity: a batch of the first requests, all admitted at once
        probe = [dict(r, arrival=0.0) for r in reqs[: min(64, len(reqs))]]
        srv = Server(args.budget_gb * 1e9, precision=xnb.PREC_MIXED, chunk=args.chunk)
        rec, wall, ast = srv.serve(probe, prebuilt[: len(probe)])
        srv.close()
        mean_work = work / len(reqs)
        capacity = ast / wall / mean_work  # requests per second of one GPU
        # the whole stream arrives at 0.8 x the capacity of all GPUs (the slowest one's x world)
        capacity = -replicas.max_over_ranks(-capacity, device=dev) * world
        rate = 0.8 * capacity
    # rescale the unit-rate arrival times of the seeded stream to the chosen rate
    for r in reqs:
        r["arrival"] = r["arrival"] / rate
    srv = Server(args.budget_gb * 1e9, precision=xnb.PREC_MIXED, chunk=args.chunk)
    rec, wall, ast = srv.serve(reqs, prebuilt)
    srv.close()
    out = {"workload": "serving_%d_requests_fcc_n5-40_steps200-2000" % args.requests,
           "arrival_rate_per_s": rate, "capacity_req_per_s": capacity, "budget_gb": args.budget_gb,
           "chunk_steps": args.chunk, "total_atom_steps": int(replicas.gather_values([work], device=dev).sum()),
           "gpus": world, "batched_mixed": summarize(rec, wall, ast, dev)}
    if not args.no_baseline:
        # the plain FP64 path at its faster traversal on one system at a time (Newton half lists)
        rec, wall, ast = serve_sequential(reqs, prebuilt, precision=xnb.PREC_FP64 | xnb.PREC_NEWTON)
        out["sequential_fp64"] = dict(summarize(rec, wall, ast, dev), traversal="newton")
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
