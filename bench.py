"""Benchmark of the LJ molecular-dynamics hot path on one GB300 (atom-steps/s).

Workload (default): periodic FCC 100^3 = 4,000,000 atoms, rho* = 0.8442,
T* = 1.44, truncated-and-shifted LJ rc = 2.5, skin 0.3, dt = 0.005; one bench
"step" is one velocity-Verlet MD step (push, trigger, conditional rebin +
neighbour rebuild, forces, push) of the whole system, in the mixed precision
path. Each precision is timed with both force traversals (full lists, bitwise
reproducible; Newton half lists with FP64 reductions) and reported at its
faster one. The state (~2.4 GB) is larger than L2 (129 MB), so no flush is needed.

Reported on one JSON line: mixed-path atom-steps/s with inputs resident in
HBM (`value`: the K timed steps run as one captured CUDA graph, the step loop of
the serving and ensemble drivers), the plain FP64 path beside it (timed the same
way), the force error of the mixed
path against FP64, an end-to-end run through the C ABI with host buffers
(`e2e`), the roofline of the dominant (force) kernel, and the CPU oracle
(restated reference OpenMP path) on the same workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N > 1) each rank advances its own replica (the systems are
independent; no collective on the data path): scaling is weak.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic work per atom-step of the LJ force kernel at rho* = 0.8442, rc = 2.5,
# skin 0.3 (77.63 list / 55.25 in-cutoff neighbours per atom, each pair counted
# once): FP64 path 0.5*(8*77.63 + 13*55.25) = 669.6 flop; mixed path
# 0.5*(3*77.63 + 6*55.25) = 282.2 FP64 flop + 0.5*(5*77.63 + 7*55.25) = 387.4 FP32 flop.
FLOP64_PER_ATOM_FP64_PATH = 669.6
FLOP64_PER_ATOM_MIXED = 282.2
FLOP32_PER_ATOM_MIXED = 387.4
# DRAM bytes (read + write) per atom of one mixed k_force launch, from an ncu capture of
# the 256,000-atom case of this workload (FCC 40^3); traffic grows with the atom count at
# fixed density, so a launch moves this many bytes per atom.
FORCE_DRAM_BYTES_PER_ATOM = 520.0

WORKLOAD = dict(n=100, rho=0.8442, T=1.44, seed=12345, rcut=2.5, skin=0.3, dt=0.005)
METRIC = "atom-steps/s, 4M-atom LJ MD step (mixed precision; FP64 path and force error reported beside it)"


def hbm_peak_gbs():
    """Measured HBM copy bandwidth of this machine's GB300 (MEASURED_PEAKS.json), else 6800."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU-baseline record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        fields = dict(l.split(":", 1) for l in out.splitlines() if ":" in l)
        name = fields.get("Model name", "").strip()
        vendor = fields.get("Vendor ID", "").strip()
        if name:
            return (vendor + " " + name).strip()
    except (OSError, subprocess.SubprocessError, ValueError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.machine()


def config_of(n, atoms, **extra):
    c = {"workload": "lj_fcc_%d^3_rho0.8442_T1.44" % n, "atoms": atoms, "rcut": 2.5, "skin": 0.3, "dt": 0.005,
         "flush": "state %.1f GB > L2 (129 MB)" % (atoms * 600 / 1e9)}
    c.update(extra)
    return c


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=WORKLOAD["n"], help="FCC unit cells per side")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--force-block", type=int, default=0, help="threads per block of the force kernel (0: library default)")
    ap.add_argument("--stage-cap", type=int, default=0, help="neighbour-build staging candidates (0: library default)")
    ap.add_argument("--build-form", default="", choices=["", "rows", "warp", "half"],
                    help="neighbour-build kernel (empty: library default)")
    ap.add_argument("--force-lanes", type=int, default=0, choices=[0, 1, 2, 4],
                    help="threads per particle of the FP64 / mixed force traversal (0: library default)")
    ap.add_argument("--force-form", default="", choices=["", "thread", "staged"],
                    help="mixed full-list force traversal form (empty: library default)")
    ap.add_argument("--cell-factor", type=float, default=1.0,
                    help="cells of at least this many times rcut + skin (> 1: dense cells with AMR sub-grids)")
    ap.add_argument("--no-subcell-pruning", action="store_true",
                    help="build dense cells' lists without the sub-cell pair pruning")
    ap.add_argument("--workload", default="lj", choices=["lj", "snap_ni", "snap_mo"],
                    help="lj: the 4M-atom LJ headline; snap_*: the reference's SNAP benchmark decks")
    return ap.parse_args()


def dist_env():
    from exanbody_gb300 import replicas

    return replicas.dist_env()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": sorted(reasons)}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(n, cell_factor=1.0):
    from exanbody_gb300 import workloads

    return workloads.lj_fcc_system(n, WORKLOAD["rho"], WORKLOAD["T"], WORKLOAD["seed"], WORKLOAD["rcut"],
                                   WORKLOAD["skin"], cell_factor)


def cpu_oracle_run(w, steps, threads):
    """The oracle (CPU restatement of the reference's OpenMP path) on workload w."""
    from oracle.oracle import OracleSystem

    g = w["geom"]
    s = OracleSystem(g["origin"], g["extent"], g["dims"], g["cell_size"], WORKLOAD["rcut"], WORKLOAD["skin"], 1.0,
                     1.0, WORKLOAD["dt"], kind="omp")
    used = s.set_threads(threads)
    s.load_flat(w["r"], w["v"], w["id"])
    s.init()
    return s, used


def run_reference(args):
    """--impl reference: the restated reference CPU path on the same workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    w = make_workload(args.n, args.cell_factor)
    threads = os.cpu_count() or 1
    s, used = cpu_oracle_run(w, args.steps, threads)
    for _ in range(args.warmup):
        s.step()
    r0 = s.rebuilds
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.step()
    dt = time.perf_counter() - t0
    v = w["n_atoms"] * args.steps / dt
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": "atom-steps/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": config_of(args.n, w["n_atoms"], parallelism="single"),
        "cpu_baseline": {"value": v, "unit": "atom-steps/s", "cores": used, "cpu_model": cpu_model(), "kind": "port",
                         "sample": "%d MD steps of the %d-atom system (%d rebuilds), oracle/xnb_oracle.cpp OpenMP"
                                   % (args.steps, w["n_atoms"], s.rebuilds - r0)},
        "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def fp64_peak_tflops(torch, dev):
    """FP64 FMA throughput measured live with cuBLAS DGEMM (2*N^3 flop)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    best = 0.0
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, 2.0 * n ** 3 / (ms * 1e-3) / 1e12)
    del a, b
    return best


def run_ours(args):
    import ctypes

    import torch

    from exanbody_gb300 import xnb

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    w = make_workload(args.n, args.cell_factor)
    N = w["n_atoms"]
    g = w["geom"]
    ncell = g["dims"][0] * g["dims"][1] * g["dims"][2]
    params = xnb.lj_params(g, rcut=WORKLOAD["rcut"], rcut_inc=WORKLOAD["skin"], dt=WORKLOAD["dt"])

    def new_batch():
        b = xnb.Batch(N + 64, ncell + 64, int(N * 160) + 4096, max_systems=1, device=local,
                      stage_cap=args.stage_cap, force_block=args.force_block)
        b.stream = sp
        if args.build_form:
            b.set_build_form({"rows": xnb.BUILD_ROWS, "warp": xnb.BUILD_WARP, "half": xnb.BUILD_HALF}[args.build_form])
        if args.force_lanes:
            b.set_force_lanes(args.force_lanes)
        if args.force_form:
            b.set_force_form({"thread": xnb.FORCE_THREAD, "staged": xnb.FORCE_STAGED}[args.force_form])
        if args.no_subcell_pruning:
            b.set_subcell_pruning(False)
        return b

    def timed(fn, reps=1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        if world > 1:
            from exanbody_gb300 import replicas

            ms = replicas.max_over_ranks(ms, device=dev)  # the job's time is its slowest rank's
        return ms

    # Each precision is timed with both traversals (full lists: every pair from
    # both sides, bitwise reproducible; Newton half lists: each pair once with
    # FP64 reductions) and reported at its faster one.
    MIXED_FULL, MIXED_NEWTON = xnb.PREC_MIXED, xnb.PREC_MIXED | xnb.PREC_NEWTON
    FP64_FULL, FP64_NEWTON = xnb.PREC_FP64, xnb.PREC_FP64 | xnb.PREC_NEWTON

    b = new_batch()
    s = b.add_system(params, w["r"], w["v"], w["id"], list_factor=1.2)
    b.init_particles(s, MIXED_FULL)
    b.step(max(3, args.warmup), MIXED_FULL, 0)
    b.check_errors()
    k64 = max(5, min(args.steps, 40))
    trials = {}
    for name, prec in (("mixed_full", MIXED_FULL), ("mixed_newton", MIXED_NEWTON), ("fp64_full", FP64_FULL),
                       ("fp64_newton", FP64_NEWTON)):
        b.step(2, prec, 0)
        trials[name] = N * k64 / (timed(lambda: b.step(k64, prec, 0)) * 1e-3)
    b.check_errors()
    MIXED = MIXED_FULL if trials["mixed_full"] >= trials["mixed_newton"] else MIXED_NEWTON
    FP64 = FP64_FULL if trials["fp64_full"] >= trials["fp64_newton"] else FP64_NEWTON

    # ---- headline: the mixed path over the timed steps, as one captured CUDA
    # graph of K steps (xnb_step_graph_create / xnb_graph_launch, the step loop
    # of the serving and ensemble drivers); its kernel count is the captured one
    b.step(max(3, args.warmup), MIXED, 0)
    l0 = b.kernel_launches()
    g_mixed = b.graph(args.steps, MIXED, 0)
    launches = b.kernel_launches() - l0
    reb0 = b.info(s).rebuilds
    with Clocks(local) as ck:
        ms = timed(g_mixed.launch)
    clocks = ck.summary()
    b.check_errors()
    rebuilds = b.info(s).rebuilds - reb0
    g_mixed.close()
    value = world * N * args.steps / (ms * 1e-3)

    # ---- the same mixed steps through the persistent step loop (xnb_step_persistent:
    # one cooperative launch per run of steps between rebuilds; full lists only) ----
    persistent = None
    if not MIXED & xnb.PREC_NEWTON:
        b.step_persistent(2, MIXED)
        msp = timed(lambda: b.step_persistent(k64, MIXED))
        persistent = {"atom_steps_per_s": N * k64 / (msp * 1e-3), "ms_per_step": msp / k64, "steps": k64}
        b.check_errors()

    # ---- plain FP64 path at its faster traversal, from the same state, the same way ----
    b.step(2, FP64, 0)
    g64 = b.graph(k64, FP64, 0)
    ms64 = timed(g64.launch)
    g64.close()
    b.check_errors()
    value64 = N * k64 / (ms64 * 1e-3)

    # ---- force error of the mixed path against FP64 on one state ----
    b.lennard_jones_force(s, xnb.PREC_FP64, False)
    P = b.download(s)
    f64 = np.stack([P["fx"], P["fy"], P["fz"]], 1)
    b.lennard_jones_force(s, MIXED, False)
    P = b.download(s)
    fmx = np.stack([P["fx"], P["fy"], P["fz"]], 1)
    d = np.linalg.norm(fmx - f64, axis=1)
    mag = np.linalg.norm(f64, axis=1)
    frms = float(np.sqrt((mag ** 2).mean()))
    rel = d / np.maximum(mag, frms)
    err_max, err_rms = float(rel.max()), float(np.sqrt((rel ** 2).mean()))

    # ---- dominant kernel timing (force traversal alone, same launch as in the step) ----
    reps = 10
    ms_force = timed(lambda: b.lennard_jones_force(s, MIXED, False), reps) / reps
    ms_force64 = timed(lambda: b.lennard_jones_force(s, FP64, False), 3) / 3
    peak64 = fp64_peak_tflops(torch, dev)
    achieved = FLOP64_PER_ATOM_MIXED * N / (ms_force * 1e-3) / 1e12
    # ---- the rebuild path's parts, each call host-synchronised like the operator ----
    ms_nbr = timed(lambda: b.chunk_neighbors(s), 5) / 5
    ms_upd = timed(lambda: b.update_particles_full(s), 5) / 5
    b.check_errors()
    b.close()
    step_phases = {
        "force_only_mixed": {"ms": ms_force, "atom_steps_per_s": N / (ms_force * 1e-3)},
        "force_only_fp64": {"ms": ms_force64, "atom_steps_per_s": N / (ms_force64 * 1e-3),
                            "traversal": "newton" if FP64 & xnb.PREC_NEWTON else "full"},
        "neighbour_build_ms_per_rebuild": ms_nbr,
        "rebuild_path_ms_per_rebuild": ms_upd,
        "rebuilds_in_timed_steps": rebuilds,
        "persistent_loop_mixed": persistent,
        "note": "force-only: lennard_jones_force on the post-run state; neighbour build: xnb_chunk_neighbors "
                "(rebuild mark + one-pass list build); rebuild path: xnb_update_particles_full (rebin, backup, "
                "list build); CUDA events around each call",
    }

    # ---- end to end through the C ABI: host arrays in, K steps, host arrays out ----
    e2e = None
    if not args.no_e2e:
        # pinned host buffers, filled before the timed region: the inputs as columns
        # and the arrays the results are read back into
        def pinned(n, dtype):
            return torch.empty(n, dtype=dtype, pin_memory=True).numpy()

        cols = {}
        for ax, k in enumerate(("rx", "ry", "rz")):
            cols[k] = pinned(N, torch.float64)
            cols[k][:] = w["r"][:, ax]
        for ax, k in enumerate(("vx", "vy", "vz")):
            cols[k] = pinned(N, torch.float64)
            cols[k][:] = w["v"][:, ax]
        ids_in = pinned(N, torch.int64).view(np.uint64)
        ids_in[:] = w["id"]
        out = {k: pinned(N, torch.float64) for k in ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")}
        out["id"] = pinned(N, torch.int64).view(np.uint64)
        out["cell"] = pinned(N, torch.int32)
        phases = {}

        def e2e_run():
            bb = new_batch()
            t = time.perf_counter()
            ss = bb.add_system_soa(params, cols, ids_in, list_factor=1.2)
            torch.cuda.synchronize()
            phases["upload_s"] = time.perf_counter() - t
            t = time.perf_counter()
            bb.init_particles(ss, MIXED)
            torch.cuda.synchronize()
            phases["init_s"] = time.perf_counter() - t
            t = time.perf_counter()
            bb.step(args.steps, MIXED, 0)
            torch.cuda.synchronize()
            phases["steps_s"] = time.perf_counter() - t
            t = time.perf_counter()
            got = bb.download(ss, out)
            bb.check_errors()
            phases["download_s"] = time.perf_counter() - t
            bb.close()
            return got

        e2e_run()  # warm the allocator and the module
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_run()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        h2d = N * (6 * 8 + 8)
        d2h = N * (10 * 8 + 8 + 4)  # r, v, f, pe, id, cell into pinned buffers
        e2e = {"value": world * N * args.steps / dt, "unit": "atom-steps/s",
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "run": "pinned host arrays -> xnb_system_add -> xnb_init_particles -> %d x xnb_step -> "
                      "xnb_system_download"
                      % args.steps, "phases": phases}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline is an N=1 figure
        threads = os.cpu_count() or 1
        so, used = cpu_oracle_run(w, 0, threads)
        sample = 10
        r0 = so.rebuilds
        t0 = time.perf_counter()
        for _ in range(sample):
            so.step()
        dt = time.perf_counter() - t0
        reb = so.rebuilds - r0
        t0 = time.perf_counter()
        so.compute_forces()
        dt_force = time.perf_counter() - t0
        t0 = time.perf_counter()
        so.chunk_neighbors()
        dt_nbr = time.perf_counter() - t0
        cpu = {"value": N * sample / dt, "unit": "atom-steps/s", "cores": used, "cpu_model": cpu_model(), "kind": "port",
               "sample": "%d MD steps of the same %d-atom system after init (%d rebuilds), oracle OpenMP build"
                         % (sample, N, reb),
               "phases": {"force_only_atom_steps_per_s": N / dt_force, "neighbour_build_ms_per_rebuild": dt_nbr * 1e3,
                          "rebuilds_in_sample": reb}}
        del so

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "atom-steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64+f32",
            "data": "synthetic",
            "config": config_of(args.n, N, parallelism="replicas" if world > 1 else "single",
                                precision="mixed", rebuilds_in_timed_steps=rebuilds,
                                **({"cell_size": g["cell_size"], "atoms_per_cell": N / ncell,
                                    "subcell_pruning": not args.no_subcell_pruning}
                                   if args.cell_factor != 1.0 else {})),
            "fp64": {"value": value64, "unit": "atom-steps/s", "steps": k64,
                     "speedup_mixed_vs_fp64": value / world / value64},
            "traversals": dict(trials, unit="atom-steps/s", steps=k64,
                               chosen={"mixed": "newton" if MIXED & xnb.PREC_NEWTON else "full",
                                       "fp64": "newton" if FP64 & xnb.PREC_NEWTON else "full"}),
            "force_error_mixed_vs_fp64": {"max": err_max, "rms": err_rms, "tolerance": 1e-5},
            "phases": step_phases,
            "clocks": clocks,
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {"bound": "fp64",
                         "kernel": ("k_force_half<mixed> (+ zero/finish launches)" if MIXED & xnb.PREC_NEWTON
                                    else "k_force<mixed>"),
                         "achieved": achieved, "peak": peak64,
                         "unit": "TFLOP/s", "frac": achieved / peak64,
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                         "ms_per_launch": ms_force, "ms_per_launch_fp64_kernel": ms_force64,
                         "traffic": FORCE_DRAM_BYTES_PER_ATOM * N,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per atom on the "
                                           "256,000-atom case, scaled to %d atoms" % N,
                         "hbm": {"achieved_gbs": FORCE_DRAM_BYTES_PER_ATOM * N / (ms_force * 1e-3) / 1e9,
                                 "peak_gbs": hbm_peak_gbs(),
                                 "frac": FORCE_DRAM_BYTES_PER_ATOM * N / (ms_force * 1e-3) / 1e9 / hbm_peak_gbs()}},
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# SNAP workloads: the systems of the reference's benchmark_lj_snap SNAP decks
# (input_snap_{Ni,Mo}.msp: FCC Ni 16^3 / BCC Mo 16^3 with Gaussian noise, 4^3
# cells, rcut_inc 2 A, dt 2 fs, mass division), started at rest, one bench step =
# one velocity-Verlet step with snap_force_generic.
SNAP_DECKS = {
    "snap_ni": dict(el="Ni", structure="FCC", n=16, a=3.48, sigma=0.05, mass=58.693, cells=4),
    "snap_mo": dict(el="Mo", structure="BCC", n=16, a=3.15, sigma=0.1, mass=95.96, cells=4),
}


def snap_setup(name):
    from exanbody_gb300 import snap

    d = SNAP_DECKS[name]
    g = os.path.join(ROOT, "tests", "golden", "snap")
    cfg = snap.read_lammps(os.path.join(g, "%s_Zuo_JPCA2020.snapparam" % d["el"]),
                           os.path.join(g, "%s_Zuo_JPCA2020.snapcoeff" % d["el"]))
    r = snap.lattice(d["structure"], d["n"], d["a"], d["sigma"], 2024)
    L = d["n"] * d["a"]
    geom = {"origin": (0.0, 0.0, 0.0), "extent": (L, L, L), "dims": (d["cells"],) * 3, "cell_size": L / d["cells"]}
    return d, cfg, r, geom


def snap_flop64_per_atom(cfg, nn):
    """FP64 flop (FMA = 2) of one atom's SNAP force in this implementation's
    formulation: per neighbour and unique U element, 20 (U recursion) + 4 (its
    weighted sum into U_tot) + 4 (F) + 16 (dF/da, dF/db) + 20 (adjoint gather);
    per Z element 10 per Clebsch-Gordan product term, 4 per row and 4 for its Y
    contribution."""
    J = int(cfg["twojmax"])
    nu = sum(((j + 1) // 2) * (j + 1) if j % 2 else (j // 2) * (j + 1) + j // 2 + 1 for j in range(J + 1))
    z = 0
    for j1 in range(J + 1):
        for j2 in range(j1 + 1):
            for j in range(j1 - j2, min(J, j1 + j2) + 1, 2):
                for mb in range(j // 2 + 1):
                    for ma in range(j + 1):
                        if 2 * mb == j and ma > mb:
                            continue
                        ma1 = max(0, (2 * ma - j - j2 + j1) // 2)
                        na = min(j1, (2 * ma - j + j2 + j1) // 2) - ma1 + 1
                        mb1 = max(0, (2 * mb - j - j2 + j1) // 2)
                        nb = min(j1, (2 * mb - j + j2 + j1) // 2) - mb1 + 1
                        z += nb * (10 * na + 4) + 4
    return nn * nu * (20 + 4 + 4 + 16 + 20) + z


def run_snap(args):
    import torch

    from exanbody_gb300 import snap, xnb

    rank, world, local = dist_env()
    name = args.workload
    d, cfg, r, geom = snap_setup(name)
    N = len(r)
    L = geom["extent"][0]
    nbh = cfg["rcutfac"] + 2.0
    params = xnb.lj_params(geom, rcut=cfg["rcutfac"], rcut_inc=2.0, dt=2e-3, mass=d["mass"], divide_by_mass=True)
    ids = np.arange(1, N + 1, dtype=np.uint64)
    v0 = np.zeros_like(r)
    metric = "atom-steps/s, SNAP MD step (%s %s %d^3, %d atoms, twojmax %d, FP64)" % (
        d["structure"], d["el"], d["n"], N, cfg["twojmax"])
    conf = {"workload": "%s_%s%d^3_snap_twojmax%d" % (name, d["structure"], d["n"], cfg["twojmax"]), "atoms": N,
            "rcut": cfg["rcutfac"], "skin": 2.0, "dt_ps": 2e-3, "deck": "input_%s.msp" % name.replace("snap_", "snap_"),
            "flush": "none: the SNAP kernel is FP64-bound; its state (%.1f MB) stays in L2" % (N * 900 / 1e6)}
    if args.impl == "reference":
        if rank != 0:
            return 0
        from oracle.oracle import OracleSystem

        s = OracleSystem((0, 0, 0), (L, L, L), geom["dims"], geom["cell_size"], cfg["rcutfac"], 2.0, 1.0, 1.0, 2e-3,
                         mass=d["mass"], divide_by_mass=True, kind="omp")
        used = s.set_threads(os.cpu_count() or 1)
        s.set_snap(cfg, snap.energy_unit())
        s.load_flat(r, v0, ids)
        s.init()
        for _ in range(args.warmup):
            s.step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.step()
        dt = time.perf_counter() - t0
        v = N * args.steps / dt
        print(json.dumps({"impl": "reference", "metric": metric, "value": v, "unit": "atom-steps/s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": conf,
                          "cpu_baseline": {"value": v, "unit": "atom-steps/s", "cores": used, "cpu_model": cpu_model(), "kind": "port",
                                           "sample": "%d SNAP MD steps, oracle/xnb_snap_oracle.h OpenMP" % args.steps},
                          "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    b = xnb.Batch(N + 64, geom["dims"][0] ** 3 + 64, N * 200 + 4096, max_systems=1, device=local)
    s = b.add_system(params, r, v0, ids)
    b.init_particles(s, xnb.PREC_FP64)
    pot = snap.Potential(cfg, device=local)
    pot.force(b, s)
    snap.md_steps(b, s, pot, max(3, args.warmup))
    steps = args.steps

    def timed_steps(mixed):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        snap.md_steps(b, s, pot, steps, mixed=mixed)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    def timed_force(mixed, reps=5):
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record()
        for _ in range(reps):
            pot.force(b, s, mixed=mixed)
        f1.record()
        f1.synchronize()
        return f0.elapsed_time(f1) / reps

    # headline: the mixed path (FP32 U/Z/Y/adjoint arithmetic, FP64 geometry and sums)
    snap.md_steps(b, s, pot, 2, mixed=True)
    reb0 = b.info(s).rebuilds
    l0 = b.kernel_launches()
    with Clocks(local) as ck:
        ms = timed_steps(True)
    launches = b.kernel_launches() - l0
    rebuilds = b.info(s).rebuilds - reb0
    ms64 = timed_steps(False)
    ms_force = timed_force(True)
    ms_force64 = timed_force(False)
    # force error of the mixed path against FP64 on one state
    pot.force(b, s)
    P = b.download(s)
    f64 = np.stack([P["fx"], P["fy"], P["fz"]], 1)
    pot.force(b, s, mixed=True)
    P = b.download(s)
    fmx = np.stack([P["fx"], P["fy"], P["fz"]], 1)
    mag = np.linalg.norm(f64, axis=1)
    frms = float(np.sqrt((mag ** 2).mean()))
    rel = np.linalg.norm(fmx - f64, axis=1) / np.maximum(mag, frms)
    err_max, err_rms = float(rel.max()), float(np.sqrt((rel ** 2).mean()))
    # neighbours inside the SNAP cutoff (for the operation count)
    P = b.download(s)
    try:
        from scipy.spatial import cKDTree

        pts = np.stack([P["rx"], P["ry"], P["rz"]], 1) % L
        tree = cKDTree(pts, boxsize=L)
        nn = float(np.mean([len(x) - 1 for x in tree.query_ball_point(pts[:2000], cfg["rcutfac"])]))
    except ImportError:
        nn = 18.0 if d["structure"] == "FCC" else 14.0
    flop = snap_flop64_per_atom(cfg, nn)
    peak64 = fp64_peak_tflops(torch, dev)
    achieved = flop * N / (ms_force64 * 1e-3) / 1e12
    b.check_errors()
    b.close()
    e2e = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        bb = xnb.Batch(N + 64, geom["dims"][0] ** 3 + 64, N * 200 + 4096, max_systems=1, device=local)
        ss = bb.add_system(params, r, v0, ids)
        bb.init_particles(ss, xnb.PREC_FP64)
        pot.force(bb, ss, mixed=True)
        snap.md_steps(bb, ss, pot, steps, mixed=True)
        out = bb.download(ss)
        dt = time.perf_counter() - t0
        bb.close()
        e2e = {"value": N * steps / dt, "unit": "atom-steps/s", "h2d_bytes_per_step": N * 56 / steps,
               "d2h_bytes_per_step": N * 92 / steps,
               "run": "host arrays -> xnb_system_add -> init + xnb_snap_force -> %d SNAP MD steps -> download"
                      % steps}
        del out
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline is an N=1 figure
        from oracle.oracle import OracleSystem

        so = OracleSystem((0, 0, 0), (L, L, L), geom["dims"], geom["cell_size"], cfg["rcutfac"], 2.0, 1.0, 1.0,
                          2e-3, mass=d["mass"], divide_by_mass=True, kind="omp")
        used = so.set_threads(os.cpu_count() or 1)
        so.set_snap(cfg, snap.energy_unit())
        so.load_flat(r, v0, ids)
        so.init()
        sample = 3
        t0 = time.perf_counter()
        for _ in range(sample):
            so.step()
        dt = time.perf_counter() - t0
        cpu = {"value": N * sample / dt, "unit": "atom-steps/s", "cores": used, "cpu_model": cpu_model(), "kind": "port",
               "sample": "%d SNAP MD steps of the same system, oracle OpenMP build" % sample}
    if rank == 0:
        print(json.dumps({
            "metric": metric.replace("FP64)", "mixed precision; FP64 beside it)"),
            "value": world * N * steps / (ms * 1e-3), "unit": "atom-steps/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
            "config": dict(conf, rebuilds_in_timed_steps=rebuilds, neighbours_in_cutoff=nn, precision="mixed"),
            "fp64": {"value": N * steps / (ms64 * 1e-3), "unit": "atom-steps/s", "ms_per_step": ms64 / steps,
                     "speedup_mixed_vs_fp64": ms64 / ms},
            "force_error_mixed_vs_fp64": {"max": err_max, "rms": err_rms, "tolerance": 1e-5},
            "clocks": ck.summary(), "e2e": e2e, "gpu_launches": launches,
            "roofline": {"bound": "fp64", "kernel": "k_snap<double> (the FP64 path)", "achieved": achieved,
                         "peak": peak64, "unit": "TFLOP/s", "frac": achieved / peak64,
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                         "flop_per_atom": flop, "ms_per_launch": ms_force64, "ms_per_launch_mixed": ms_force,
                         "traffic": None},
            "cpu_baseline": cpu}), flush=True)
    return 0


def main():
    args = parse()
    if args.workload != "lj":
        return run_snap(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
