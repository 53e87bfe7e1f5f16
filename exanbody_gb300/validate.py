"""Accuracy runs of the mixed path against FP64: force error and NVE drift.

  python -m exanbody_gb300.validate drift [--n 100] [--steps 1000]
  python -m exanbody_gb300.validate slab  [--n 100] [--steps 1000]

Both start from the same seeded state in two batches (mixed, FP64), record the
total energy (kinetic + truncated-and-shifted LJ) every `--every` steps, and
report the relative drift (E_t - E_0)/|E_0| and the least-squares slope per
1000 steps, plus the max/RMS relative force error of the mixed forces against
FP64 forces evaluated on the same positions at the start and at the end.
"""
import argparse
import ctypes
import json

import numpy as np

from . import workloads, xnb


def force_err(fm, f64):
    """max/RMS of |dF_i| / max(|F_i|, F_rms); None when the reference forces
    vanish (F_rms < 1e-6, e.g. a perfect lattice where all forces cancel)."""
    d = np.linalg.norm(fm - f64, axis=1)
    mag = np.linalg.norm(f64, axis=1)
    frms = float(np.sqrt((mag ** 2).mean()))
    if frms < 1e-6:
        return None, None
    rel = d / np.maximum(mag, frms)
    return float(rel.max()), float(np.sqrt((rel ** 2).mean()))


def forces(P):
    return np.stack([P["fx"], P["fy"], P["fz"]], 1)


def run(w, steps, every, stream):
    g = w["geom"]
    N = w["n_atoms"]
    ncell = int(np.prod(g["dims"]))
    out = {}
    mixed_state = None
    for name, prec in (("mixed", xnb.PREC_MIXED), ("fp64", xnb.PREC_FP64)):
        b = xnb.Batch(N + 64, ncell + 64, int(N * 160) + 4096)
        b.stream = ctypes.c_void_p(stream.cuda_stream)
        s = b.add_system(xnb.lj_params(g), w["r"], w["v"], w["id"], list_factor=1.2)
        b.init_particles(s, prec)
        # force error at t = 0 (same positions)
        if name == "mixed":
            f_m = forces(b.download(s))
            b.lennard_jones_force(s, xnb.PREC_FP64, True)
            f64_0 = forces(b.download(s))
            e0max, e0rms = force_err(f_m, f64_0)
            frms0 = float(np.sqrt((np.linalg.norm(f64_0, axis=1) ** 2).mean()))
            b.lennard_jones_force(s, prec, True)
        ts, es = [], []
        ke, pe = b.energy(s)
        ts.append(0)
        es.append(ke + pe)
        done = 0
        while done < steps:
            k = min(every, steps - done)
            b.step(k, prec, xnb.STEP_ENERGY)
            done += k
            ke, pe = b.energy(s)
            ts.append(done)
            es.append(ke + pe)
        b.check_errors()
        es = np.array(es)
        rel = (es - es[0]) / abs(es[0])
        slope = float(np.polyfit(np.array(ts, float), rel, 1)[0] * 1000.0)
        out[name] = {"E0": float(es[0]), "E_end": float(es[-1]), "drift_rel": float(rel[-1]),
                     "drift_slope_per_1000_steps": slope, "max_abs_rel_dev": float(np.abs(rel).max()),
                     "rebuilds": int(b.info(s).rebuilds), "energy_every": every}
        if name == "mixed":
            P = b.download(s)
            f_m = forces(P)
            b.lennard_jones_force(s, xnb.PREC_FP64, False)
            e1max, e1rms = force_err(f_m, forces(b.download(s)))
            out["force_error_mixed_vs_fp64"] = {"t0": {"max": e0max, "rms": e0rms, "f_rms": frms0},
                                               "t_end": {"max": e1max, "rms": e1rms}, "tolerance": 1e-5}
        b.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["drift", "slab"])
    ap.add_argument("--n", type=int, default=100)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--every", type=int, default=50)
    args = ap.parse_args()
    import torch

    stream = torch.cuda.Stream()
    if args.what == "drift":
        w = workloads.lj_fcc_system(args.n, 0.8442, 1.44, 12345)
        name = "lj_fcc_%d^3_rho0.8442_T1.44" % args.n
    else:
        w = workloads.lj_slab_system(args.n, 0.8442, 0.8, 12345)
        name = "lj_slab_%d^3_rho0.8442_T0.8_box_LxLx2L" % args.n
    res = run(w, args.steps, args.every, stream)
    res.update(workload=name, atoms=w["n_atoms"], steps=args.steps, dims=list(w["geom"]["dims"]))
    print(json.dumps(res))


if __name__ == "__main__":
    main()
