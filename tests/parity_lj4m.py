"""Full-length parity run of the 4,000,000-atom configuration against the CPU oracle.

FCC 100^3 (rho* = 0.8442, T* = 1.44, rc 2.5, skin 0.3, dt 0.005), 1000 steps of
the FP64_EXACT path through the C ABI (host-synchronised schedule) beside the
oracle's OpenMP build. At init and after every rebuild the neighbour lists are
compared as ids in the reference's stream order, slice by slice; every step's
rebuild decision is compared; at the end positions, velocities, forces and
energies are compared bit for bit, and the FP64 / mixed traversals on the final
state against the oracle's forces and potential energy.

    python tests/parity_lj4m.py [--steps 1000] [--out results/parity_lj4m_1000_steps.json]
"""
import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from exanbody_gb300 import workloads, xnb  # noqa: E402
from helpers import compare_pairs_sliced, force_error, forces, ncells, new_batch, oracle_from  # noqa: E402

FIELDS = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "pe")


def bit_mismatches(G, O):
    out = {"id": int(np.count_nonzero(G["id"] != O["id"]))}
    for k in FIELDS:
        out[k] = int(np.count_nonzero(G[k].view(np.uint64) != O[k].view(np.uint64)))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--n", type=int, default=100)
    ap.add_argument("--out", default=os.path.join(ROOT, "results", "parity_lj4m_1000_steps.json"))
    args = ap.parse_args()

    w = workloads.lj_fcc_system(args.n, 0.8442, 1.44, 12345)
    t_start = time.time()
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    G = b.download(s)
    init_mis = bit_mismatches(G, o.particles())
    records = [{"step": 0, "entries": compare_pairs_sliced(b, s, o, G), "mismatches": 0}]
    decision_mismatch = []
    gpu_rebuilds = oracle_rebuilds = 0
    for step in range(1, args.steps + 1):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC | xnb.STEP_ENERGY)
        g_reb = b.info(s).rebuilds - r0
        o_reb = o.step()
        gpu_rebuilds += g_reb
        oracle_rebuilds += o_reb
        if g_reb != o_reb:
            decision_mismatch.append(step)
            break
        if o_reb:
            try:
                n = compare_pairs_sliced(b, s, o, b.download(s))
                records.append({"step": step, "entries": n, "mismatches": 0})
            except AssertionError as e:
                records.append({"step": step, "mismatches": str(e)})
                break
        if step % 100 == 0:
            print("step %d: %d rebuilds, %.0f s" % (step, gpu_rebuilds, time.time() - t_start), flush=True)
    G, O = b.download(s), o.particles()
    final_mis = bit_mismatches(G, O)
    ke_g, pe_g = b.energy(s)
    ke_o, pe_o = o.energy()
    ref = forces(O)
    on_final = {}
    for name, prec in (("fp64", xnb.PREC_FP64), ("fp64_newton", xnb.PREC_FP64 | xnb.PREC_NEWTON),
                       ("mixed", xnb.PREC_MIXED)):
        b.lennard_jones_force(s, prec, True)
        e_max, e_rms = force_error(forces(b.download(s)), ref)
        _, pe = b.energy(s)
        on_final[name] = {"force_error_max": e_max, "force_error_rms": e_rms,
                          "pe_relative_error": abs(pe - pe_o) / abs(pe_o)}
    list_failures = [r for r in records if r["mismatches"] != 0]
    out = {
        "workload": "lj_fcc_%d^3_rho0.8442_T1.44 (%d atoms), rc 2.5, skin 0.3, dt 0.005" % (args.n, w["n_atoms"]),
        "steps": step,
        "path": "XNB_PREC_FP64_EXACT, XNB_STEP_HOST_SYNC, through the C ABI; oracle OpenMP build (%d threads)"
                % (os.cpu_count() or 1),
        "host": platform.machine(),
        "rebuilds_gpu": gpu_rebuilds,
        "rebuilds_oracle": oracle_rebuilds,
        "rebuild_decision_mismatch_steps": decision_mismatch,
        "list_comparisons": len(records),
        "list_comparisons_failed": len(list_failures),
        "entries_compared_total": int(sum(r.get("entries", 0) for r in records)),
        "lists": records,
        "bitwise_mismatches_at_init": init_mis,
        "bitwise_mismatches_at_end": final_mis,
        "energy_gpu": [ke_g, pe_g],
        "energy_oracle": [ke_o, pe_o],
        "energy_bitwise_equal": bool(ke_g == ke_o and pe_g == pe_o),
        "traversals_on_final_state_vs_oracle": on_final,
        "tolerances": {"fp64": 1e-12, "mixed": 1e-5},
        "wall_s": time.time() - t_start,
    }
    ok = (not decision_mismatch and not list_failures and all(v == 0 for v in final_mis.values())
          and all(v == 0 for v in init_mis.values()) and out["energy_bitwise_equal"]
          and on_final["fp64"]["force_error_max"] <= 1e-12 and on_final["fp64_newton"]["force_error_max"] <= 1e-12
          and on_final["mixed"]["force_error_max"] <= 1e-5)
    out["pass"] = bool(ok)
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("steps", "rebuilds_gpu", "rebuilds_oracle", "list_comparisons",
                                          "list_comparisons_failed", "pass", "wall_s")}))
    b.close()
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
