"""Batched ensemble, autotuner and the continuous-batching request loop."""
import numpy as np
import pytest

from exanbody_gb300 import ensemble, serving, workloads, xnb
from helpers import force_error, forces, ncells, new_batch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_autotuner_trials_and_choice():
    specs = workloads.ensemble_specs(12, seed=5, nmin=4, nmax=10)
    systems = ensemble.make_systems(specs)
    best, rate, log = ensemble.autotune(systems, xnb.PREC_MIXED, steps=20)
    assert rate > 0 and len(log) >= 4
    assert rate == max(t["rate"] for t in log if all(t[k] == best[k] for k in best))
    assert best["stage_cap"] in (384, 640, 1024) and best["force_block"] in (64, 128, 256)
    assert best["build_form"] in ("warp", "rows") and best["force_lanes"] in (1, 2, 4)


def test_serving_results_equal_alone_and_admission_by_budget():
    """Overlapping requests under a budget that cannot hold them all at once:
    every request completes, and each result matches the same request run alone
    (mixed precision, full lists: bitwise, so well inside the force tolerance)."""
    reqs = workloads.serving_stream(8, seed=11, nmin=4, nmax=9, steps=(40, 120), rate=200.0)
    built = [serving.request_system(r) for r in reqs]
    need = sorted(serving.footprint(w) for w in built)
    budget = need[-1] + need[-2] + need[-3]  # at most ~3 systems resident at a time
    srv = serving.Server(budget, max_systems=16, precision=xnb.PREC_MIXED, chunk=20)
    rec, wall, ast = srv.serve(reqs, built, keep_results=True)
    srv.close()
    assert len([r for r in rec.values() if "latency" in r]) == len(reqs)
    assert ast == sum(w["n_atoms"] * r["steps"] for w, r in zip(built, reqs))
    for k, (w, r) in enumerate(zip(built, reqs)):
        b = xnb.Batch(w["n_atoms"] + 64, int(np.prod(w["geom"]["dims"])) + 64, w["n_atoms"] * 170 + 4096)
        s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=1.25)
        b.init_particles(s, xnb.PREC_MIXED)
        b.step(r["steps"], xnb.PREC_MIXED, 0)
        alone = b.download(s)
        b.close()
        got = rec[k]["result"]
        assert np.array_equal(got["id"], alone["id"])
        e, _ = force_error(forces(got), forces(alone))
        assert e <= 1e-5
        assert np.max(np.abs(got["rx"] - alone["rx"])) <= 1e-9


def test_sequential_baseline_runs():
    reqs = workloads.serving_stream(3, seed=12, nmin=4, nmax=6, steps=(20, 40), rate=100.0)
    rec, wall, ast = serving.serve_sequential(reqs, precision=xnb.PREC_FP64)
    summ = serving.summarize(rec, wall, ast)
    assert summ["completed"] == 3 and summ["p99_s"] >= summ["p50_s"] > 0


def test_native_online_autotune():
    """xnb_autotune: times real steps per configuration, leaves the batch on the
    fastest one, and the batch keeps stepping normally afterwards."""
    specs = workloads.ensemble_specs(12, seed=9, nmin=5, nmax=9)
    systems = [workloads.lj_fcc_system(sp["n"], sp["rho"], sp["T"], sp["seed"]) for sp in specs]
    b = new_batch([w["n_atoms"] for w in systems], [ncells(w["geom"]) for w in systems])
    ids = [b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=1.25) for w in systems]
    b.init_particles(-1, xnb.PREC_MIXED)
    r0 = sum(b.info(s).rebuilds for s in ids)
    t = b.autotune(10, xnb.PREC_MIXED)
    assert t["stage_cap"] in (384, 640, 1024) and t["force_block"] in (64, 128, 256) and t["newton"] in (0, 1)
    assert t["trials"] >= 4 and t["atom_steps_per_s"] > 0
    assert sum(b.info(s).rebuilds for s in ids) > r0  # the trials were real steps
    prec = xnb.PREC_MIXED | (xnb.PREC_NEWTON if t["newton"] else 0)
    b.step(20, prec, 0)
    b.check_errors()
    with pytest.raises(xnb.XnbError):
        b.set_tuning(2048, 128)
