"""Host logic of the ensemble autotuner (exanbody_gb300/ensemble.py: autotune):
a coordinate search over build form, stage, force block, threads per particle,
Newton lists and skin, one knob at a time in that order, each alternative tried
once against the best so far. The trials are replaced by a synthetic rate
landscape, so no GPU is needed."""
import pytest

from exanbody_gb300 import ensemble

KEYS = ("build_form", "stage_cap", "force_block", "force_lanes", "newton", "skin")


def landscape(best):
    """Separable rates with a known optimum; returns (rate function, calls list)."""
    calls = []

    def rate(cfg):
        r = 100.0
        for k in KEYS:
            r -= 0.0 if cfg[k] == best[k] else 7.0 + len(k)
        return r

    def fake_trial(systems, cfg, steps, precision, stream):
        calls.append(dict(cfg))
        return rate(cfg)

    return fake_trial, calls


@pytest.mark.parametrize("tune_skin", [False, True])
def test_coordinate_search_finds_separable_optimum(monkeypatch, tune_skin):
    target = dict(build_form="rows", stage_cap=1024, force_block=64, force_lanes=2, newton=True,
                  skin=0.4 if tune_skin else 0.3)
    fake, calls = landscape(target)
    monkeypatch.setattr(ensemble, "trial", fake)
    best, rate, log = ensemble.autotune([], steps=5, tune_skin=tune_skin, stream=object())
    assert best == target
    assert rate == 100.0
    # one trial for the defaults, then each alternative of each knob once
    alts = {"build_form": 1, "stage_cap": 2, "force_block": 2, "force_lanes": 2, "newton": 1,
            "skin": 2 if tune_skin else 0}
    assert len(calls) == 1 + sum(alts.values()) == len(log)
    assert calls[0] == ensemble.DEFAULTS
    # knobs are searched in order; a knob's trials keep the earlier knobs at their best
    order = [k for c, prev in zip(calls[1:], calls[:-1]) for k in KEYS if c[k] != prev[k]]
    firsts = [k for i, k in enumerate(order) if k not in order[:i]]
    assert firsts == [k for k in KEYS if alts[k]]
    for entry in log:
        assert entry["rate"] == pytest.approx(100.0 - sum(0.0 if entry[k] == target[k] else 7.0 + len(k)
                                                            for k in KEYS))
    assert not tune_skin or {c["skin"] for c in calls} == {0.3, 0.4, 0.5}
    assert tune_skin or {c["skin"] for c in calls} == {0.3}


def test_ties_keep_the_earlier_configuration(monkeypatch):
    """A candidate replaces the best only when strictly faster."""
    monkeypatch.setattr(ensemble, "trial", lambda systems, cfg, steps, precision, stream: 1.0)
    best, rate, log = ensemble.autotune([], steps=5, stream=object())
    assert best == ensemble.DEFAULTS and rate == 1.0
    assert len(log) == 1 + 1 + 2 + 2 + 2 + 1
