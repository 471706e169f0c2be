"""The autotuner's selection and sweep logic without a GPU: the runner that
advances a candidate is replaced by a fake whose timing and error are known,
so the choice -- the fastest adaptive candidate within the error bound, the
candidate order breaking ties, none when nothing qualifies -- can be checked
exactly.  (The reference fixes tile, monitor and threshold at compile time
and sweeps them by rewriting headers: snowflake/end2end_mix.py:13-75.)"""
import math

import numpy as np
import pytest

import w3914777_gb300 as w
from w3914777_gb300 import autotune as at


def row(name, seconds, err, mode=w.END2END_MIX):
    return {"name": name, "seconds": seconds, "err": err, "overrides": {"mode": mode}}


def test_select_best_fastest_within_bound():
    table = [row("a", 3.0, 1e-4), row("b", 1.0, 5e-3), row("c", 2.0, 9e-4), row("d", 2.5, 1e-3)]
    assert at.select_best(table, 1e-3)["name"] == "c"      # b is faster but outside the bound
    assert at.select_best(table, 1e-2)["name"] == "b"
    assert at.select_best(table, 1e-3 - 1e-12)["name"] == "c"
    assert at.select_best(table, 1e-5) is None              # nothing qualifies


def test_select_best_ties_failures_and_reference_points():
    table = [row("first", 2.0, 1e-4), row("second", 2.0, 1e-5),
             row("all fp32", 0.5, 1e-5, mode=w.PUREHIGH), row("all half", 0.1, 1e-5, mode=w.PURELOW),
             {"name": "failed", "error": "staging does not fit"}, row("nan", 0.2, float("nan"))]
    best = at.select_best(table, 1e-3)
    assert best["name"] == "first"                          # equal times: the earlier candidate
    assert at.select_best([table[2], table[3], table[4], table[5]], 1.0) is None


def _fake_runner(cost, err_of):
    """A runner whose time is cost(params) and whose final state is the initial
    state shifted by err_of(params) (zero for the plain FP64 reference)."""
    calls = []

    def run(p, init_state, steps, repeats=1):
        calls.append(p)
        e = 0.0 if (p.mode == w.PUREHIGH and p.high_tier == w.TIER_FP64) else err_of(p)
        return cost(p), init_state + e, {"tile_steps": [1, 2, 3]}
    return run, calls


def test_tune_sweeps_candidates_and_picks_the_fastest_passing_one():
    p = w.Params.preset("graingrowth", 0, nx=128, ny=128, nfields=4)
    cands = at.default_candidates(p)
    # time falls with the low threshold, error grows with it; 16^2 tiles slower
    cost = lambda q: (2.0 if q.tile == 16 else 1.0) / (1.0 + 1e3 * min(q.thr_lo, 1.0))  # noqa: E731
    err = lambda q: q.thr_lo * 0.1 if q.mode == w.END2END_MIX else 1.0  # noqa: E731
    run, calls = _fake_runner(cost, err)
    best, table = at.tune(p, w.INIT_SEEDED, 10, err_bound=2e-3, candidates=cands, runner=run)
    assert calls[0].mode == w.PUREHIGH and calls[0].high_tier == w.TIER_FP64   # the reference first
    assert len(table) == 1 + len(cands)
    assert best["err"] <= 2e-3
    passing = [r for r in table[1:] if r["err"] <= 2e-3 and r["overrides"]["mode"] == w.END2END_MIX]
    assert best["seconds"] == min(r["seconds"] for r in passing)
    assert best["overrides"]["tile"] == 32 and best["overrides"]["thr_lo"] == pytest.approx(2e-2)  # err 2e-3, at the bound
    # a bound nothing meets
    best, _ = at.tune(p, w.INIT_SEEDED, 10, err_bound=1e-9, candidates=cands, runner=run)
    assert best is None


def test_tune_records_candidates_the_library_refuses():
    p = w.Params.preset("graingrowth", 0, nx=128, ny=128, nfields=4)

    def run(q, init_state, steps, repeats=1):
        if q.tile == 16:
            raise w.AmpsError(6, "staging exceeds shared memory")
        return 1.0, init_state, {"tile_steps": [0, 1, 0]}
    cands = [c for c in at.default_candidates(p) if c[1].get("mode") == w.END2END_MIX][:4]
    cands.append(("t16", dict(cands[0][1], tile=16)))
    best, table = at.tune(p, w.INIT_SEEDED, 5, candidates=cands, runner=run)
    assert table[-1]["name"] == "t16" and "error" in table[-1]
    assert best is not None and best["overrides"]["tile"] == 32


def test_tune_ensemble_error_is_the_worst_member():
    members = [w.Params.preset("graingrowth", 0, nx=64, ny=64, nfields=4, seed=s) for s in (1, 2, 3)]

    def run(ps, states, steps, repeats=1):
        if ps[0].mode == w.PUREHIGH:
            return 4.0, [s.copy() for s in states], np.zeros(3)
        # member k is off by (k + 1) * thr_lo; tile 16 is slower
        t = (1.5 if ps[0].tile == 16 else 1.0) / (1.0 + ps[0].thr_lo * 1e4)
        return t, [st + (k + 1) * p.thr_lo for k, (p, st) in enumerate(zip(ps, states))], np.array([1.0, 3.0, 0.0])
    best, table = at.tune_ensemble(members, 10, err_bound=1e-4, runner=run)
    for r in table[1:]:
        assert r["err"] == pytest.approx(3 * r["overrides"]["thr_lo"])
    assert best["err"] <= 1e-4 and best["overrides"]["tile"] == 32
    assert best["overrides"]["thr_lo"] == pytest.approx(3e-5)
    assert best["mix"] == pytest.approx([0.25, 0.75, 0.0])


def test_ensemble_candidates_cover_both_tiles_and_only_temporal_monitors():
    c = at.ensemble_candidates()
    assert {ov["tile"] for _, ov in c} == {16, 32}
    assert {ov["monitor"] for _, ov in c} <= {w.MONITOR_RATE, w.MONITOR_TEM}
    assert all(ov["thr_lo"] <= ov["thr_hi"] for _, ov in c)
    assert all(math.isfinite(ov["thr_hi"]) for _, ov in c)
