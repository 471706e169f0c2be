"""Ensemble of grain-growth runs (amps_ensemble_*): a step's launches over
every member's tiles (one per group of members) must give each member exactly the results
amps_run gives it alone -- fields, tier maps, statistics -- for members of
different sizes, field counts, coefficients and time steps, in adaptive and
plain modes, over whole and partial cadence periods, with and without
graphs."""
import numpy as np
import pytest

from w3914777_gb300 import amps, ensemble

pytestmark = pytest.mark.gpu

MIXED = dict(mode=amps.END2END_MIX, monitor=amps.MONITOR_RATE, monitor_samples=1, monitor_field=-1)
_THR = {}


def mixed(monitor=amps.MONITOR_RATE):
    """MIXED (with the given monitor) with thresholds at the 40% / 75%
    quantiles of one probe member's tile metrics after a period, so that the
    members mix all three tiers."""
    if monitor not in _THR:
        p = small_members(dict(MIXED, monitor=monitor, thr_lo=0.0, thr_hi=0.0))[2]
        with amps.Simulation(p, init=amps.INIT_SEEDED) as s:
            s.run(10)
            m = s.metric().ravel()
        _THR[monitor] = (float(np.quantile(m, 0.4)), float(np.quantile(m, 0.75)))
    lo, hi = _THR[monitor]
    return dict(MIXED, monitor=monitor, thr_lo=lo, thr_hi=hi)


def small_members(extra=None):
    specs = [(64, 4, 2.0, 1.0), (96, 2, 1.3, 1.7), (128, 8, 2.7, 0.6), (64, 12, 1.1, 1.9), (32, 3, 2.2, 1.2)]
    out = []
    for i, (side, q, kap, mob) in enumerate(specs):
        p = amps.Params.preset(amps.GRAINGROWTH, 0, nx=side, ny=side, nfields=q, grcoef=kap, mobil=mob, tile=32,
                               seed=100 + i, init_amp=0.3)
        p.dt = ensemble.stable_dt(mob, kap)
        for k, v in (extra or {}).items():
            setattr(p, k, v)
        out.append(p)
    return out


def run_alone(params, steps):
    res = []
    for p in params:
        with amps.Simulation(p, init=amps.INIT_SEEDED) as s:
            s.run(steps)
            s.synchronize()
            res.append((s.fields(), s.tiers(), s.stats()))
    return res


def run_together(params, steps, graphs=True, chunks=None):
    sims = [amps.Simulation(p, init=amps.INIT_SEEDED) for p in params]
    with amps.Ensemble(sims, graphs=graphs) as ens:
        for c in (chunks or [steps]):
            ens.run(c)
        ens.synchronize()
    res = [(s.fields(), s.tiers(), s.stats()) for s in sims]
    for s in sims:
        s.close()
    return res


@pytest.mark.parametrize("graphs,monitor", [(True, amps.MONITOR_RATE), (False, amps.MONITOR_RATE),
                                            (True, amps.MONITOR_TEM)])
def test_ensemble_matches_individual_runs_adaptive(graphs, monitor):
    params = small_members(mixed(monitor))
    alone = run_alone(params, 37)
    together = run_together(params, 37, graphs=graphs, chunks=[20, 3, 14])
    for (fa, ta, sa), (fb, tb, sb) in zip(alone, together):
        assert np.array_equal(fa, fb)
        assert np.array_equal(ta, tb)
        assert sa == sb
    # the thresholds must actually mix tiers during the run for this to test
    # anything (the FP32 tile path is covered by the plain FP32 case)
    steps_per_tier = np.sum([st["tile_steps"] for _, _, st in alone], axis=0)
    assert np.count_nonzero(steps_per_tier) >= 2


@pytest.mark.parametrize("tier", [amps.TIER_FP32, amps.TIER_FP64])
def test_ensemble_matches_individual_runs_plain(tier):
    params = small_members(dict(mode=amps.PUREHIGH, high_tier=tier))
    alone = run_alone(params, 23)
    together = run_together(params, 23)
    for (fa, _, sa), (fb, _, sb) in zip(alone, together):
        # the all-FP64 single run uses the staged FP64 kernel, the ensemble the
        # fused kernel's FP64 tile path: same arithmetic, rounding may differ
        if tier == amps.TIER_FP64:
            assert np.abs(fa - fb).max() <= 1e-13
        else:
            assert np.array_equal(fa, fb)
        assert sa["steps"] == sb["steps"]


@pytest.mark.parametrize("monitor", [amps.MONITOR_RATE, amps.MONITOR_TEM])
def test_ensemble_ragged_members_match_individual_runs(monitor):
    """Members whose sides are not multiples of the tile (partial edge tiles,
    storage of whole tiles), mixed with whole-tile members, as the ensemble
    workload draws them: each member's fields, tiers and statistics equal its
    run alone."""
    specs = [(100, 4, 2.0, 1.0), (75, 3, 1.3, 1.7), (64, 8, 2.7, 0.6), (129, 2, 1.1, 1.9), (33, 5, 2.2, 1.2)]
    params = []
    for i, (side, q, kap, mob) in enumerate(specs):
        p = amps.Params.preset(amps.GRAINGROWTH, 0, nx=side, ny=side, nfields=q, grcoef=kap, mobil=mob, tile=32,
                               seed=300 + i, init_amp=0.3)
        p.dt = ensemble.stable_dt(mob, kap)
        for k, v in mixed(monitor).items():
            setattr(p, k, v)
        params.append(p)
    alone = run_alone(params, 33)
    together = run_together(params, 33, chunks=[13, 20])
    for (fa, ta, sa), (fb, tb, sb) in zip(alone, together):
        assert np.array_equal(fa, fb)
        assert np.array_equal(ta, tb)
        assert sa == sb
    steps_per_tier = np.sum([st["tile_steps"] for _, _, st in alone], axis=0)
    assert np.count_nonzero(steps_per_tier) >= 2


def test_ensemble_members_keep_their_own_step_counters_and_stats():
    params = small_members(mixed())
    sims = [amps.Simulation(p, init=amps.INIT_SEEDED) for p in params]
    with amps.Ensemble(sims) as ens:
        ens.run(30)
        ens.synchronize()
    for s, p in zip(sims, params):
        st = s.stats()
        assert st["steps"] == 30
        assert sum(st["tile_steps"]) == 30 * (p.nx // 32) * (p.ny // 32)
        assert st["monitor_evals"] == 1 + 3  # the classification at init, then one per period
        s.close()


def test_ensemble_rejects_incompatible_members():
    a = amps.Simulation(small_members(mixed())[0], init=amps.INIT_SEEDED)
    b = amps.Simulation(amps.Params.preset(amps.GRAINGROWTH, 0, nx=64, ny=64, nfields=2, tile=16, **mixed()),
                        init=amps.INIT_SEEDED)
    k = amps.Simulation(amps.Params.preset(amps.KOBAYASHI, 0, nx=64, ny=64, tile=32), init=amps.INIT_REFERENCE)
    for members in ([a, b], [a, a], [a, k]):
        with pytest.raises(amps.AmpsError):
            amps.Ensemble(members)
    a.run(3)  # a different phase of the cadence
    c = amps.Simulation(small_members(mixed())[1], init=amps.INIT_SEEDED)
    with pytest.raises(amps.AmpsError):
        amps.Ensemble([a, c])
    for s in (a, b, k, c):
        s.close()


def test_ensemble_groups_past_the_launch_cap_match_individual_runs():
    """More members than one launch carries (40 step-argument records in
    the kernel's parameter space): 45 members of Q = 4 and 8, which share an
    occupancy class and so split into two launches of that class, and 3 of
    Q = 16 in a class of their own -- every member still exactly its single
    run, adaptive, over two whole periods and a partial one."""
    base = small_members(mixed())[0]
    params = []
    for i in range(48):
        q = 16 if i >= 45 else (4 if i % 2 else 8)
        side = 32 + 16 * (i % 5)  # 32..96, partial tiles included
        p = base.replace(nx=side, ny=side, nfields=q, seed=500 + i)
        params.append(p)
    alone = run_alone(params, 25)
    together = run_together(params, 25, chunks=[20, 5])
    for k, ((fa, ta, sa), (fb, tb, sb)) in enumerate(zip(alone, together)):
        assert np.array_equal(fa, fb), k
        assert np.array_equal(ta, tb), k
        assert sa == sb, k


@pytest.mark.parametrize("mode", ["adaptive", "fp32", "half"])
def test_ensemble_split_tiles_match_individual_runs(mode, monkeypatch):
    """Split tiles (opt-in, AMPS_ENS_PAIR=1): members of 16 fields run
    their non-monitor steps as two-CTA clusters (8 fields each, the sum of
    squares from both halves' staging in field order).  Whole and ragged
    members, interior tiles (tensor copies) and edge tiles, every tier and
    mixed neighbourhoods: each member exactly its run alone, with split and
    with whole tiles."""
    base = small_members(mixed())[0]
    extra = {"adaptive": {}, "fp32": dict(mode=amps.PUREHIGH, high_tier=amps.TIER_FP32),
             "half": dict(mode=amps.PURELOW)}[mode]
    params = []
    for i, (side, q) in enumerate([(160, 16), (130, 16), (97, 16), (64, 16), (224, 16), (96, 8)]):
        p = base.replace(nx=side, ny=side, nfields=q, seed=700 + i, **extra)
        params.append(p)
    alone = run_alone(params, 25)
    for pair in ("1", "0"):
        monkeypatch.setenv("AMPS_ENS_PAIR", pair)
        together = run_together(params, 25, chunks=[20, 5])
        for k, ((fa, ta, sa), (fb, tb, sb)) in enumerate(zip(alone, together)):
            assert np.array_equal(fa, fb), (pair, k)
            assert np.array_equal(ta, tb), (pair, k)
            assert sa == sb, (pair, k)
    if mode == "adaptive":
        steps_per_tier = np.sum([st["tile_steps"] for _, _, st in alone[:5]], axis=0)
        assert np.count_nonzero(steps_per_tier) == 3
