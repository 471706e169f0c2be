"""Tier control for the cost and selection experiments, through the C ABI:
a replayed decision log (amps_set_tier_schedule) reproduces the monitored
run bit for bit without the monitor; a static tier map set on a live state
(amps_set_tile_tiers) runs like the same map chosen at creation; the
on-demand monitor (amps_measure_tiles) equals the fused monitor's metric and
a numpy restatement of the sample-lattice reductions; the experiment drivers
run end to end."""
import numpy as np
import pytest

from w3914777_gb300 import amps, experiments as E

pytestmark = pytest.mark.gpu


def adaptive(model, monitor, thr=None, **kw):
    """Two-tier adaptive run of the model's first reference preset; without a
    threshold, the median of the non-zero tile metrics after one period (so
    that the run mixes tiers)."""
    p = amps.Params.preset(model, 1, **kw).replace(mode=amps.END2END_MIX, monitor=monitor, max_log=64)
    if thr is None:
        with amps.Simulation(p.replace(thr_lo=1e300, thr_hi=1e300), init=amps.INIT_REFERENCE) as s:
            s.run(p.cadence)
            m = s.metric()
            thr = float(np.median(m[m > 0])) if (m > 0).any() else 0.5
    return p.replace(thr_lo=thr, thr_hi=thr)


CASES = [
    ("kobayashi", amps.MONITOR_SPA, {}),
    ("kobayashi", amps.MONITOR_TEM, {}),
    ("graingrowth", amps.MONITOR_SPA, {}),
    ("graingrowth", amps.MONITOR_TEM, {}),
    ("sintering", amps.MONITOR_TEM, {}),
    ("sintering", amps.MONITOR_SPA, {}),
    # FMA-form kernels: 32x32 tiles (eight grain fields: the one-warp-per-field
    # step beside the monitor steps' kernel), sintering's FP64 row bands
    ("graingrowth", amps.MONITOR_SPA, dict(ref_order=0, tile=32, nfields=8)),
    ("sintering", amps.MONITOR_SPA, dict(ref_order=0, tile=32)),
]


@pytest.mark.parametrize("model,monitor,kw", CASES)
@pytest.mark.parametrize("graphs", [True, False])
def test_replayed_schedule_equals_monitored_run(model, monitor, kw, graphs):
    p = adaptive(model, monitor, **kw)
    steps = 105  # ten periods and a partial one
    with amps.Simulation(p, init=amps.INIT_REFERENCE, graphs=graphs) as s:
        s.run(steps)
        log = s.decision_log()
        f_mon, st_mon = s.fields(), s.stats()
    assert len(log) == steps // p.cadence + 1
    tiers_seen = np.unique(log)
    assert len(tiers_seen) >= 2, "the case should mix tiers"
    with amps.Simulation(p, graphs=graphs) as s:
        s.set_tier_schedule(log)
        s.init(amps.INIT_REFERENCE)
        s.run(steps)
        assert np.array_equal(s.fields(), f_mon)
        assert np.array_equal(s.decision_log(), log)
        st = s.stats()
        assert st["tile_steps"] == st_mon["tile_steps"]
        assert (st["promotions"], st["demotions"]) == (st_mon["promotions"], st_mon["demotions"])
        # a second run from the same state restarts the schedule at its first map
        s.init(amps.INIT_REFERENCE)
        s.run(steps)
        assert np.array_equal(s.fields(), f_mon)
        # clearing the schedule restores the monitor
        s.set_tier_schedule(None)
        s.init(amps.INIT_REFERENCE)
        s.run(steps)
        assert np.array_equal(s.fields(), f_mon)


def test_short_schedule_holds_its_last_map():
    p = adaptive("kobayashi", amps.MONITOR_SPA)
    with amps.Simulation(p, init=amps.INIT_REFERENCE) as s:
        s.run(20)
        first = s.decision_log()[:2]
    with amps.Simulation(p) as s:
        s.set_tier_schedule(first)
        s.init(amps.INIT_REFERENCE)
        s.run(50)
        log = s.decision_log()
        assert len(log) == 6
        assert np.array_equal(log[0], first[0]) and all(np.array_equal(m, first[1]) for m in log[1:])


def test_schedule_and_tier_map_arguments_are_checked():
    p = adaptive("kobayashi", amps.MONITOR_SPA)
    with amps.Simulation(p, init=amps.INIT_REFERENCE) as s:
        bad = np.full((1,) + s.ntiles, amps.TIER_FP32, dtype=np.uint8)  # two-tier run: no FP32 storage
        with pytest.raises(amps.AmpsError):
            s.set_tier_schedule(bad)
        with pytest.raises(amps.AmpsError):
            s.set_tiers(np.full(s.ntiles, amps.TIER_FP64, dtype=np.uint8))  # adaptive: tiers come from the monitor
    with amps.Simulation(amps.Params.preset("kobayashi", 1).replace(mode=amps.GRAM1, gram_ratio=0.5),
                         init=amps.INIT_REFERENCE) as s:
        with pytest.raises(amps.AmpsError):
            s.set_tier_schedule(np.zeros((1,) + s.ntiles, dtype=np.uint8))  # static mode: nothing classifies
        with pytest.raises(amps.AmpsError):
            s.set_tiers(np.full(s.ntiles, 7, dtype=np.uint8))


@pytest.mark.parametrize("model", ["kobayashi", "graingrowth", "sintering"])
@pytest.mark.parametrize("mode,ratio", [(amps.GRAM1, 0.4), (amps.GRAM2, 0.63)])
def test_set_tiers_on_a_live_state_equals_the_static_map(model, mode, ratio):
    base = amps.Params.preset(model, 1)
    with amps.Simulation(base.replace(mode=mode, gram_ratio=ratio), init=amps.INIT_REFERENCE) as s:
        target = s.tiers()
        s.run(30)
        f_ref = s.fields()
    assert 0 < (target == amps.TIER_HALF).sum() < target.size
    with amps.Simulation(base.replace(mode=mode, gram_ratio=0.0), init=amps.INIT_REFERENCE) as s:
        assert (s.tiers() == base.high_tier).all()
        s.set_tiers(target)
        assert np.array_equal(s.tiers(), target)
        s.run(30)
        assert np.array_equal(s.fields(), f_ref)


def lattice(T, kind):
    if kind == amps.MONITOR_SPA:
        return [(k * (T - 1) * 2 + 3) // 6 for k in range(4)]
    return [T // 8 + k * (T // 4) for k in range(4)]


def lattice_view(f, T, kind):
    """[nty][ntx][16] samples of one field on the monitor's lattice."""
    idx = lattice(T, kind)
    ny, nx = f.shape
    tiles = f.reshape(ny // T, T, nx // T, T).transpose(0, 2, 1, 3)
    return tiles[:, :, idx][:, :, :, idx].reshape(ny // T, nx // T, 16)


@pytest.mark.parametrize("model", ["kobayashi", "graingrowth"])
def test_measure_tiles_matches_fused_monitor_and_numpy(model):
    p = adaptive(model, amps.MONITOR_SPA)
    mf = p.monitor_field
    with amps.Simulation(p, init=amps.INIT_REFERENCE) as s:
        # the initial classification's metric is the spatial metric of the state
        assert np.array_equal(s.measure_tiles(amps.MONITOR_SPA), s.metric())
    with amps.Simulation(amps.Params.preset(model, 1), init=amps.INIT_REFERENCE) as s:  # plain FP64
        s.run(40)
        f0 = s.fields()
        fields = range(s.nf) if mf < 0 else [mf]
        spa = np.zeros(s.ntiles)
        for k in fields:
            v = lattice_view(f0[k], p.tile, amps.MONITOR_SPA)
            spa = np.maximum(spa, np.maximum(v.max(-1), 0.0) - np.minimum(v.min(-1), 1.0))
        assert np.array_equal(s.measure_tiles(amps.MONITOR_SPA), spa)
        with pytest.raises(amps.AmpsError):
            s.measure_tiles(amps.MONITOR_TEM)  # no temporal reference yet
        s.store_temporal_reference()
        assert (s.measure_tiles(amps.MONITOR_TEM) == 0).all()
        s.run(9)
        f1 = s.fields()
        tem = np.zeros(s.ntiles)
        for k in fields:
            d = np.abs(lattice_view(f1[k], p.tile, amps.MONITOR_TEM) - lattice_view(f0[k], p.tile, amps.MONITOR_TEM))
            tem = np.maximum(tem, d.max(-1))
        got = s.measure_tiles(amps.MONITOR_TEM)
        assert np.array_equal(got, tem) and got.max() > 0


@pytest.mark.parametrize("strategy,monitor", [("AMSTENCIL", amps.MONITOR_SPA), ("AMSTENCIL", amps.MONITOR_TEM),
                                              ("GRAM1", 0), ("GRAM2", 0)])
def test_motivation_runs(strategy, monitor):
    hi = E.motivation("kobayashi", 1, 100, 0.5, strategy=strategy, monitor=monitor or amps.MONITOR_SPA)
    lo = E.motivation("kobayashi", 1, 100, 0.9, strategy=strategy, monitor=monitor or amps.MONITOR_SPA)
    assert 0 <= hi["error"] < 0.1 and np.isfinite(lo["error"])
    assert lo["low_share"] >= hi["low_share"] > 0
    if strategy == "AMSTENCIL":
        # quota n: every tile with a non-zero metric and its surroundings stay high
        full = E.motivation("kobayashi", 1, 100, 0.0, strategy=strategy, monitor=monitor)
        assert full["low_share"] == 0.0 and full["error"] < 1e-13
    else:
        assert hi["low_share"] == pytest.approx(0.5, abs=0.02)


def test_monitor_cost_and_sweeps_run():
    c = E.monitor_cost(adaptive("kobayashi", amps.MONITOR_SPA), 200, repeats=2)
    assert c["identical"] and c["ms_with"] > 0 and c["ms_without"] > 0 and c["classifications"] == 21
    assert np.isfinite(c["monitor_percent"])
    rows = E.end2end_sweep("kobayashi", presets=(1,), high_tiers=(amps.TIER_FP64,), steps=60, spa_thresholds=[0.1],
                           tem_thresholds=[1e-4], ratios=[0.5], repeats=1)
    assert [r["strategy"] for r in rows] == ["PURE", "AMSTENCIL", "AMSTENCIL", "GRAM1", "GRAM2"]
    assert all(r["ms"] > 0 for r in rows) and all(np.isfinite(r["error"]) for r in rows)
    assert len(E.speedup_table(rows)) == 4


@pytest.mark.parametrize("high,thr", [(amps.TIER_FP64, (1e-4, 1e-4)), (amps.TIER_FP64, (1e-5, 1e-3)),
                                      (amps.TIER_FP32, (1e-4, 1e-4))])
def test_tile_types_use_the_reference_encoding(high, thr):
    p = amps.Params.preset("graingrowth", 0, nx=128, ny=128, nfields=4, high_tier=high, thr_lo=thr[0],
                           thr_hi=thr[1])
    with amps.Simulation(p, init=amps.INIT_SEEDED) as s:
        s.run(40)
        t, ty = s.tiers(), s.tile_types()
    want = np.where(t == amps.TIER_HALF, 1, np.where(t == high, 2, 3))
    assert np.array_equal(ty, want) and set(np.unique(ty)) <= ({1, 2, 3} if thr[0] < thr[1] else {1, 2})
