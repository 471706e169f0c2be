"""Grain growth on ragged grids: sides that are not multiples of the tile.

Storage keeps whole tiles (row pitch ntx*tile); the last tile column and row
are partial and compute only their cells inside the domain, each neighbour
read at the tier of the tile that owns it after the boundary map (the
periodic wrap of the last column lands in column 0).  The reference has no
such grids (its sizes are compile-time multiples of the tile,
graingrowth/paras/para1.h); the ensemble workload draws arbitrary integer
sides.  Checked against the oracle's restatement of graingrowth/function.h:5-30
(sizes independent of any tile) and its monitor/get_type rule with samples past
the domain skipped."""
import numpy as np
import pytest

import oracle_bind as ob

pytestmark = pytest.mark.gpu


def amps():
    from w3914777_gb300 import amps as w
    return w


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _oracle_params(p, nx, ny, q):
    return ob.gg_params(nx, ny, q=q, bc=p.bc, stencil=p.stencil, dx=p.dx, dy=p.dy, dt=p.dt, mobil=p.mobil,
                        grcoef=p.grcoef, gamma=p.gamma)


@pytest.mark.parametrize("nx,ny,tile,bc,ref_order", [
    (100, 72, 32, 0, 1), (100, 72, 32, 1, 0), (45, 70, 16, 0, 0), (33, 33, 32, 1, 1), (129, 40, 32, 0, 0),
    (47, 47, 16, 1, 1)])
def test_ragged_fp64_vs_oracle(nx, ny, tile, bc, ref_order):
    """All-FP64 runs (the staged FP64 kernel for whole tiles, the cell path for
    partial ones) against the oracle: <= 1e-12 relative after 25 steps."""
    w = amps()
    q, steps = 4, 25
    p = w.Params.preset("graingrowth", 0, mode="purehigh", nx=nx, ny=ny, nfields=q, tile=tile, bc=bc,
                        ref_order=ref_order, init_amp=0.3)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        assert s.ntiles == (-(-ny // tile), -(-nx // tile))
        s.run(steps)
        f = s.fields()
    o = ob.gg_run(_oracle_params(p, nx, ny, q), list(f0), steps)
    e = max(rel_err(f[k], o[k]) for k in range(q))
    print(f"ragged {nx}x{ny} tile {tile} bc {bc} ref {ref_order}: {e:.3e}")
    assert e <= 1e-12


@pytest.mark.parametrize("nx,ny,bc", [(100, 72, 0), (75, 41, 1)])
def test_ragged_fp32_and_half_vs_oracle(nx, ny, bc):
    """All-FP32 and all-half runs: whole tiles stage through shared memory
    (and, at 32x32, by tensor copy), partial tiles take the cell path; both
    within their storage precision of the FP64 oracle."""
    w = amps()
    q, steps = 3, 30
    res = {}
    for mode, tier in (("purehigh", w.TIER_FP32), ("purelow", w.TIER_FP32)):
        p = w.Params.preset("graingrowth", 0, mode=mode, high_tier=tier, nx=nx, ny=ny, nfields=q, bc=bc,
                            init_amp=0.3)
        f0 = w.init_host(p, w.INIT_SEEDED)
        with w.Simulation(p, init=w.INIT_SEEDED) as s:
            s.run(steps)
            res[mode] = s.fields()
    o = ob.gg_run(_oracle_params(p, nx, ny, q), list(f0), steps)
    e32 = max(float(np.abs(res["purehigh"][k] - o[k]).max()) for k in range(q))
    e16 = max(float(np.abs(res["purelow"][k] - o[k]).max()) for k in range(q))
    print(f"ragged {nx}x{ny}: fp32 {e32:.3e}, half {e16:.3e}")
    assert e32 <= 1e-5
    assert e16 <= 2e-2


def _oracle_decisions(w, p, prev, now):
    fields = range(p.nfields) if p.monitor_field < 0 else [p.monitor_field]
    m = None
    for k in fields:
        if p.monitor == w.MONITOR_SPA:
            mk = ob.monitor_spa(now[k], p.tile, p.monitor_samples)
        elif p.monitor == w.MONITOR_RATE:
            mk = ob.monitor_rate(now[k], prev[k], p.tile, p.cadence, p.monitor_samples)
        else:
            mk = ob.monitor_tem(now[k], prev[k], p.tile, p.monitor_samples)
        m = mk if m is None else np.maximum(m, mk)
    return m, ob.classify(m, p.thr_lo, p.thr_hi)


@pytest.mark.parametrize("monitor,samples,nx,ny,tile", [
    (3, 1, 100, 72, 32), (3, 0, 100, 72, 32), (2, 1, 90, 51, 16), (2, 0, 100, 72, 32), (1, 1, 70, 100, 32),
    (1, 0, 61, 45, 16)])
def test_ragged_adaptive_decisions_match_oracle(monitor, samples, nx, ny, tile):
    """The fused step's monitor on partial tiles (cells past the domain are
    not samples) and the classification against the oracle on the GPU's own
    state, with thresholds at quantiles of the metric so that every tier
    occurs."""
    w = amps()
    back = 1 if monitor == 3 else 10
    base = dict(mode="end2end_mix", nx=nx, ny=ny, nfields=4, tile=tile, monitor=monitor, monitor_samples=samples,
                monitor_field=-1, init_amp=0.3, max_log=16)
    probe = w.Params.preset("graingrowth", 0, thr_lo=0.0, thr_hi=0.0, **base)
    with w.Simulation(probe, init=w.INIT_SEEDED) as s:
        s.run(20)
        m = s.metric().ravel()
    lo, hi = float(np.quantile(m, 0.3)), float(np.quantile(m, 0.7))
    p = w.Params.preset("graingrowth", 0, thr_lo=lo, thr_hi=hi, **base)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(40 - back)
        prev = s.fields()
        s.run(back)
        now = s.fields()
        m_gpu, t_gpu, st = s.metric(), s.tiers(), s.stats()
    m, t = _oracle_decisions(w, p, prev, now)
    print(f"ragged {nx}x{ny} tile {tile} monitor {monitor} samples {samples}: tiers {np.bincount(t.ravel(), minlength=3)}"
          f", tile steps {st['tile_steps']}")
    assert np.array_equal(m_gpu, m), float(np.nanmax(np.abs(m_gpu - m)))
    assert np.array_equal(t_gpu, t)
    assert sum(st["tile_steps"]) == 40 * t.size


@pytest.mark.parametrize("monitor", [3, 2])
def test_ragged_adaptive_envelope_and_partial_tiles_at_every_tier(monitor):
    """An adaptive ragged run against the FP64 oracle, with the partial
    tiles forced through every tier by the tier schedule (one map per period:
    all half, all FP32, all FP64)."""
    w = amps()
    nx, ny, q, steps = 100, 72, 4, 60
    base = dict(mode="end2end_mix", nx=nx, ny=ny, nfields=q, monitor=monitor, monitor_samples=1, monitor_field=-1,
                init_amp=0.3, thr_lo=1e-5, thr_hi=1e-3)
    p = w.Params.preset("graingrowth", 0, **base)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(steps)
        f = s.fields()
        st = s.stats()
    o = ob.gg_run(_oracle_params(p, nx, ny, q), list(f0), steps)
    e = max(float(np.abs(f[k] - o[k]).max()) for k in range(q))
    print(f"ragged adaptive monitor {monitor}: max abs {e:.3e}, tile steps {st['tile_steps']}")
    assert e <= 1e-3
    # a forced schedule: every tile (partial ones included) at each tier in
    # turn, one period each after the resting classification's
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        nt = s.ntiles
        maps = np.stack([np.full(nt, t, np.uint8) for t in (w.TIER_HALF, w.TIER_FP32, w.TIER_FP64, w.TIER_FP64)])
        s.set_tier_schedule(maps)
        s.run(40)
        g = s.fields()
        st = s.stats()
    o = ob.gg_run(_oracle_params(p, nx, ny, q), list(f0), 40)
    e = max(float(np.abs(g[k] - o[k]).max()) for k in range(q))
    print(f"ragged forced tiers: max abs {e:.3e}, tile steps {st['tile_steps']}")
    assert all(x > 0 for x in st["tile_steps"])
    assert e <= 2e-2


def test_ragged_fields_round_trip_and_reductions():
    """set/get of a ragged grid's fields at every tier, and the FP64
    reductions over the domain only (the storage's padding is never read)."""
    w = amps()
    nx, ny = 77, 45
    rng = np.random.default_rng(5)
    for mode, tier in (("purehigh", w.TIER_FP64), ("purehigh", w.TIER_FP32), ("purelow", w.TIER_FP32)):
        p = w.Params.preset("graingrowth", 0, mode=mode, high_tier=tier, nx=nx, ny=ny, nfields=3)
        x = rng.uniform(-1, 1, (3, ny, nx))
        with w.Simulation(p) as s:
            s.set_fields(x)
            y = s.fields()
            tot = s.reduce(1, w.REDUCE_SUM)
        if mode == "purelow":
            x = x.astype(np.float16).astype(np.float64)
        elif tier == w.TIER_FP32:
            x = x.astype(np.float32).astype(np.float64)
        assert np.array_equal(y, x)
        assert abs(tot - x[1].sum()) <= 1e-12 * np.abs(x[1]).sum()
