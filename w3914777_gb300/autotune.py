"""Autotuner for tile shape, monitor and thresholds.

The reference fixes the tile (16x16), the monitor (Monitor1/Monitor2) and the
threshold at compile time and sweeps them from Python by rewriting header
lines (snowflake/end2end_mix.py:13-75).  Here the same sweep runs at run
time through the C ABI: every candidate configuration advances the workload
from the same initial state, its final fields are compared with the plain
FP64 run (max-abs error over every field), and the fastest candidate whose
error is within the bound wins.

    from w3914777_gb300 import autotune
    best, table = autotune.tune(params, init_kind, steps, err_bound=1e-3)
"""
import math
import time

import numpy as np

from . import amps as A


def default_candidates(params):
    """Candidate (name, overrides) list for a workload: three-tier spatial
    and temporal monitors over a threshold grid, both tile shapes, plus the
    all-FP32 and all-half runs as reference points."""
    c = []
    tiles = [32, 16]
    spa = [(1e-3, math.inf), (3e-3, math.inf), (1e-2, math.inf), (2e-2, math.inf), (5e-2, math.inf),
           (1e-3, 1.5), (1e-2, 1.5), (1e-3, 0.9), (1e-3, 0.5)]
    tem = [(1e-6, math.inf), (1e-5, math.inf), (1e-4, math.inf), (1e-3, math.inf), (1e-5, 1e-1), (1e-5, 1e-2),
           (1e-5, 1e-3)]
    rate = [(1e-5, math.inf), (1e-4, math.inf), (1e-3, math.inf), (1e-4, 1e-1), (1e-4, 1e-2), (1e-4, 1e-3)]
    for t in tiles:
        for lo, hi in spa:
            c.append((f"spa t{t} lo={lo:g} hi={hi:g}",
                      dict(mode=A.END2END_MIX, tile=t, monitor=A.MONITOR_SPA, monitor_samples=1, monitor_field=-1,
                           thr_lo=lo, thr_hi=hi if math.isfinite(hi) else 1e300)))
        for lo, hi in tem:
            c.append((f"tem t{t} lo={lo:g} hi={hi:g}",
                      dict(mode=A.END2END_MIX, tile=t, monitor=A.MONITOR_TEM, monitor_samples=1, monitor_field=-1,
                           thr_lo=lo, thr_hi=hi if math.isfinite(hi) else 1e300)))
        for lo, hi in rate:
            c.append((f"rate t{t} lo={lo:g} hi={hi:g}",
                      dict(mode=A.END2END_MIX, tile=t, monitor=A.MONITOR_RATE, monitor_samples=1, monitor_field=-1,
                           thr_lo=lo, thr_hi=hi if math.isfinite(hi) else 1e300)))
    c.append(("all fp32", dict(mode=A.PUREHIGH, high_tier=A.TIER_FP32)))
    c.append(("all half", dict(mode=A.PURELOW)))
    return c


def _run(params, init_state, steps, repeats=1):
    """Advance `steps` from init_state; returns (seconds, final fields, stats)."""
    with A.Simulation(params) as s:
        s.set_fields(init_state)
        s.run(min(steps, 2 * params.cadence))  # warm: captures the period graph
        s.synchronize()
        best = math.inf
        for _ in range(repeats):
            s.set_fields(init_state)
            s.synchronize()
            t0 = time.perf_counter()
            s.run(steps)
            s.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best, s.fields(), s.stats()


def select_best(table, err_bound):
    """The row of the fastest adaptive (end2end_mix) candidate whose max-abs
    error is within err_bound; among equally fast rows the earliest (the
    candidate order is the tie-break); None when no row qualifies.  Rows
    without a timing or an error (failed candidates, NaN errors) and the
    non-adaptive reference points (plain FP64, all-FP32, all-half) never
    win."""
    ok = [r for r in table
          if r.get("seconds") is not None and r.get("err") is not None and r["err"] <= err_bound
          and r.get("overrides", {}).get("mode") == A.END2END_MIX]
    return min(ok, key=lambda r: r["seconds"]) if ok else None


def tune(params, init_kind, steps, err_bound=1e-3, candidates=None, reference=None, repeats=1, log=None,
         runner=None):
    """Return (best, table).  `best` is the table row of the fastest candidate
    with max-abs error <= err_bound (None if none qualifies).  runner(params,
    init_state, steps, repeats) -> (seconds, fields, stats) advances one
    candidate (default: a Simulation on the GPU)."""
    run = runner or _run
    init_state = A.init_host(params, init_kind)
    base = params.replace(mode=A.PUREHIGH, high_tier=A.TIER_FP64, ref_order=0)
    if reference is None:
        t64, reference, _ = run(base, init_state, steps, repeats)
    else:
        t64 = None
    cells = params.nx * params.ny * steps
    table = [{"name": "plain fp64", "seconds": t64, "gcells": cells / t64 / 1e9 if t64 else None, "err": 0.0,
              "overrides": {"mode": A.PUREHIGH, "high_tier": A.TIER_FP64}}]
    for name, ov in candidates or default_candidates(params):
        p = params.replace(**ov)
        if p.check()[0] != 0:
            continue
        try:
            t, f, st = run(p, init_state, steps, repeats)
        except A.AmpsError as e:  # e.g. the staging of this tile does not fit
            table.append({"name": name, "error": str(e)})
            continue
        err = float(np.max(np.abs(f - reference)))
        ts = st["tile_steps"]
        tot = max(sum(ts), 1)
        row = {"name": name, "seconds": t, "gcells": cells / t / 1e9, "err": err,
               "mix": [ts[0] / tot, ts[1] / tot, ts[2] / tot], "overrides": ov}
        table.append(row)
        if log:
            log(row)
    return select_best(table[1:], err_bound), table


def _run_ensemble(members, states, steps, repeats=1):
    """Advance an ensemble of members (amps.Params) from `states` by `steps`:
    (seconds, [final fields], summed tile-steps per tier)."""
    sims = [A.Simulation(p) for p in members]
    try:
        for s, f in zip(sims, states):
            s.set_fields(f)
        best = math.inf
        with A.Ensemble(sims) as ens:
            warm = min(steps, 2 * members[0].cadence)
            ens.run(warm)  # captures the period graphs
            ens.synchronize()
            for _ in range(repeats):
                for s, f in zip(sims, states):
                    s.set_fields(f)
                ens.synchronize()
                t0 = time.perf_counter()
                ens.run(steps)
                ens.synchronize()
                best = min(best, time.perf_counter() - t0)
        fields = [s.fields() for s in sims]
        ts = np.sum([s.stats()["tile_steps"] for s in sims], axis=0)
        return best, fields, ts
    finally:
        for s in sims:
            s.close()


def ensemble_candidates():
    """Candidates for the ensemble: the tile shape and the temporal-family
    monitors (rate, temporal) over a threshold grid; the spatial range
    fails the coarsening workload (shrinking grains change in time, not in
    space)."""
    c = []
    for t in (32, 16):
        for lo, hi in ((1e-5, math.inf), (3e-5, math.inf), (1e-4, math.inf), (1e-5, 1e-2), (1e-5, 1e-3)):
            c.append((f"rate t{t} lo={lo:g} hi={hi:g}",
                      dict(mode=A.END2END_MIX, tile=t, monitor=A.MONITOR_RATE, monitor_samples=1, monitor_field=-1,
                           thr_lo=lo, thr_hi=hi if math.isfinite(hi) else 1e300)))
        for lo, hi in ((1e-5, math.inf), (1e-4, math.inf)):
            c.append((f"tem t{t} lo={lo:g} hi={hi:g}",
                      dict(mode=A.END2END_MIX, tile=t, monitor=A.MONITOR_TEM, monitor_samples=1, monitor_field=-1,
                           thr_lo=lo, thr_hi=hi if math.isfinite(hi) else 1e300)))
    return c


def tune_ensemble(members, steps, err_bound=1e-3, candidates=None, repeats=1, log=None, runner=None):
    """Tile shape, monitor and thresholds for an ensemble (every member takes
    the same overrides): each candidate advances the whole ensemble `steps`
    from the members' seeded states; its error is the largest max-abs
    difference of any member from the plain-FP64 ensemble; the fastest
    candidate within err_bound wins (select_best).  Returns (best, table)."""
    run = runner or _run_ensemble
    states = [A.init_host(p, A.INIT_SEEDED) for p in members]
    base = [p.replace(mode=A.PUREHIGH, high_tier=A.TIER_FP64, ref_order=0) for p in members]
    t64, ref, _ = run(base, states, steps, repeats)
    ncells = sum(p.nx * p.ny for p in members) * steps
    table = [{"name": "plain fp64", "seconds": t64, "gcells": ncells / t64 / 1e9, "err": 0.0,
              "overrides": {"mode": A.PUREHIGH, "high_tier": A.TIER_FP64}}]
    for name, ov in candidates or ensemble_candidates():
        ps = [p.replace(**ov) for p in members]
        if any(p.check()[0] != 0 for p in ps):
            continue
        try:
            t, fields, ts = run(ps, states, steps, repeats)
        except A.AmpsError as e:
            table.append({"name": name, "error": str(e)})
            continue
        err = max(float(np.max(np.abs(f - r))) for f, r in zip(fields, ref))
        tot = max(float(np.sum(ts)), 1.0)
        row = {"name": name, "seconds": t, "gcells": ncells / t / 1e9, "err": err,
               "mix": [float(x) / tot for x in ts], "overrides": ov}
        table.append(row)
        if log:
            log(row)
    return select_best(table[1:], err_bound), table


WORKLOADS = {
    # name: (preset model, tuned file, description, default steps, initial state, candidate tiles)
    "graingrowth": ("graingrowth", "graingrowth_1024_q8.json", "graingrowth preset 0 (1024x1024, Q=8)", 10000,
                    A.INIT_SEEDED, (32, 16)),
    "kobayashi": ("kobayashi", "kobayashi_512.json",
                  "kobayashi preset 0 (512x512 zero-flux, seeded noise)", 2000, A.INIT_SEEDED, (32, 16)),
    "sintering": ("sintering", "sintering_1024_n16.json", "sintering preset 0 (1024x1024, 16 particles)", 2000,
                  A.INIT_SEEDED, (32,)),
    "ensemble": ("graingrowth", "ensemble_64.json",
                 "64 seeded grain-growth members (sides 128..1024, Q in {4,8,12,16}, seed 2024)", 1000,
                 A.INIT_SEEDED, (32, 16)),
}


def workload_params(name):
    """Parameters, initial-state kind and default tuning length of a named workload."""
    model, _, _, steps, init, _ = WORKLOADS[name]
    return A.Params.preset(model, 0), init, steps


def _main():
    """python -m w3914777_gb300.autotune {graingrowth|kobayashi|sintering|ensemble} [steps] [err_bound] [out]
    Tunes the named preset-0 workload (or the 64-member ensemble) and writes
    w3914777_gb300/tuned/<file>.json (or `out`)."""
    import json
    import os
    import sys
    name = sys.argv[1] if len(sys.argv) > 1 else "graingrowth"
    if name not in WORKLOADS:
        raise SystemExit(f"unknown workload {name!r}: one of {sorted(WORKLOADS)}")
    p, init, default_steps = workload_params(name)
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else default_steps
    bound = float(sys.argv[3]) if len(sys.argv) > 3 else 1e-3
    tiles = WORKLOADS[name][5]
    log = lambda r: print(json.dumps(r), flush=True)  # noqa: E731
    if name == "ensemble":
        from . import ensemble
        best, table = tune_ensemble(ensemble.member_params(count=64, seed=2024), steps, bound, log=log)
    else:
        cands = [c for c in default_candidates(p) if c[1].get("tile", tiles[0]) in tiles]
        best, table = tune(p, init, steps, bound, candidates=cands, log=log)
    out = sys.argv[4] if len(sys.argv) > 4 else os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned",
                                                               WORKLOADS[name][1])
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        json.dump({"workload": WORKLOADS[name][2], "steps": steps, "err_bound": bound, "best": best, "table": table},
                  f, indent=1)
    print("best:", json.dumps(best))


if __name__ == "__main__":
    _main()
