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


def tune(params, init_kind, steps, err_bound=1e-3, candidates=None, reference=None, repeats=1, log=None):
    """Return (best, table).  `best` is the table row of the fastest candidate
    with max-abs error <= err_bound (None if none qualifies)."""
    init_state = A.init_host(params, init_kind)
    base = params.replace(mode=A.PUREHIGH, high_tier=A.TIER_FP64, ref_order=0)
    if reference is None:
        t64, reference, _ = _run(base, init_state, steps, repeats)
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
            t, f, st = _run(p, init_state, steps, repeats)
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
    ok = [r for r in table[1:] if "err" in r and r["err"] <= err_bound and r["overrides"].get("mode") == A.END2END_MIX]
    best = min(ok, key=lambda r: r["seconds"]) if ok else None
    return best, table


WORKLOADS = {
    # name: (preset model, tuned file, description, default steps, initial state, candidate tiles)
    "graingrowth": ("graingrowth", "graingrowth_1024_q8.json", "graingrowth preset 0 (1024x1024, Q=8)", 10000,
                    A.INIT_SEEDED, (32, 16)),
    "kobayashi": ("kobayashi", "kobayashi_512.json",
                  "kobayashi preset 0 (512x512 zero-flux, seeded noise)", 2000, A.INIT_SEEDED, (32, 16)),
    "sintering": ("sintering", "sintering_1024_n16.json", "sintering preset 0 (1024x1024, 16 particles)", 2000,
                  A.INIT_SEEDED, (32,)),
}


def workload_params(name):
    """Parameters, initial-state kind and default tuning length of a named workload."""
    model, _, _, steps, init, _ = WORKLOADS[name]
    return A.Params.preset(model, 0), init, steps


def _main():
    """python -m w3914777_gb300.autotune {graingrowth|kobayashi|sintering} [steps] [err_bound] [out]
    Tunes the named preset-0 workload and writes w3914777_gb300/tuned/<file>.json
    (or `out`)."""
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
    cands = [c for c in default_candidates(p) if c[1].get("tile", tiles[0]) in tiles]
    best, table = tune(p, init, steps, bound, candidates=cands, log=lambda r: print(json.dumps(r), flush=True))
    out = sys.argv[4] if len(sys.argv) > 4 else os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned",
                                                               WORKLOADS[name][1])
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        json.dump({"workload": WORKLOADS[name][2], "steps": steps, "err_bound": bound, "best": best, "table": table},
                  f, indent=1)
    print("best:", json.dumps(best))


if __name__ == "__main__":
    _main()
