"""Threshold / ratio sweeps, errors, speedups, monitor cost and oracle tile
selection, driven through the C ABI.

The reference runs each experiment by rewriting its parameter headers and
recompiling one program per configuration (snowflake/end2end_mix.py,
end2end_pure.py, monitor_independent_with{,out}monitor.py, motivation_mix.py,
motivation_pure.py and their graingrowth/ and sintering/ twins), then
post-processes the CSVs with pandas (end2enderror.py, get_speedup.py,
monitor_percent.py, motivationerror.py).  Here a configuration is a
`Params` value, a run is a `Simulation`, and results are plain dict rows
(written as CSV with the csv module).

Runs are timed with CUDA events on the run's stream over steps
[skip, steps) -- the reference's window starts at step 5
(snowflake/end2end_mix.cu, `if(i==5)` before the loop body) -- after an
untimed warm-up that captures the period graphs.
"""
import argparse
import csv
import json
import os
from collections import deque

import numpy as np

from . import amps as A

# snowflake/end2end_mix.py:19-21 (spatial / temporal threshold lists) and
# :9-11 (GRAM ratios 0.01 .. 1.00)
REFERENCE_SPA_THRESHOLDS = [1e-6, 1e-5, 1e-4, 1e-3, 0.1, 0.15, 0.2, 0.25, 0.3, 0.35, 0.4, 0.45, 0.5, 0.55, 0.6,
                            0.65, 0.7, 0.75, 0.8, 0.85, 0.9, 0.91, 0.92, 0.93, 0.94, 0.95, 0.96, 0.97, 0.98, 0.99]
REFERENCE_TEM_THRESHOLDS = [1e-20, 1e-19, 1e-18, 1e-17, 1e-16, 1e-15, 1e-14, 1e-13, 1e-12, 1e-11, 1e-10, 1e-9,
                            1e-8, 1e-7, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 1e-1, 0.15, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7,
                            0.8, 0.9, 0.99]
REFERENCE_RATIOS = [round(0.01 * i, 2) for i in range(1, 101)]
# snowflake/motivation_mix.py:5,9: low-tile ratios and step counts
MOTIVATION_RATIOS = [0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9]
MOTIVATION_STEPS = [500, 1000, 1500, 2000]

# The field each reference program writes out: phi (snowflake), eta2
# (graingrowth/end2end_mix.cu:109-113), con (sintering/main.cu:470).
OUTPUT_FIELD = {A.KOBAYASHI: 0, A.GRAINGROWTH: 1, A.SINTERING: 0}
MODEL_NAMES = {A.KOBAYASHI: "kobayashi", A.GRAINGROWTH: "graingrowth", A.SINTERING: "sintering"}
TIER_NAMES = {A.TIER_FP64: "double", A.TIER_FP32: "float"}


def mean_abs_error(a, b):
    """sum |a - b| / cells: the reference's error of a run against the plain
    high-precision one (snowflake/end2enderror.py:34, graingrowth/:33,
    sintering/:36; their divisor is the 512x512 grid)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        raise ValueError(f"shape mismatch {a.shape} vs {b.shape}")
    return float(np.abs(a - b).sum() / a.size)


def _stream():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("the experiments run on the GPU: no CUDA device")
    return torch.cuda.Stream()


def run_case(params, steps, init=A.INIT_REFERENCE, repeats=5, skip=5, schedule=None, stream=None):
    """`repeats` runs of `steps` steps from the initial state `init` (an
    INIT_* kind or an array of fields) on one handle.  Returns
    {"ms": device ms of steps [skip, steps) per repeat, "field": the output
    field after the last repeat, "stats": its statistics}.  `schedule`: tier
    maps that replace the monitor (Simulation.set_tier_schedule)."""
    import torch

    stream = stream or _stream()
    skip = min(skip, steps)

    def start(s):
        if isinstance(init, (int, np.integer)):
            s.init(int(init))
        else:
            s.set_fields(init)

    with A.Simulation(params) as s:
        s.set_stream(stream.cuda_stream)
        if schedule is not None:
            s.set_tier_schedule(schedule)
        start(s)
        s.run(min(steps, 2 * params.cadence))  # warm-up: captures the period graphs
        ms = []
        for _ in range(repeats):
            start(s)
            s.run(skip)
            s.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.run(steps - skip)
            b.record(stream)
            s.synchronize()
            ms.append(a.elapsed_time(b))
        return {"ms": ms, "field": s.field(OUTPUT_FIELD[params.model]), "stats": s.stats()}


def decision_log(params, steps, init=A.INIT_REFERENCE, stream=None):
    """The tier map of every classification of one monitored run (the
    initial one first)."""
    p = params.replace(max_log=steps // params.cadence + 2)
    with A.Simulation(p) as s:
        s.set_stream((stream or _stream()).cuda_stream)
        if isinstance(init, (int, np.integer)):
            s.init(int(init))
        else:
            s.set_fields(init)
        s.run(steps)
        return s.decision_log()


def _mixed(params, monitor, threshold):
    """The reference's two-tier adaptive configuration at one threshold."""
    return params.replace(mode=A.END2END_MIX, monitor=monitor, thr_lo=threshold, thr_hi=threshold)


def end2end_sweep(model, presets=(1, 2, 3, 4, 5), high_tiers=(A.TIER_FP64, A.TIER_FP32), steps=500,
                  spa_thresholds=REFERENCE_SPA_THRESHOLDS, tem_thresholds=REFERENCE_TEM_THRESHOLDS,
                  ratios=REFERENCE_RATIOS, repeats=5, skip=5, **overrides):
    """Time and error of every strategy against the plain high-precision run
    (snowflake/end2end_mix.py and end2end_pure.py): for each high tier and
    preset, PURE, then AMSTENCIL with the spatial and the temporal monitor
    at each threshold, then GRAM1 and GRAM2 at each ratio.  One row per run:
    model, high, preset, strategy, monitor, param (threshold or ratio), ms
    (mean over repeats), error (mean_abs_error of the output field against
    PURE) and low_share (fraction of tile-steps below the high tier)."""
    stream = _stream()
    rows = []
    for high in high_tiers:
        for preset in presets:
            base = A.Params.preset(model, preset, **overrides).replace(high_tier=high)
            pure = run_case(base.replace(mode=A.PUREHIGH), steps, repeats=repeats, skip=skip, stream=stream)
            common = {"model": model, "high": TIER_NAMES[high], "preset": preset}
            rows.append(dict(common, strategy="PURE", monitor=0, param=0.0, ms=float(np.mean(pure["ms"])),
                             error=0.0, low_share=0.0))

            def add(strategy, monitor, param, p):
                r = run_case(p, steps, repeats=repeats, skip=skip, stream=stream)
                ts = r["stats"]["tile_steps"]
                low = (sum(ts) - ts[high]) / max(sum(ts), 1)
                rows.append(dict(common, strategy=strategy, monitor=monitor, param=float(param),
                                 ms=float(np.mean(r["ms"])), error=mean_abs_error(r["field"], pure["field"]),
                                 low_share=low))

            for monitor, thresholds in ((A.MONITOR_SPA, spa_thresholds), (A.MONITOR_TEM, tem_thresholds)):
                for thr in thresholds:
                    add("AMSTENCIL", monitor, thr, _mixed(base, monitor, thr))
            for mode, name in ((A.GRAM1, "GRAM1"), (A.GRAM2, "GRAM2")):
                for ratio in ratios:
                    add(name, 0, ratio, base.replace(mode=mode, gram_ratio=ratio))
    return rows


def _group(rows, keys):
    out = {}
    for r in rows:
        out.setdefault(tuple(r[k] for k in keys), []).append(r)
    return out


def speedup_table(rows):
    """Speedup of each strategy / monitor / parameter over PURE, per high
    tier: the mean PURE time over presets divided by the strategy's mean
    time over presets (snowflake/get_speedup.py:6-20)."""
    out = []
    pure = {k: np.mean([r["ms"] for r in v]) for k, v in _group(
        [r for r in rows if r["strategy"] == "PURE"], ("model", "high")).items()}
    for (model, high, strategy, monitor, param), v in _group(
            [r for r in rows if r["strategy"] != "PURE"], ("model", "high", "strategy", "monitor", "param")).items():
        out.append({"model": model, "high": high, "strategy": strategy, "monitor": monitor, "param": param,
                    "speedup": float(pure[(model, high)] / np.mean([r["ms"] for r in v]))})
    return out


def error_table(rows):
    """Mean over presets of each strategy's error (snowflake/end2enderror.py:25-40)."""
    return [{"model": k[0], "high": k[1], "strategy": k[2], "monitor": k[3], "param": k[4],
             "avg_error": float(np.mean([r["error"] for r in v]))}
            for k, v in _group([r for r in rows if r["strategy"] != "PURE"],
                               ("model", "high", "strategy", "monitor", "param")).items()]


def write_csv(rows, path):
    """Rows (dicts with the same keys) as a CSV file with a header line."""
    if not rows:
        raise ValueError("no rows")
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w", newline="") as f:
        w = csv.DictWriter(f, fieldnames=list(rows[0].keys()))
        w.writeheader()
        w.writerows(rows)
    return path


def monitor_cost(params, steps=500, repeats=5, skip=5, init=A.INIT_REFERENCE, stream=None):
    """Share of an adaptive run's time spent on the monitor and its
    classifications (the reference's Table-4 harness:
    snowflake/monitor_independent_withmonitor.cu times the whole loop,
    monitor_independent_withoutmonitor.cu the update kernels alone, and
    monitor_percent.py reports (with - without) / with * 100).  "without" here
    is the same run with the monitored run's decision log replayed in place
    of the monitor (Simulation.set_tier_schedule): the same tiles at the same
    tiers, in-register conversions included, no monitor epilogue and no
    metric-driven classification.  `identical` records that both runs end in
    the same output field, bit for bit."""
    if params.mode != A.END2END_MIX:
        raise ValueError("monitor_cost needs an adaptive (END2END_MIX) configuration")
    stream = stream or _stream()
    log = decision_log(params, steps, init=init, stream=stream)
    with_m = run_case(params, steps, init=init, repeats=repeats, skip=skip, stream=stream)
    without = run_case(params, steps, init=init, repeats=repeats, skip=skip, schedule=log, stream=stream)
    tw, to = float(np.mean(with_m["ms"])), float(np.mean(without["ms"]))
    return {"ms_with": tw, "ms_without": to, "monitor_percent": (tw - to) / tw * 100.0,
            "classifications": int(len(log)),
            "identical": bool(np.array_equal(with_m["field"], without["field"], equal_nan=True))}


def monitor_cost_sweep(model, presets=(1, 2, 3, 4, 5), high_tiers=(A.TIER_FP64, A.TIER_FP32), steps=500,
                       spa_thresholds=REFERENCE_SPA_THRESHOLDS, tem_thresholds=REFERENCE_TEM_THRESHOLDS,
                       repeats=5, **overrides):
    """monitor_cost over the reference's thresholds, monitors, high tiers
    and presets (snowflake/monitor_independent_withmonitor.py), and the
    per-threshold percentage from the preset-mean times
    (snowflake/monitor_percent.py:11-21).  Returns (rows, table)."""
    stream = _stream()
    rows = []
    for high in high_tiers:
        for monitor, thresholds in ((A.MONITOR_SPA, spa_thresholds), (A.MONITOR_TEM, tem_thresholds)):
            for thr in thresholds:
                for preset in presets:
                    base = A.Params.preset(model, preset, **overrides).replace(high_tier=high)
                    c = monitor_cost(_mixed(base, monitor, thr), steps, repeats=repeats, stream=stream)
                    rows.append(dict({"model": model, "high": TIER_NAMES[high], "monitor": monitor,
                                      "threshold": float(thr), "preset": preset}, **c))
    table = []
    for (model, high, monitor, thr), v in _group(rows, ("model", "high", "monitor", "threshold")).items():
        tw = np.mean([r["ms_with"] for r in v])
        to = np.mean([r["ms_without"] for r in v])
        table.append({"model": model, "high": high, "monitor": monitor, "threshold": thr,
                      "monitor_percentage": float((tw - to) / tw * 100.0)})
    return rows, table


def _neighbour(t, direction, ntx, nty):
    """Tile index of one of the 8 periodic neighbours, directions 1..8 as in
    snowflake/tools.h:82-106 (left, right, down, up, then the diagonals)."""
    x, y = t % ntx, t // ntx
    dx, dy = {1: (-1, 0), 2: (1, 0), 3: (0, -1), 4: (0, 1),
              5: (-1, -1), 6: (1, -1), 7: (1, 1), 8: (-1, 1)}[direction]
    return (y + dy) % nty * ntx + (x + dx) % ntx


def oracle_tile_selection(metric, ratio, high_tier=A.TIER_FP64):
    """The motivation experiment's tile choice (snowflake/motivation_mix.cu:
    84-109): n - n*ratio tiles (truncated) stay at the high tier, taken first
    in descending order of the monitor metric (a stable order: the
    reference's bubble sort keeps ties in tile order) while the metric is
    non-zero, then by breadth-first growth over the 8 periodic neighbours of
    the chosen tiles, in choice order.  As in the reference, the first chosen
    tile is always marked, and the growth marks a neighbour before testing
    the quota.  A NaN metric ranks first (the reference's comparisons leave
    NaN order undefined).  metric: [nty][ntx]; returns tiers [nty][ntx]."""
    m = np.asarray(metric, dtype=np.float64)
    if m.ndim != 2:
        raise ValueError("metric must be [nty][ntx]")
    nty, ntx = m.shape
    flat = np.where(np.isnan(m), np.inf, m).ravel()
    n = flat.size
    quota = int(n - n * float(ratio))
    tiers = np.full(n, A.TIER_HALF, dtype=np.uint8)
    order = np.argsort(-flat, kind="stable")
    chosen = 0
    queue = deque()
    for t in order:
        if flat[t] == 0:
            break
        tiers[t] = high_tier
        chosen += 1
        queue.append(int(t))
        if chosen >= quota:
            break
    while queue:
        c = queue.popleft()
        for d in range(1, 9):
            nb = _neighbour(c, d, ntx, nty)
            if tiers[nb] != high_tier:
                chosen += 1
                tiers[nb] = high_tier
                queue.append(nb)
                if chosen >= quota:
                    break
        if chosen >= quota:
            break
    return tiers.reshape(nty, ntx)


def motivation(model, preset, steps, ratio, strategy="AMSTENCIL", monitor=A.MONITOR_SPA, high_tier=A.TIER_FP64,
               extra_steps=50, stream=None, **overrides):
    """One motivation run (snowflake/motivation_mix.cu, motivation_pure.py,
    motivationerror.py): `steps` plain high-precision steps from the
    reference initial state, then `extra_steps` steps at a fixed tier map --
    AMSTENCIL: oracle_tile_selection of the monitor metric measured at that
    point (the temporal metric against the state 9 steps earlier, the
    reference's copy at step steps-10); GRAM1 / GRAM2: the static ratio map
    -- and the error of the output field against `steps + extra_steps` plain
    steps.  Returns {"error", "low_share", "tiers"}."""
    stream = stream or _stream()
    base = A.Params.preset(model, preset, **overrides).replace(high_tier=high_tier)
    with A.Simulation(base.replace(mode=A.PUREHIGH)) as s:
        s.set_stream(stream.cuda_stream)
        s.init(A.INIT_REFERENCE)
        if strategy == "AMSTENCIL" and monitor == A.MONITOR_TEM:
            s.run(max(steps - 9, 0))
            s.store_temporal_reference()
            s.run(min(steps, 9))
        else:
            s.run(steps)
        metric = s.measure_tiles(monitor) if strategy == "AMSTENCIL" else None
        state = s.fields()
        s.run(extra_steps)
        pure = s.field(OUTPUT_FIELD[base.model])
    if strategy == "AMSTENCIL":
        # every tile at the high tier (the state keeps its precision), then the chosen map
        mode, gram = A.GRAM1, 0.0
    elif strategy in ("GRAM1", "GRAM2"):
        mode, gram = (A.GRAM1 if strategy == "GRAM1" else A.GRAM2), float(ratio)
    else:
        raise ValueError(f"unknown strategy {strategy!r}")
    with A.Simulation(base.replace(mode=mode, gram_ratio=gram)) as s:
        s.set_stream(stream.cuda_stream)
        s.set_fields(state)
        if metric is not None:
            s.set_tiers(oracle_tile_selection(metric, ratio, high_tier))
        tiers = s.tiers()
        s.run(extra_steps)
        out = s.field(OUTPUT_FIELD[base.model])
    return {"error": mean_abs_error(out, pure), "low_share": float(np.mean(tiers == A.TIER_HALF)), "tiers": tiers}


def motivation_sweep(model, presets=(1, 2, 3, 4, 5), step_counts=MOTIVATION_STEPS, ratios=MOTIVATION_RATIOS,
                     strategies=("AMSTENCIL", "GRAM1", "GRAM2"), monitors=(A.MONITOR_SPA, A.MONITOR_TEM),
                     **overrides):
    """motivation() over presets, step counts, ratios, strategies and
    monitors (snowflake/motivation_mix.py), with the preset-mean error per
    (strategy, monitor, steps, ratio) (motivationerror.py:14-40).  Returns
    (rows, table)."""
    stream = _stream()
    rows = []
    for strategy in strategies:
        for monitor in (monitors if strategy == "AMSTENCIL" else (0,)):
            for steps in step_counts:
                for ratio in ratios:
                    for preset in presets:
                        r = motivation(model, preset, steps, ratio, strategy=strategy,
                                       monitor=monitor or A.MONITOR_SPA, stream=stream, **overrides)
                        rows.append({"model": model, "strategy": strategy, "monitor": monitor, "timestep": steps,
                                     "ratio": ratio, "preset": preset, "error": r["error"],
                                     "low_share": r["low_share"]})
    table = [{"model": k[0], "strategy": k[1], "monitor": k[2], "timestep": k[3], "ratio": k[4],
              "avg_error": float(np.mean([r["error"] for r in v]))}
             for k, v in _group(rows, ("model", "strategy", "monitor", "timestep", "ratio")).items()]
    return rows, table


def main(argv=None):
    """Command line: one experiment, CSV files under --out."""
    ap = argparse.ArgumentParser(prog="python -m w3914777_gb300.experiments", description=__doc__.split("\n")[0])
    ap.add_argument("experiment", choices=["end2end", "monitor", "motivation"])
    ap.add_argument("--model", default="kobayashi", choices=["kobayashi", "graingrowth", "sintering"])
    ap.add_argument("--presets", type=int, nargs="+", default=[1, 2, 3, 4, 5])
    ap.add_argument("--high", nargs="+", default=["double", "float"], choices=["double", "float"])
    ap.add_argument("--steps", type=int, nargs="+", default=None,
                    help="steps per run (end2end, monitor: one value, default 500; motivation: the step counts)")
    ap.add_argument("--spa-thresholds", type=float, nargs="+", default=REFERENCE_SPA_THRESHOLDS)
    ap.add_argument("--tem-thresholds", type=float, nargs="+", default=REFERENCE_TEM_THRESHOLDS)
    ap.add_argument("--ratios", type=float, nargs="+", default=None)
    ap.add_argument("--repeats", type=int, default=5)
    ap.add_argument("--out", default="experiments_out")
    a = ap.parse_args(argv)
    highs = [A.TIER_FP64 if h == "double" else A.TIER_FP32 for h in a.high]
    written = []
    if a.experiment == "end2end":
        rows = end2end_sweep(a.model, a.presets, highs, (a.steps or [500])[0], a.spa_thresholds, a.tem_thresholds,
                             a.ratios or REFERENCE_RATIOS, repeats=a.repeats)
        written.append(write_csv(rows, os.path.join(a.out, f"{a.model}_end2end_runs.csv")))
        written.append(write_csv(speedup_table(rows), os.path.join(a.out, f"{a.model}_speedup.csv")))
        written.append(write_csv(error_table(rows), os.path.join(a.out, f"{a.model}_error.csv")))
    elif a.experiment == "monitor":
        rows, table = monitor_cost_sweep(a.model, a.presets, highs, (a.steps or [500])[0], a.spa_thresholds,
                                         a.tem_thresholds, repeats=a.repeats)
        written.append(write_csv(rows, os.path.join(a.out, f"{a.model}_monitor_runs.csv")))
        written.append(write_csv(table, os.path.join(a.out, f"{a.model}_monitor_percentage.csv")))
    else:
        rows, table = motivation_sweep(a.model, a.presets, a.steps or MOTIVATION_STEPS, a.ratios or MOTIVATION_RATIOS)
        written.append(write_csv(rows, os.path.join(a.out, f"{a.model}_motivation_runs.csv")))
        written.append(write_csv(table, os.path.join(a.out, f"{a.model}_motivation_error.csv")))
    print(json.dumps({"experiment": a.experiment, "model": a.model, "files": written}))


if __name__ == "__main__":
    main()
