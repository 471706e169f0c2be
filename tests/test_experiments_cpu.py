"""Host logic of the experiment drivers (w3914777_gb300/experiments.py): the
oracle tile selection against a literal restatement of the reference's
host loop (snowflake/motivation_mix.cu:84-109 with the bubble sort and
periodic neighbours of snowflake/tools.h:67-106), the error metric, the
speedup / error / monitor tables and the CSV writer.  No GPU."""
import csv

import numpy as np
import pytest

from w3914777_gb300 import amps, experiments as E


def reference_selection(metric, ratio, ntx, nty):
    """The reference's selection, loop for loop (1 = low, 2 = high)."""
    n = ntx * nty
    p = list(metric)
    ind = list(range(n))
    for i in range(n):  # BubbleSort: descending, swaps only on strict <
        for j in range(n - i - 1):
            if p[j] < p[j + 1]:
                p[j], p[j + 1] = p[j + 1], p[j]
                ind[j], ind[j + 1] = ind[j + 1], ind[j]

    def neighbour(index, direct):
        x, y = index % ntx, index // ntx
        if direct == 1: x = (x - 1 + ntx) % ntx
        if direct == 2: x = (x + 1) % ntx
        if direct == 3: y = (y - 1 + nty) % nty
        if direct == 4: y = (y + 1) % nty
        if direct == 5: x, y = (x - 1 + ntx) % ntx, (y - 1 + nty) % nty
        if direct == 6: x, y = (x + 1) % ntx, (y - 1 + nty) % nty
        if direct == 7: x, y = (x + 1) % ntx, (y + 1) % nty
        if direct == 8: x, y = (x - 1 + ntx) % ntx, (y + 1) % nty
        return y * ntx + x

    quota = int(n - n * ratio)
    total = 0
    type_new = [1] * n
    queue = []
    j = 0
    while j < n and p[j] != 0:
        type_new[ind[j]] = 2
        total += 1
        queue.append(ind[j])
        if total >= quota:
            break
        j += 1
    while queue:
        c = queue.pop(0)
        for d in range(1, 9):
            nb = neighbour(c, d)
            if type_new[nb] != 2:
                total += 1
                type_new[nb] = 2
                queue.append(nb)
                if total >= quota:
                    break
        if total >= quota:
            break
    return np.array(type_new).reshape(nty, ntx)


@pytest.mark.parametrize("seed", range(12))
def test_oracle_tile_selection_matches_reference_loop(seed):
    rng = np.random.default_rng(seed)
    nty, ntx = [(4, 4), (5, 7), (8, 8), (3, 11)][seed % 4]
    n = ntx * nty
    # ties, zeros and a spread of values
    metric = rng.choice([0.0, 0.0, 0.1, 0.2, 0.2, 0.5, 1.0], size=n) * rng.choice([1.0, 1e-3], size=n)
    if seed % 3 == 0:
        metric = rng.random(n)  # all non-zero
    for ratio in (0.0, 0.1, 0.25, 0.5, 0.77, 0.9, 1.0):
        ref = reference_selection(metric, ratio, ntx, nty)
        got = E.oracle_tile_selection(metric.reshape(nty, ntx), ratio, amps.TIER_FP64)
        assert np.array_equal(got == amps.TIER_FP64, ref == 2), (ratio, got, ref)
        assert np.array_equal(got == amps.TIER_HALF, ref == 1)


def test_oracle_tile_selection_quirks():
    m = np.zeros((4, 4))
    m[1, 1] = 3.0
    # ratio 1: the quota is 0, yet the top tile and one grown neighbour are marked
    t = E.oracle_tile_selection(m, 1.0)
    assert (t == amps.TIER_FP64).sum() == 2 and t[1, 1] == amps.TIER_FP64 and t[1, 0] == amps.TIER_FP64
    # an all-zero metric selects nothing
    assert (E.oracle_tile_selection(np.zeros((4, 4)), 0.0) == amps.TIER_HALF).all()
    # growth wraps around the periodic edges
    m = np.zeros((4, 4))
    m[0, 0] = 1.0
    t = E.oracle_tile_selection(m, 0.5)
    assert t[0, 3] == amps.TIER_FP64 and t[3, 0] == amps.TIER_FP64 and t[3, 3] == amps.TIER_FP64
    # FP32 as the high tier; NaN ranks first
    m = np.array([[0.5, np.nan], [0.0, 0.0]])
    t = E.oracle_tile_selection(m, 0.75, amps.TIER_FP32)
    assert t[0, 1] == amps.TIER_FP32 and set(np.unique(t)) <= {amps.TIER_HALF, amps.TIER_FP32}


def test_mean_abs_error_is_the_reference_metric():
    a = np.zeros((2, 3))
    b = np.array([[1.0, -2.0, 0.0], [0.0, 0.0, 3.0]])
    assert E.mean_abs_error(a, b) == 1.0
    with pytest.raises(ValueError):
        E.mean_abs_error(a, b[:, :2])


def _rows():
    rows = []
    for preset, pure_ms in ((1, 10.0), (2, 30.0)):
        common = {"model": "kobayashi", "high": "double", "preset": preset}
        rows.append(dict(common, strategy="PURE", monitor=0, param=0.0, ms=pure_ms, error=0.0, low_share=0.0))
        rows.append(dict(common, strategy="AMSTENCIL", monitor=1, param=0.1, ms=pure_ms / 2, error=preset * 1e-4,
                         low_share=0.5))
        rows.append(dict(common, strategy="GRAM1", monitor=0, param=0.5, ms=pure_ms / 4, error=preset * 1e-3,
                         low_share=0.5))
    return rows


def test_speedup_and_error_tables(tmp_path):
    rows = _rows()
    sp = {(r["strategy"], r["param"]): r["speedup"] for r in E.speedup_table(rows)}
    # mean PURE time (20) over the mean strategy time (10 and 5)
    assert sp[("AMSTENCIL", 0.1)] == pytest.approx(2.0) and sp[("GRAM1", 0.5)] == pytest.approx(4.0)
    er = {(r["strategy"], r["param"]): r["avg_error"] for r in E.error_table(rows)}
    assert er[("AMSTENCIL", 0.1)] == pytest.approx(1.5e-4) and er[("GRAM1", 0.5)] == pytest.approx(1.5e-3)
    path = E.write_csv(rows, str(tmp_path / "sub" / "runs.csv"))
    with open(path) as f:
        back = list(csv.DictReader(f))
    assert len(back) == len(rows) and float(back[1]["ms"]) == rows[1]["ms"]
    with pytest.raises(ValueError):
        E.write_csv([], str(tmp_path / "x.csv"))


def test_experiment_constants_follow_the_reference_sweeps():
    assert len(E.REFERENCE_SPA_THRESHOLDS) == 30 and len(E.REFERENCE_TEM_THRESHOLDS) == 30
    assert E.REFERENCE_RATIOS[0] == 0.01 and E.REFERENCE_RATIOS[-1] == 1.0 and len(E.REFERENCE_RATIOS) == 100
    assert E.OUTPUT_FIELD == {amps.KOBAYASHI: 0, amps.GRAINGROWTH: 1, amps.SINTERING: 0}


def test_monitor_cost_rejects_static_modes():
    p = amps.Params.preset("kobayashi", 1)  # purehigh
    with pytest.raises(ValueError):
        E.monitor_cost(p, 20)
