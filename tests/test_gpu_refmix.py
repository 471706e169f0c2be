"""The library's reference-faithful mixed mode against the reference's own
adaptive grain-growth runs (AMSTENCIL, graingrowth/end2end_mix.cu), which
tests/golden/make_golden_mix.py executed on the CPU from the reference's
kernels (oracle/_ref/libref_ggmix_m*.so) into
tests/golden/graingrowth_mix_ref.npz.

The mode: end2end_mix with two tiers at the reference's threshold,
ref_order=1 (FP64 tiles in the reference's expression order),
half_arith=AMPS_HALF_REF (half tiles in binary16, every operation rounded in
the reference's order, graingrowth/function.h:163-166) and ref_snapshot=1
(the temporal monitor's snapshot as the reference keeps it).

Bars, per run of 500 steps at the reference's para1 (512^2, 16^2 tiles):
  * tier decisions: every period's map equals the reference's type_curr;
  * fields: equal to the reference's final fields to 1e-12 (the FP64 tiles
    call the device pow(), the reference's CPU build glibc's: an ulp apart
    at most per call);
  * error: the run's mean and max |mixed - plain FP64| per field (the
    reference's error metric, graingrowth/end2enderror.py:34) at most the
    reference's own mixed-vs-FP64 error + 1e-12.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "graingrowth_mix_ref.npz")


def amps():
    import w3914777_gb300 as w
    return w


def _gold():
    return np.load(GOLD)


def _runs():
    return [(int(m), float(t)) for m, t in np.load(GOLD)["runs"]]


def _key(monitor, thr):
    return f"m{monitor}_{thr:g}"


def _params(w, monitor, thr, half_arith):
    return w.Params.preset("graingrowth", 1, mode="end2end_mix", monitor=monitor, monitor_samples=0,
                           monitor_field=1, thr_lo=thr, thr_hi=thr, ref_order=1, half_arith=half_arith,
                           ref_snapshot=1, max_log=64)


_pure_cache = {}


def _pure(w, steps):
    if steps not in _pure_cache:
        p = w.Params.preset("graingrowth", 1, mode="purehigh", ref_order=1)
        with w.Simulation(p, init=w.INIT_REFERENCE) as s:
            s.run(steps)
            _pure_cache[steps] = s.fields()
    return _pure_cache[steps]


@pytest.mark.parametrize("monitor,thr", _runs())
def test_reference_mixed_run_decisions_fields_and_error(monitor, thr):
    w = amps()
    g = _gold()
    k = _key(monitor, thr)
    steps = int(g["steps"])
    with w.Simulation(_params(w, monitor, thr, w.HALF_REF), init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
        log = s.decision_log()
        st = s.stats()
    ref_types = g[k + "_types"]
    ours = np.where(log.reshape(log.shape[0], -1) == w.TIER_HALF, 1, 2).astype(np.uint8)
    # the resting classification and one per period: the reference classifies at steps 0, 10, ..., 490
    assert ours.shape[0] >= ref_types.shape[0]
    bad = [i for i in range(ref_types.shape[0]) if not np.array_equal(ours[i], ref_types[i])]
    print(f"{k}: half tiles first/last period {int((ours[0] == 1).sum())}/{int((ours[ref_types.shape[0] - 1] == 1).sum())}"
          f", periods differing from the reference: {bad[:5]}, tile-steps {st['tile_steps']}")
    assert not bad
    if k + "_eta2" in g.files:
        e = max(float(np.abs(f[0] - g[k + "_eta1"]).max()), float(np.abs(f[1] - g[k + "_eta2"]).max()))
        print(f"{k}: fields vs the reference's mixed run: {e:.3e}")
        assert e <= 1e-12
    pure = _pure(w, steps)
    d1, d2 = np.abs(f[0] - pure[0]), np.abs(f[1] - pure[1])
    ours_err = np.array([d1.mean(), d2.mean(), d1.max(), d2.max()])
    ref_err = g[k + "_err"]
    print(f"{k}: error vs plain FP64 (mean eta1, eta2, max eta1, eta2): ours {ours_err}, reference {ref_err}")
    assert np.all(ours_err <= ref_err + 1e-12)


@pytest.mark.parametrize("monitor,thr", [(2, 1e-2), (1, 0.5)])
def test_hfma2_half_tiles_rerun_and_error(monitor, thr):
    """half_arith=AMPS_HALF_HFMA2 (packed fused multiply-adds on the half
    tiles): a rerun is bit-identical, and the error against plain FP64 stays
    within 4x the reference's own half2 error at the same threshold (the
    fused form rounds fewer times, but differently)."""
    w = amps()
    g = _gold()
    k = _key(monitor, thr)
    steps = int(g["steps"])
    out = []
    for _ in range(2):
        with w.Simulation(_params(w, monitor, thr, w.HALF_HFMA2), init=w.INIT_REFERENCE) as s:
            s.run(steps)
            out.append((s.fields(), s.decision_log()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    pure = _pure(w, steps)
    f = out[0][0]
    d2 = np.abs(f[1] - pure[1])
    ref_err = g[k + "_err"]
    print(f"{k} HFMA2: mean |d eta2| {d2.mean():.3e} (reference half2 {ref_err[1]:.3e}), max {d2.max():.3e} "
          f"(reference {ref_err[3]:.3e})")
    assert d2.mean() <= 4 * ref_err[1] + 1e-12 and d2.max() <= 4 * ref_err[3] + 1e-12


SINT_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sintering_mix_ref.npz")


def _sint_runs():
    return [(int(m), float(t)) for m, t in np.load(SINT_GOLD)["runs"]]


_sint_pure_cache = {}


@pytest.mark.parametrize("monitor,thr", _sint_runs())
def test_reference_mixed_sintering_decisions_fields_and_error(monitor, thr):
    """Sintering in the reference's own mixed arithmetic (half_arith =
    AMPS_HALF_REF: the chemical potential at each cell's owner tier, half
    tiles in binary16 in the reference's order) against the reference's
    AMSTENCIL runs on the CPU (tests/golden/sintering_mix_ref.npz; para5,
    512^2, 16^2 tiles, 500 steps).  Both sides take pow(x, 3) as the
    correctly rounded cube: this run amplifies a one-ulp difference about
    1.5x per step, so any other cube (the C library's, CUDA's) moves the
    decisions within ~100 steps.  Bars: every period's tier map equals the
    reference's type_con; the final c, eta1, eta2 equal the reference's bit
    for bit; the max |mixed - plain FP64| per field equals the reference's,
    the mean agrees to 1e-12 (numpy's summation order on each machine)."""
    w = amps()
    g = np.load(SINT_GOLD)
    k = _key(monitor, thr)
    steps = int(g["steps"])
    p = w.Params.preset("sintering", 5, mode="end2end_mix", monitor=monitor, monitor_samples=0, monitor_field=0,
                        thr_lo=thr, thr_hi=thr, ref_order=1, half_arith=w.HALF_REF, max_log=64)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
        log = s.decision_log()
        st = s.stats()
    ref_types = g[k + "_types"]
    ours = np.where(log.reshape(log.shape[0], -1) == w.TIER_HALF, 1, 2).astype(np.uint8)
    bad = [i for i in range(ref_types.shape[0]) if not np.array_equal(ours[i], ref_types[i])]
    print(f"sintering {k}: half tiles first/last period {int((ours[0] == 1).sum())}/"
          f"{int((ours[ref_types.shape[0] - 1] == 1).sum())}, periods differing: {bad[:5]}, tiles {st['tile_steps']}")
    assert not bad
    if k + "_c" in g.files:
        e = max(float(np.abs(f[i] - g[k + n]).max()) for i, n in enumerate(("_c", "_eta1", "_eta2")))
        print(f"sintering {k}: fields vs the reference's mixed run: {e:.3e}")
        assert e == 0.0
    if steps not in _sint_pure_cache:
        q = w.Params.preset("sintering", 5, mode="purehigh", ref_order=1)
        with w.Simulation(q, init=w.INIT_REFERENCE) as s:
            s.run(steps)
            _sint_pure_cache[steps] = s.fields()
    pure = _sint_pure_cache[steps]
    d = [np.abs(f[i] - pure[i]) for i in range(3)]
    ours_err = np.array([x.mean() for x in d] + [x.max() for x in d])
    print(f"sintering {k}: error vs plain FP64: ours {ours_err}, reference {g[k + '_err']}")
    # the maxima bit for bit; the means within numpy's summation order
    assert np.array_equal(ours_err[3:], g[k + "_err"][3:])
    np.testing.assert_allclose(ours_err[:3], g[k + "_err"][:3], rtol=1e-12, atol=0)
