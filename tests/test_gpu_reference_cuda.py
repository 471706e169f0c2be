"""The reference's own CUDA kernels run on the same GPU (baseline/_ref: its
device code built from its sources for sm_103a, driven by baseline/ref_cuda.cpp's
restatement of its host time loops), against its CPU build and against the
library.  Skipped where the cubins are not built (they need the reference
tree, and travel with the working copy to the GPU).

What is pinned:
  * the reference's GPU plain grain growth equals its CPU build (the goldens
    of tests/golden/) to the rounding of fused multiply-adds;
  * the reference's GPU AMSTENCIL grain growth (graingrowth/end2end_mix.cu) makes
    the same tier decision in every period as the library's reference mode
    (half_arith = AMPS_HALF_REF, ref_snapshot = 1), with fields equal to 1e-15;
  * the reference's GPU AMSTENCIL Kobayashi dendrite (snowflake/end2end_mix.cu,
    whose half tiles call the device-only h2cos/h2sin) makes the same tier
    decision in every period as the library's mixed mode at the same monitor
    and threshold (the library's half tiles compute in FP32, the reference's
    in half2).  Mixed-vs-own-FP64 error after 500 steps, to-nearest storage:
    mean and max |d phi| below the reference's at three of the four settings,
    within 1.9x / 2.7x at Monitor2 1e-2 (bars 2.5x / 3x); at the dendrite's
    centre (T ~ 1.1, a half's ulp 2^-10) T's small diffusive increments round
    away and max |d T| is ~3x the reference's.  With stochastic rounding of
    the half stores (half_arith = AMPS_HALF_SR) the mean |d phi| and |d T| --
    the reference's error metric -- are below the reference's at every
    setting (asserted);
  * sintering (sintering/main.cu, para5): the reference's GPU plain run from
    the library's reference initial state equals its CPU build to 1e-7 after
    40 steps, and its GPU AMSTENCIL run makes the library's reference-mode
    decisions in the first five periods.  Later periods part: this run is
    chaotic (a one-ulp change grows ~1.5x per step), and the reference's GPU
    build (CUDA's pow, fused multiply-adds) parts from its own CPU build in
    the same way."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

refcuda = pytest.importorskip("baseline.refcuda")


def amps():
    from w3914777_gb300 import amps as w
    return w


def need(*names):
    for n in names:
        if not refcuda.available(n):
            pytest.skip(f"baseline/_ref/{n}.cubin not built (needs the reference tree)")


GOLD = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden")


def test_reference_gpu_plain_graingrowth_equals_its_cpu_build():
    need("graingrowth_pure")
    g = np.load(f"{GOLD}/graingrowth_ref.npz")
    e1, e2, _ = refcuda.gg_pure(int(g["steps"]))
    d = max(float(np.abs(e1 - g["eta1"]).max()), float(np.abs(e2 - g["eta2"]).max()))
    print(f"reference GPU vs its CPU build, grain growth {int(g['steps'])} steps: {d:.3e}")
    assert d <= 1e-15


@pytest.mark.parametrize("monitor,thr", [(2, 1e-4), (1, 0.5)])
def test_reference_gpu_amstencil_graingrowth_decisions_equal_ours(monitor, thr):
    need(f"graingrowth_mix_m{monitor}")
    w = amps()
    steps = 500
    e1, e2, types, _ = refcuda.gg_mix(steps, thr, monitor)
    p = w.Params.preset("graingrowth", 1, mode="end2end_mix", monitor=monitor, monitor_samples=0, monitor_field=1,
                        thr_lo=thr, thr_hi=thr, ref_order=1, half_arith=w.HALF_REF, ref_snapshot=1, max_log=64)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
        log = s.decision_log()
    ours = np.where(log.reshape(log.shape[0], -1) == w.TIER_HALF, 1, 2)
    bad = [i for i in range(types.shape[0]) if not np.array_equal(ours[i], types[i])]
    d = max(float(np.abs(f[0] - e1).max()), float(np.abs(f[1] - e2).max()))
    print(f"grain growth monitor {monitor} {thr:g}: periods differing {bad[:5]}, fields {d:.3e}")
    assert not bad
    assert d <= 1e-15


@pytest.mark.parametrize("monitor,thr", [(1, 0.5), (1, 0.1), (2, 1e-4), (2, 1e-2)])
def test_reference_gpu_amstencil_kobayashi_decisions_and_envelope(monitor, thr):
    need("snowflake_pure", f"snowflake_mix_m{monitor}")
    w = amps()
    steps = 500
    rp, rt, _ = refcuda.kob_pure(steps)
    mp, mt, types, _ = refcuda.kob_mix(steps, thr, monitor)
    q = w.Params.preset("kobayashi", 2, mode="purehigh", ref_order=1)
    with w.Simulation(q, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        op = s.fields()
    ref_err = [float(np.abs(mp - rp).mean()), float(np.abs(mp - rp).max()), float(np.abs(mt - rt).mean()),
               float(np.abs(mt - rt).max())]
    # the plain FP64 runs agree (the reference's seed is symmetric and
    # ill-conditioned: ulps of atan2 grow to ~1e-7 by step 500)
    assert float(np.abs(op[0] - rp).max()) <= 1e-5
    errs = {}
    for name, ha in (("nearest", w.HALF_FP32), ("stochastic", w.HALF_SR)):
        p = w.Params.preset("kobayashi", 2, mode="end2end_mix", monitor=monitor, monitor_samples=0, monitor_field=0,
                            thr_lo=thr, thr_hi=thr, ref_order=1, max_log=64, half_arith=ha)
        with w.Simulation(p, init=w.INIT_REFERENCE) as s:
            s.run(steps)
            f = s.fields()
            log = s.decision_log()
        ours = np.where(log.reshape(log.shape[0], -1) == w.TIER_HALF, 1, 2)
        bad = [i for i in range(types.shape[0]) if not np.array_equal(ours[i], types[i])]
        assert not bad, (name, bad)
        errs[name] = [float(np.abs(f[0] - op[0]).mean()), float(np.abs(f[0] - op[0]).max()),
                      float(np.abs(f[1] - op[1]).mean()), float(np.abs(f[1] - op[1]).max())]
    print(f"kobayashi monitor {monitor} {thr:g}: decisions equal; mixed vs FP64 (mean phi, max phi, mean T, max T) "
          f"reference {np.array(ref_err)} nearest {np.array(errs['nearest'])} stochastic {np.array(errs['stochastic'])}")
    rn, sr = errs["nearest"], errs["stochastic"]
    assert rn[0] <= ref_err[0] * 2.5 and rn[1] <= ref_err[1] * 3.0
    # the reference's error metric, the mean |d f| over the grid
    # (snowflake/end2enderror.py): stochastic rounding within the reference's
    # own envelope for both fields; the max within 3.5x (one ulp of a
    # stochastically rounded cell)
    assert sr[0] <= ref_err[0] and sr[2] <= ref_err[2]
    assert sr[1] <= ref_err[1] * 3.5 and sr[3] <= ref_err[3] * 3.5


def test_reference_gpu_plain_sintering_equals_its_cpu_build():
    need("sintering_pure")
    w = amps()
    g = np.load(f"{GOLD}/sintering_ref.npz")
    f0 = w.init_host(w.Params.preset("sintering", 5, mode="purehigh", ref_order=1), w.INIT_REFERENCE)
    c, e1, e2, _ = refcuda.sint_pure(int(g["steps"]), f0[0], f0[1], f0[2])
    d = [float(np.abs(c - g["c"]).max()), float(np.abs(e1 - g["eta1"]).max()), float(np.abs(e2 - g["eta2"]).max())]
    print(f"reference GPU vs its CPU build, sintering {int(g['steps'])} steps: {d}")
    assert max(d) <= 1e-7


@pytest.mark.parametrize("monitor,thr", [(2, 1e-4), (1, 0.5), (2, 1e-2)])
def test_reference_gpu_amstencil_sintering_early_decisions_equal_ours(monitor, thr):
    need("sintering_mix")
    w = amps()
    steps = 50
    p = w.Params.preset("sintering", 5, mode="end2end_mix", monitor=monitor, monitor_samples=0, monitor_field=0,
                        thr_lo=thr, thr_hi=thr, ref_order=1, half_arith=w.HALF_REF, max_log=64)
    f0 = w.init_host(p, w.INIT_REFERENCE)
    _, _, _, types, _ = refcuda.sint_mix(steps, thr, monitor, f0[0], f0[1], f0[2])
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        log = s.decision_log()
    ours = np.where(log.reshape(log.shape[0], -1) == w.TIER_HALF, 1, 2)
    bad = [i for i in range(types.shape[0]) if not np.array_equal(ours[i], types[i])]
    print(f"sintering monitor {monitor} {thr:g}: half tiles {int((types[-1] == 1).sum())}, periods differing {bad}")
    assert not bad
