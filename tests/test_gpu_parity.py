"""GPU parity: the CUDA path (through the C ABI) against the CPU FP64 oracle
and against the reference's own outputs (tests/golden/).

Tolerances, written per test:
  * FP64 tiles in reference order (ref_order=1) -- the plain FP64 parity path:
    every +,-,*,/ is rounded as the reference writes it, so the only source
    of difference is the device libm (atan2/cos/sin/atan/pow(x,3)) against
    glibc, at most a few ulp per call.  Bar: max |gpu - ref| <= 1e-12 *
    max|ref| after N steps.
  * FP32 tiles: 1e-4 * max|ref| after N steps.
  * half tiles (purelow) and mixed runs: envelopes stated in each test.
"""
import os

import numpy as np
import pytest

import oracle_bind as ob

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def amps():
    import w3914777_gb300 as w
    return w


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ------------------------------------------------------------- golden ----
def test_kobayashi_fp64_matches_reference_golden():
    """The reference's own parameters and symmetric seed (snowflake/paras/para2.h,
    snowflake/tools.h:24-33).  Bar: <= 1e-12 relative at the early snapshot.
    Later, where the symmetric seed produces an exactly zero gradient, the
    reference's theta = atan2(phi_y, phi_x) (snowflake/function.h:32) is
    discontinuous and a one-ulp difference in the device libm makes theta
    arbitrary there; tests/test_oracle_conditioning.py shows the oracle itself
    moves by ~1e-4 under a one-ulp perturbation.  Bar after 40 steps: 1e-3
    relative (phi) / 1e-2 relative (T, whose magnitude is ~1e-3 of phi's)."""
    w = amps()
    g = np.load(os.path.join(GOLD, "kobayashi_ref.npz"))
    p = w.Params.preset("kobayashi", 2, mode="purehigh")
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(int(g["early"]))
        f8 = s.fields()
        s.run(int(g["steps"]) - int(g["early"]))
        f = s.fields()
    e8 = max(rel_err(f8[0], g["phi_early"]), rel_err(f8[1], g["T_early"]))
    e_phi, e_T = rel_err(f[0], g["phi"]), rel_err(f[1], g["T"])
    print(f"kobayashi fp64 vs reference: {int(g['early'])} steps {e8:.3e}; "
          f"{int(g['steps'])} steps phi {e_phi:.3e} T {e_T:.3e}")
    assert e8 <= 1e-12
    assert e_phi <= 1e-3 and e_T <= 1e-2


def test_kobayashi_fp64_reference_params_asymmetric_seed():
    """Reference parameters (para2) with a seed whose gradient never vanishes
    exactly: a disc plus a seeded 1e-3 perturbation.  Bar: <= 1e-12 after 40 steps."""
    w = amps()
    p = w.Params.preset("kobayashi", 2, mode="purehigh", nx=128, ny=128, init_offset=0, init_r2=60.0)
    f0 = w.init_host(p, w.INIT_REFERENCE)
    rng = np.random.default_rng(11)
    f0[0] += 1e-3 * rng.random(f0[0].shape)
    with w.Simulation(p) as s:
        s.set_fields(f0)
        s.run(40)
        f = s.fields()
    phi, T = ob.kob_run(ob.kob_params(128, 128), f0[0], f0[1], 40)
    e = max(rel_err(f[0], phi), rel_err(f[1], T))
    print(f"kobayashi para2 asymmetric seed, 40 steps: {e:.3e}")
    assert e <= 1e-12


def test_graingrowth_fp64_matches_reference_golden():
    w = amps()
    g = np.load(os.path.join(GOLD, "graingrowth_ref.npz"))
    p = w.Params.preset("graingrowth", 1, mode="purehigh")
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(int(g["steps"]))
        f = s.fields()
    e1, e2 = rel_err(f[0], g["eta1"]), rel_err(f[1], g["eta2"])
    print(f"graingrowth fp64 vs reference: {e1:.3e} {e2:.3e}")
    assert e1 <= 1e-12 and e2 <= 1e-12


def test_sintering_fp64_matches_reference_golden():
    w = amps()
    g = np.load(os.path.join(GOLD, "sintering_ref.npz"))
    p = w.Params.preset("sintering", 5, mode="purehigh")
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(int(g["steps"]))
        f = s.fields()
    errs = [rel_err(f[0], g["c"]), rel_err(f[1], g["eta1"]), rel_err(f[2], g["eta2"])]
    print("sintering fp64 vs reference:", errs)
    assert max(errs) <= 1e-12


# ------------------------------------------------- oracle, other cases ----
@pytest.mark.parametrize("tile", [16, 32])
@pytest.mark.parametrize("bc", [0, 1])
def test_kobayashi_fp64_vs_oracle_bc_tile_noise(tile, bc):
    """Zero-flux and periodic boundaries, 32x32 tiles, seeded noise; 96 x 64 grid."""
    w = amps()
    nx, ny, steps = 96, 64, 30
    p = w.Params.preset("kobayashi", 4, mode="purehigh", nx=nx, ny=ny, tile=tile, bc=bc, noise=0.01, seed=7,
                        init_offset=3, init_r2=40.0)
    f0 = w.init_host(p, w.INIT_REFERENCE)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
    q = ob.kob_params(nx, ny, bc=bc, aniso=p.aniso, theta0=p.theta0, noise=0.01, seed=7)
    phi, T = ob.kob_run(q, f0[0], f0[1], steps)
    e = max(rel_err(f[0], phi), rel_err(f[1], T))
    print(f"kobayashi tile={tile} bc={bc}: {e:.3e}")
    assert e <= 1e-12


@pytest.mark.parametrize("q,stencil,bc", [(2, 0, 0), (5, 0, 1), (3, 1, 0)])
def test_graingrowth_fp64_vs_oracle_q_general(q, stencil, bc):
    w = amps()
    nx, ny, steps = 64, 96, 25
    p = w.Params.preset("graingrowth", 0, mode="purehigh", nx=nx, ny=ny, nfields=q, stencil=stencil, bc=bc,
                        ref_order=1, dt=0.05, init_amp=0.3)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(steps)
        f = s.fields()
    o = ob.gg_run(ob.gg_params(nx, ny, q=q, bc=bc, stencil=stencil, dx=1.0, dy=1.0, dt=0.05, mobil=1.0,
                               grcoef=2.0, gamma=1.5), list(f0), steps)
    e = max(rel_err(f[k], o[k]) for k in range(q))
    print(f"graingrowth Q={q}: {e:.3e}")
    assert e <= 1e-12


@pytest.mark.parametrize("model,nx,ny,tile,bc", [
    ("graingrowth", 32, 32, 32, 0), ("graingrowth", 32, 32, 32, 1), ("graingrowth", 16, 16, 16, 0),
    ("graingrowth", 64, 32, 32, 0), ("graingrowth", 16, 48, 16, 1),
    ("kobayashi", 16, 16, 16, 0), ("kobayashi", 32, 32, 32, 1), ("kobayashi", 32, 64, 32, 0)])
def test_smallest_grids_fp64_vs_oracle(model, nx, ny, tile, bc):
    """Grids of one tile, or one tile across: every periodic neighbour of a
    tile is the tile itself (or its one partner), and the zero-flux mirror
    folds the halo back into it."""
    w = amps()
    steps = 20
    if model == "graingrowth":
        p = w.Params.preset("graingrowth", 0, mode="purehigh", nx=nx, ny=ny, tile=tile, nfields=3, bc=bc,
                            ref_order=1, dt=0.05, init_amp=0.3)
        f0 = w.init_host(p, w.INIT_SEEDED)
        with w.Simulation(p, init=w.INIT_SEEDED) as s:
            s.run(steps)
            f = s.fields()
        o = ob.gg_run(ob.gg_params(nx, ny, q=3, bc=bc, dx=1.0, dy=1.0, dt=0.05, mobil=1.0, grcoef=2.0, gamma=1.5),
                      list(f0), steps)
        e = max(rel_err(f[k], o[k]) for k in range(3))
    else:
        p = w.Params.preset("kobayashi", 4, mode="purehigh", nx=nx, ny=ny, tile=tile, bc=bc, noise=0.01, seed=7,
                            init_offset=1, init_r2=20.0)
        f0 = w.init_host(p, w.INIT_REFERENCE)
        with w.Simulation(p, init=w.INIT_REFERENCE) as s:
            s.run(steps)
            f = s.fields()
        q = ob.kob_params(nx, ny, bc=bc, aniso=p.aniso, theta0=p.theta0, noise=0.01, seed=7)
        phi, T = ob.kob_run(q, f0[0], f0[1], steps)
        e = max(rel_err(f[0], phi), rel_err(f[1], T))
    print(f"{model} {nx}x{ny} tile {tile} bc {bc}: {e:.3e}")
    assert e <= 1e-12


@pytest.mark.parametrize("nx,ny,tile,bc,ref_order", [(32, 32, 32, 0, 1), (32, 32, 32, 1, 0), (32, 32, 32, 0, 0),
                                                     (32, 64, 16, 0, 1)])
def test_smallest_grids_sintering_fp64_vs_oracle(nx, ny, tile, bc, ref_order):
    """Sintering on one tile (or one tile across): the chemical potential's
    2-cell halo wraps or mirrors into the tile itself."""
    w = amps()
    p = w.Params.preset("sintering", 0, mode="purehigh", nx=nx, ny=ny, tile=tile, nfields=2, rmin=3, rmax=5,
                        ref_order=ref_order, bc=bc)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(20)
        f = s.fields()
    op = ob.sint_params(nx, ny, n=2, coefm=p.coefm, coefk=p.coefk, coefl=p.coefl, dsur=p.dsur, bc=bc)
    c, e = ob.sint_run(op, f0[0], list(f0[1:]), 20)
    errs = [rel_err(f[0], c)] + [rel_err(f[k + 1], e[k]) for k in range(2)]
    print(f"sintering {nx}x{ny} tile {tile} bc {bc} ref {ref_order}:", errs)
    assert max(errs) <= 1e-12


@pytest.mark.parametrize("nx,ny,tile,monitor", [(32, 32, 32, 1), (32, 32, 16, 2), (64, 32, 32, 3)])
def test_smallest_grids_kobayashi_decisions_match_oracle(nx, ny, tile, monitor):
    """Kobayashi's per-tier kernels, monitor and classification on grids of
    one or two tiles across."""
    w = amps()
    thr = (0.3, 0.6) if monitor == 1 else (1e-4, 1e-2)
    p = w.Params.preset("kobayashi", 2, mode="end2end_mix", nx=nx, ny=ny, tile=tile, monitor=monitor,
                        monitor_samples=0, thr_lo=thr[0], thr_hi=thr[1], init_r2=40.0, init_offset=1, max_log=16)
    back = 1 if monitor == 3 else 10
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(50 - back)
        prev = s.fields()
        s.run(back)
        now = s.fields()
        m_gpu, t_gpu = s.metric(), s.tiers()
    m, t = _oracle_decisions(w, s, p, prev, now)
    assert np.array_equal(m_gpu, m)
    assert np.array_equal(t_gpu, t)


@pytest.mark.parametrize("nx,ny,bc", [(32, 32, 0), (64, 32, 1), (32, 96, 0)])
def test_smallest_grids_adaptive_decisions_match_oracle(nx, ny, bc):
    """The fused grain-growth step, its rate monitor and the classification
    on grids one tile wide or high."""
    w = amps()
    p = w.Params.preset("graingrowth", 0, nx=nx, ny=ny, nfields=4, bc=bc, monitor=w.MONITOR_RATE,
                        monitor_samples=1, thr_lo=1e-5, thr_hi=3e-3, max_log=16)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(39)
        prev = s.fields()
        s.run(1)
        now = s.fields()
        m_gpu, t_gpu, st = s.metric(), s.tiers(), s.stats()
    m, t = _oracle_decisions(w, s, p, prev, now)
    assert np.array_equal(m_gpu, m)
    assert np.array_equal(t_gpu, t)
    assert sum(st["tile_steps"]) == 40 * t.size


@pytest.mark.parametrize("ref_order,bc", [(1, 0), (0, 0), (0, 1)])
def test_sintering_fp64_vs_oracle_n_particles(ref_order, bc):
    """ref_order=0: the FMA-form FP64 tiles, computed in 8-row bands on
    non-monitor steps (zero flux: mirrored rings at the band edges)."""
    w = amps()
    nx = ny = 128
    p = w.Params.preset("sintering", 0, mode="purehigh", nx=nx, ny=ny, nfields=4, rmin=10, rmax=16,
                        ref_order=ref_order, bc=bc)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(20)
        f = s.fields()
    op = ob.sint_params(nx, ny, n=4, coefm=p.coefm, coefk=p.coefk, coefl=p.coefl, dsur=p.dsur, bc=bc)
    c, e = ob.sint_run(op, f0[0], list(f0[1:]), 20)
    errs = [rel_err(f[0], c)] + [rel_err(f[k + 1], e[k]) for k in range(4)]
    print("sintering N=4:", errs)
    assert max(errs) <= 1e-12


@pytest.mark.parametrize("model", ["graingrowth", "kobayashi"])
def test_fma_form_fp64_vs_oracle(model):
    """ref_order=0: the FP64 arithmetic in fused multiply-add form, which the
    seeded workloads' plain FP64 baselines run (their error yardstick).  It
    rounds differently from the reference's expression order, but it is the
    same update: <= 1e-12 relative to the oracle after 40 steps, on the
    seeded workloads' own settings (grain growth: the Fan-Chen Q=8 start,
    periodic; Kobayashi: the zero-flux dendrite with noise)."""
    w = amps()
    steps = 40
    if model == "graingrowth":
        p = w.Params.preset("graingrowth", 0, mode="purehigh", nx=128, ny=96, ref_order=0)
        f0 = w.init_host(p, w.INIT_SEEDED)
        with w.Simulation(p) as s:
            s.set_fields(f0)
            s.run(steps)
            f = s.fields()
        o = ob.gg_run(ob.gg_params(128, 96, q=8, dx=1.0, dy=1.0, dt=0.05, mobil=1.0, grcoef=2.0, gamma=1.5),
                      list(f0), steps)
        e = max(rel_err(f[k], o[k]) for k in range(8))
    else:
        p = w.Params.preset("kobayashi", 0, mode="purehigh", nx=128, ny=128, ref_order=0)
        f0 = w.init_host(p, w.INIT_SEEDED)
        with w.Simulation(p) as s:
            s.set_fields(f0)
            s.run(steps)
            f = s.fields()
        q = ob.kob_params(128, 128, bc=1, kappa=p.kappa, aniso=p.aniso, theta0=p.theta0, noise=p.noise,
                          seed=p.seed)
        phi, T = ob.kob_run(q, f0[0], f0[1], steps)
        e = max(rel_err(f[0], phi), rel_err(f[1], T))
    print(f"{model} FMA-form FP64 vs oracle after {steps} steps: {e:.3e}")
    assert e <= 1e-12


def _gram_map(mode, ntiles, ratio):
    """snowflake/function.h:72-79: GRAM1 marks tile t low when
    t < ntiles*ratio, GRAM2 when t % 100 < 100*ratio (t = blockIdx.z, the
    row-major tile index); 0 = half, 2 = high."""
    t = np.arange(ntiles)
    low = t < ntiles * ratio if mode == "gram1" else (t % 100) < 100 * ratio
    return np.where(low, 0, 2).astype(np.uint8)


@pytest.mark.parametrize("mode", ["gram1", "gram2"])
@pytest.mark.parametrize("ratio", [0.0, 0.3, 0.5, 0.77, 1.0])
def test_gram_static_maps_match_the_reference_rule(mode, ratio):
    """The GRAM1/GRAM2 static tier maps against an independent numpy
    statement of the reference's rule, on the reference's 512^2 grid of 16^2
    tiles (1024 tiles: not a multiple of 100, so GRAM2's last block is
    partial), and the run's tile-steps per tier follow the map."""
    w = amps()
    p = w.Params.preset("graingrowth", 1, mode=mode, gram_ratio=ratio)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(3)
        got = s.tiers().ravel()
        st = s.stats()
    want = _gram_map(mode, got.size, ratio)
    assert np.array_equal(got, want)
    assert st["tile_steps"][0] == 3 * int((want == 0).sum()) and st["tile_steps"][2] == 3 * int((want == 2).sum())


# --------------------------------------------------------- lower tiers ----
def test_fp32_high_tier_vs_oracle():
    w = amps()
    g = np.load(os.path.join(GOLD, "graingrowth_ref.npz"))
    p = w.Params.preset("graingrowth", 1, mode="purehigh", high_tier=w.TIER_FP32)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(int(g["steps"]))
        f = s.fields()
    e = max(rel_err(f[0], g["eta1"]), rel_err(f[1], g["eta2"]))
    print(f"graingrowth fp32 vs reference fp64: {e:.3e}")
    assert e <= 1e-4


def test_purelow_half_envelope():
    """All-half run (snowflake/purelow.cu): the half storage bounds the error."""
    w = amps()
    g = np.load(os.path.join(GOLD, "graingrowth_ref.npz"))
    p = w.Params.preset("graingrowth", 1, mode="purelow")
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(int(g["steps"]))
        f = s.fields()
    e = max(np.max(np.abs(f[0] - g["eta1"])), np.max(np.abs(f[1] - g["eta2"])))
    print(f"graingrowth half vs reference fp64: max abs {e:.3e}")
    assert e <= 2e-2


# --------------------------------------------------------------- mixed ----
def _oracle_decisions(w, s, p, state_prev, state_now):
    """Oracle get_type on the GPU's own stored state (snowflake/tools.h:177-230)."""
    T = p.tile
    fields = range(s.nf) if p.monitor_field < 0 else [p.monitor_field]
    m = None
    for k in fields:
        if p.monitor == w.MONITOR_SPA:
            mk = ob.monitor_spa(state_now[k], T, p.monitor_samples)
        elif p.monitor == w.MONITOR_RATE:
            mk = ob.monitor_rate(state_now[k], state_prev[k], T, p.cadence, p.monitor_samples)
        else:
            mk = ob.monitor_tem(state_now[k], state_prev[k], T, p.monitor_samples)
        m = mk if m is None else np.maximum(m, mk)
    thr_lo = p.thr_lo if p.high_tier == w.TIER_FP64 else p.thr_hi
    t = ob.classify(m, thr_lo, p.thr_hi)
    if p.high_tier == w.TIER_FP32:
        t = np.where(t == 2, 1, 0).astype(np.uint8)
    return m, t


@pytest.mark.parametrize("monitor,samples", [(1, 0), (2, 0), (1, 1), (2, 1), (3, 0), (3, 1)])
def test_mixed_decisions_match_oracle(monitor, samples):
    """The fused monitor + classification against the oracle on the same state."""
    w = amps()
    thr = (0.3, 0.6) if monitor == 1 else (1e-4, 1e-2)
    p = w.Params.preset("kobayashi", 2, mode="end2end_mix", nx=256, ny=256, monitor=monitor,
                        monitor_samples=samples, thr_lo=thr[0], thr_hi=thr[1], init_r2=400.0, max_log=16)
    back = 1 if monitor == 3 else 10  # the rate monitor compares with the previous step
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(50 - back)
        prev = s.fields()
        s.run(back)
        now = s.fields()
        m_gpu = s.metric()
        t_gpu = s.tiers()
        log = s.decision_log()
    m, t = _oracle_decisions(w, s, p, prev, now)
    assert np.array_equal(m_gpu, m), f"metric mismatch: {np.max(np.abs(m_gpu - m))}"
    assert np.array_equal(t_gpu, t)
    assert np.array_equal(log[-1], t_gpu)
    assert len(log) == 6  # the resting classification + one per period


def test_mixed_error_envelope_kobayashi():
    """Adaptive run against the FP64 oracle: the monitor keeps the interface in
    FP64, so the error stays near the half-precision storage floor."""
    w = amps()
    steps = 200
    p = w.Params.preset("kobayashi", 2, mode="end2end_mix", nx=256, ny=256, init_r2=400.0, monitor=1,
                        monitor_samples=1, thr_lo=0.02, thr_hi=0.2)
    f0 = w.init_host(p, w.INIT_REFERENCE)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
        st = s.stats()
    phi, T = ob.kob_run(ob.kob_params(256, 256), f0[0], f0[1], steps)
    e = max(np.max(np.abs(f[0] - phi)), np.max(np.abs(f[1] - T)))
    frac = np.array(st["tile_steps"]) / max(sum(st["tile_steps"]), 1)
    print(f"kobayashi mixed vs fp64 oracle: max abs {e:.3e}; tier mix half/fp32/fp64 {frac}")
    assert sum(st["tile_steps"]) == steps * s.ntiles[0] * s.ntiles[1]
    assert e <= 1e-3


def _spread_thresholds(w, p, steps, f0):
    """Thresholds from the monitor metric seen after `steps` steps of an
    all-FP64 run of the same workload: half the smallest positive value (so
    tiles whose metric is exactly 0 -- the sintering bulk -- go to half) and
    the 70th percentile of the positive values, so that a run with them
    populates all three tiers."""
    with w.Simulation(p.replace(thr_lo=0.0, thr_hi=0.0)) as s:
        s.set_fields(f0)
        s.run(steps)
        m = s.metric().ravel()
    pos = m[m > 0]
    lo, hi = 0.5 * pos.min(), np.quantile(pos, 0.7)
    return float(lo), float(max(hi, lo))


@pytest.mark.parametrize("monitor,samples", [(1, 0), (1, 1), (2, 0), (2, 1), (3, 1)])
def test_sintering_decisions_match_oracle(monitor, samples):
    """Adaptive sintering (sintering/main.cu:162-206, the AMSTENCIL loop;
    monitor on c, sintering/tools.h:3-56): the fused monitor and the
    classification against the oracle's get_max_diff / get_type on the GPU's
    own stored state, four particles on 128^2, three tiers populated."""
    w = amps()
    p = w.Params.preset("sintering", 0, nx=128, ny=128, nfields=4, rmin=10, rmax=16, tile=16, monitor=monitor,
                        monitor_samples=samples, monitor_field=0, max_log=32)
    f0 = w.init_host(p, w.INIT_SEEDED)
    lo, hi = _spread_thresholds(w, p, 60, f0)
    p = p.replace(thr_lo=lo, thr_hi=hi)
    back = 1 if monitor == 3 else 10
    with w.Simulation(p) as s:
        s.set_fields(f0)
        s.run(60 - back)
        prev = s.fields()
        s.run(back)
        now = s.fields()
        m_gpu, t_gpu, st = s.metric(), s.tiers(), s.stats()
    m, t = _oracle_decisions(w, s, p, prev, now)
    print(f"sintering monitor {monitor} samples {samples}: thresholds {lo:.3e} {hi:.3e}, tiers",
          np.bincount(t.ravel(), minlength=3))
    assert np.array_equal(m_gpu, m)
    assert np.array_equal(t_gpu, t)
    assert len(np.unique(t)) == 3
    assert sum(st["tile_steps"]) == 60 * t.size


def test_mixed_error_envelope_sintering():
    """Adaptive sintering against the FP64 oracle (reference expression
    order) over 200 steps: interface tiles in FP64 by the spatial monitor on
    c, the bulk (c and every eta exactly 0 or 1, stored exactly in half) in
    half.  Bar: the 1e-3 max-abs target on every field."""
    w = amps()
    p = w.Params.preset("sintering", 0, nx=128, ny=128, nfields=4, rmin=10, rmax=16, tile=16, ref_order=1,
                        monitor=w.MONITOR_SPA, monitor_samples=1, monitor_field=0, thr_lo=1e-3, thr_hi=0.9)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p) as s:
        s.set_fields(f0)
        s.run(200)
        f = s.fields()
        st = s.stats()
    op = ob.sint_params(128, 128, n=4, coefm=p.coefm, coefk=p.coefk, coefl=p.coefl, dsur=p.dsur)
    c, e = ob.sint_run(op, f0[0], list(f0[1:]), 200)
    errs = [float(np.max(np.abs(f[0] - c)))] + [float(np.max(np.abs(f[k + 1] - e[k]))) for k in range(4)]
    print("sintering mixed vs fp64 oracle, max abs per field:", errs, "tiles", st["tile_steps"])
    assert st["tile_steps"][0] > 0 and st["tile_steps"][2] > 0
    assert max(errs) <= 1e-3


def test_purelow_kobayashi_vs_oracle():
    """Kobayashi all-half run (snowflake/purelow.cu:19-26, kernel1/2_purelow,
    snowflake/function.h:607-700) against the FP64 oracle: phi and T are
    stored in binary16 after every step (half an ulp is 2^-12 at 1), so the
    error grows with the steps at most by about that much per step.  Bar after
    40 steps: max-abs <= 40 * 2^-12 ~ 9.8e-3, per field."""
    w = amps()
    steps = 40
    p = w.Params.preset("kobayashi", 2, mode="purelow", nx=256, ny=256, init_r2=400.0)
    f0 = w.init_host(p, w.INIT_REFERENCE)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
    phi, T = ob.kob_run(ob.kob_params(256, 256), f0[0], f0[1], steps)
    e_phi, e_T = float(np.max(np.abs(f[0] - phi))), float(np.max(np.abs(f[1] - T)))
    print(f"kobayashi purelow vs fp64 oracle after {steps} steps: phi {e_phi:.3e} T {e_T:.3e}")
    assert e_phi <= steps * 2.0 ** -12 and e_T <= steps * 2.0 ** -12
    assert e_phi > 0  # the half storage is really in use


@pytest.mark.parametrize("monitor,samples", [(1, 1), (2, 1), (3, 1), (2, 0)])
def test_graingrowth_decisions_match_oracle(monitor, samples):
    """Fused grain-growth kernel: every tier in one launch; monitor over all fields."""
    w = amps()
    thr = (1e-3, 0.5) if monitor == 1 else (1e-5, 3e-3)
    p = w.Params.preset("graingrowth", 0, nx=256, ny=192, nfields=5, monitor=monitor, monitor_samples=samples,
                        thr_lo=thr[0], thr_hi=thr[1], max_log=32)
    back = 1 if monitor == 3 else 10
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(200 - back)
        prev = s.fields()
        s.run(back)
        now = s.fields()
        m_gpu, t_gpu, st = s.metric(), s.tiers(), s.stats()
    m, t = _oracle_decisions(w, s, p, prev, now)
    assert np.array_equal(m_gpu, m)
    assert np.array_equal(t_gpu, t)
    assert sum(st["tile_steps"]) == 200 * t.size
    print("graingrowth tiers after 200 steps:", np.bincount(t.ravel(), minlength=3))


def test_mixed_graingrowth_envelope():
    w = amps()
    steps = 100
    p = w.Params.preset("graingrowth", 0, nx=128, ny=128, nfields=4)
    f0 = w.init_host(p, w.INIT_SEEDED)
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(steps)
        f = s.fields()
        st = s.stats()
    o = ob.gg_run(ob.gg_params(128, 128, q=4, dx=1.0, dy=1.0, dt=0.05, mobil=1.0, grcoef=2.0, gamma=1.5),
                  list(f0), steps)
    e = max(np.max(np.abs(f[k] - o[k])) for k in range(4))
    print(f"graingrowth mixed Q=4 vs fp64 oracle: max abs {e:.3e}; tiles {st['tile_steps']}")
    assert e <= 1e-3


# ------------------------------------------------------------- plumbing ----
def test_graph_replay_equals_eager():
    w = amps()
    p = w.Params.preset("graingrowth", 0, nx=128, ny=128, nfields=4)
    out = []
    for graphs in (True, False):
        with w.Simulation(p, init=w.INIT_SEEDED, graphs=graphs) as s:
            s.run(23)
            s.run(17)
            out.append((s.fields(), s.tiers(), s.stats()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


@pytest.mark.parametrize("tile,ref_order,monitor", [(32, 0, 3), (32, 1, 2), (16, 0, 3), (16, 1, 2)])
def test_graingrowth_fp64_tiles_staged_and_fused_agree(tile, ref_order, monitor):
    """An adaptive run whose tiles all stay FP64 (thresholds 0): its first
    period (every tile FP64 by construction) runs the staged FP64 kernel, the
    later ones the fused kernel's FP64 path, monitor steps included; both
    give the plain FP64 run's results bit for bit."""
    w = amps()
    p = w.Params.preset("graingrowth", 0, nx=128, ny=96, nfields=5, tile=tile, ref_order=ref_order, monitor=monitor,
                        monitor_samples=1, thr_lo=0.0, thr_hi=0.0)
    out = []
    for mode in ("end2end_mix", "purehigh"):
        with w.Simulation(p.replace(mode=mode), init=w.INIT_SEEDED) as s:
            s.run(7)
            s.run(28)
            out.append(s.fields())
            if mode == "end2end_mix":
                assert (s.tiers() == w.TIER_FP64).all()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("model", ["graingrowth", "kobayashi"])
def test_profiled_run_equals_plain_and_times_every_launch(model):
    """Profiling (whole periods captured with their event records as graph
    nodes, the partial period eager) changes no result and times each step."""
    import torch

    w = amps()
    p = w.Params.preset(model, 0, nx=128, ny=128)
    stream = torch.cuda.Stream()
    out = []
    for prof in (False, True):
        with w.Simulation(p, init=w.INIT_SEEDED) as s:
            s.set_stream(stream.cuda_stream)
            s.run(3)
            s.set_profiling(prof)
            s.run(2 * p.cadence + 3)
            s.synchronize()
            if prof:
                ms, launches, tiles = s.kernel_times()
                st = s.stats()
            out.append((s.fields(), s.tiers()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    steps = 2 * p.cadence + 3
    if model == "graingrowth":
        assert launches[3] == steps and ms[3] > 0
    else:
        assert sum(launches) >= steps and all(m >= 0 for m in ms) and sum(ms) > 0
    assert tiles[3] > 0 and st["tile_steps"]


@pytest.mark.parametrize("monitor", [1, 2, 3])
def test_monitor_flags_non_finite_values(monitor):
    """A NaN in the input state reaches the monitor step of every monitor kind
    and sets the numeric-error flag; a clean run leaves it clear."""
    w = amps()
    # FP32 high tier: the monitor steps run on the half/FP32 path from the start
    p = w.Params.preset("graingrowth", 0, nx=128, ny=128, nfields=4, tile=32, mode="end2end_mix",
                        monitor=monitor, monitor_samples=1, thr_lo=1e-5, high_tier=w.TIER_FP32)
    f0 = w.init_host(p, w.INIT_SEEDED)
    for poison in (False, True):
        f = f0.copy()
        if poison:
            f[2, 70, 45] = np.nan
        with w.Simulation(p) as s:
            s.set_fields(f)
            s.run(2 * p.cadence)
            assert s.stats()["numeric_error"] == int(poison)


@pytest.mark.parametrize("mode", ["purehigh", "end2end_mix"])
def test_tma_step_kernel_matches_default(mode, monkeypatch):
    """The opt-in persistent TMA kernel (AMPS_ENABLE_TMA=1: tensor copies of
    whole FP32 neighbourhoods, double-buffered) gives the default kernel's
    results bit for bit."""
    w = amps()
    extra = dict(high_tier=w.TIER_FP32) if mode == "purehigh" else dict(monitor=w.MONITOR_RATE, monitor_samples=1,
                                                                          thr_lo=1e-5)
    p = w.Params.preset("graingrowth", 0, nx=256, ny=256, nfields=8, tile=32, mode=mode, **extra)
    out = []
    for tma in ("0", "1"):
        monkeypatch.setenv("AMPS_ENABLE_TMA", tma)
        with w.Simulation(p, init=w.INIT_SEEDED) as s:
            s.run(25)
            out.append((s.fields(), s.tiers(), s.stats()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


@pytest.mark.parametrize("case", ["adaptive_q8", "adaptive_q5_noflux", "fp32_q8", "ref_half_q2"])
def test_bulk_tensor_staging_matches_per_thread_copies(case, monkeypatch):
    """Interior tiles of the fused grain-growth step fetch their FP32
    neighbourhood by one bulk tensor copy (the default); with
    AMPS_DISABLE_TMA_STAGE=1 every tile stages by per-thread asynchronous
    copies.  Bit for bit the same fields, tiers and statistics: three tiers
    with a rate monitor, Q = 5 with zero flux, all-FP32, and the
    binary16-arithmetic half tiles."""
    w = amps()
    q = 2 if "q2" in case else (5 if "q5" in case else 8)
    if case.startswith("fp32"):
        extra = dict(mode="purehigh", high_tier=w.TIER_FP32)
    elif case.startswith("ref_half"):
        extra = dict(monitor=w.MONITOR_RATE, monitor_samples=1, thr_lo=1e-4, thr_hi=3e-3, half_arith=w.HALF_REF)
    else:
        extra = dict(monitor=w.MONITOR_RATE, monitor_samples=1, thr_lo=1e-5, thr_hi=3e-3)
    p = w.Params.preset("graingrowth", 0, nx=256, ny=192, nfields=q, tile=32, bc=1 if "noflux" in case else 0,
                        **extra)
    out = []
    for off in ("1", "0"):
        monkeypatch.setenv("AMPS_DISABLE_TMA_STAGE", off)
        with w.Simulation(p, init=w.INIT_SEEDED) as s:
            s.run(23)
            s.run(57)
            out.append((s.fields(), s.tiers(), s.stats()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    print(case, "tile-steps", out[1][2]["tile_steps"])


@pytest.mark.parametrize("case", ["adaptive_q8", "adaptive_q5_noflux", "fp32_q8", "adaptive_q8_eager"])
def test_multi_step_kernel_matches_one_launch_per_step(case, monkeypatch):
    """The opt-in multi-step kernel (AMPS_ENABLE_FLOW=1: the interior steps of
    a period in one launch, a CTA per (step, tile), each tile starting once
    its neighbourhood finished the previous step) gives the default
    one-launch-per-step results bit for bit:
    three tiers with a rate monitor, Q = 5 on the 4-row path with zero flux,
    the all-FP32 plain mode (whole periods in one launch), graphs off; runs
    split into partial periods."""
    w = amps()
    q = 5 if "q5" in case else 8
    extra = dict(mode="purehigh", high_tier=w.TIER_FP32) if case.startswith("fp32") else \
        dict(monitor=w.MONITOR_RATE, monitor_samples=1, thr_lo=1e-5, thr_hi=3e-3)
    p = w.Params.preset("graingrowth", 0, nx=256, ny=192, nfields=q, tile=32,
                        bc=1 if "noflux" in case else 0, **extra)
    out = []
    for on in ("0", "1"):
        monkeypatch.setenv("AMPS_ENABLE_FLOW", on)
        with w.Simulation(p, init=w.INIT_SEEDED, graphs=not case.endswith("eager")) as s:
            s.run(23)
            s.run(17)
            s.run(60)
            out.append((s.fields(), s.tiers(), s.stats(), s.kernel_launches()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    assert out[1][3] < out[0][3]  # fewer launches with the multi-step kernel
    print(case, "launches per 100 steps: one per step", out[0][3], "multi-step", out[1][3])


def test_set_get_roundtrip_and_reduce():
    w = amps()
    p = w.Params.preset("sintering", 1, mode="purehigh", nx=64, ny=64)
    rng = np.random.default_rng(3)
    a = rng.random((3, 64, 64))
    with w.Simulation(p) as s:
        s.set_fields(a)
        assert np.array_equal(s.fields(), a)
        b = rng.random((64, 64))
        s.set_field(1, b)
        assert np.array_equal(s.field(1), b) and np.array_equal(s.field(0), a[0])
        assert abs(s.reduce(0) - a[0].sum()) <= 1e-12 * a[0].size
        assert s.reduce(0, w.amps.REDUCE_MAX) == a[0].max()
        mx, rms = s.compare(2, a[2] + 0.5)
        assert abs(mx - 0.5) < 1e-15 and abs(rms - 0.5) < 1e-15


@pytest.mark.parametrize("aniso,bc", [(6.0, 0), (4.0, 1), (5.0, 0), (6.5, 1)])
def test_kobayashi_fp32_anisotropy_paths_vs_oracle(aniso, bc):
    """FP32 Kobayashi tiles take the anisotropy cos/sin of aniso*(theta -
    theta0) by de Moivre's formula when aniso is an even integer (the
    reference's 6), by atan2/cos/sin otherwise: both within the FP32 tier's
    bound of the FP64 oracle (snowflake/function.h:30-34), theta0 != 0 and an
    off-centre seed so that every angle occurs."""
    w = amps()
    nx, ny, steps = 96, 64, 40
    p = w.Params.preset("kobayashi", 4, mode="purehigh", high_tier=w.TIER_FP32, nx=nx, ny=ny, bc=bc, noise=0.0,
                        aniso=aniso, theta0=0.3, init_offset=3, init_r2=60.0)
    f0 = w.init_host(p, w.INIT_REFERENCE)
    with w.Simulation(p, init=w.INIT_REFERENCE) as s:
        s.run(steps)
        f = s.fields()
    q = ob.kob_params(nx, ny, bc=bc, aniso=aniso, theta0=0.3)
    phi, T = ob.kob_run(q, f0[0], f0[1], steps)
    e = max(float(np.abs(f[0] - phi).max()), float(np.abs(f[1] - T).max()))
    print(f"kobayashi fp32 aniso {aniso} bc {bc}: max abs vs fp64 oracle {e:.3e}")
    assert e <= 1e-6  # measured 1.5-1.8e-7 on either path
