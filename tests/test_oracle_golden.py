"""The CPU oracle against the committed golden fixtures (reference outputs made
by tests/golden/make_golden.py from the reference's own kernels).  Bit-exact."""
import os

import numpy as np

import oracle_bind as ob

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
N = 512


def test_kobayashi_golden():
    g = np.load(os.path.join(GOLD, "kobayashi_ref.npz"))
    phi0, T0 = ob.kob_init_disc(N, N, N // 2 + 8, N // 2 + 8, 10.0)
    phi, T = ob.kob_run(ob.kob_params(N, N), phi0, T0, int(g["steps"]))
    assert np.array_equal(phi, g["phi"]) and np.array_equal(T, g["T"])


def test_graingrowth_golden():
    g = np.load(os.path.join(GOLD, "graingrowth_ref.npz"))
    a1, a2 = ob.gg_init_circle(N, N, 256, 256, 50)
    e = ob.gg_run(ob.gg_params(N, N), [a1, a2], int(g["steps"]))
    assert np.array_equal(e[0], g["eta1"]) and np.array_equal(e[1], g["eta2"])


def test_sintering_golden():
    g = np.load(os.path.join(GOLD, "sintering_ref.npz"))
    pr = g["params"]
    c, s1, s2 = ob.sint_init_two(N, N, pr[12], pr[13], pr[10], pr[14], pr[11])
    c2, (u1, u2) = ob.sint_run(ob.sint_params(N, N), c, [s1, s2], int(g["steps"]))
    assert np.array_equal(c2, g["c"]) and np.array_equal(u1, g["eta1"]) and np.array_equal(u2, g["eta2"])


def test_timed_baseline_build_matches_the_checker():
    """The CPU baseline that bench.py times (liboracle_fast.so: -O3, fused
    multiply-add, the row-restructured grain-growth loop) computes the same
    update as the checker, to rounding, on both boundaries and stencils; it
    is never used as a checker itself."""
    for bc in (0, 1):
        for stencil in (0, 1):
            etas = ob.gg_init_uniform(96, 64, 5, 0.5, 7)
            p = ob.gg_params(96, 64, q=5, bc=bc, stencil=stencil, dx=1.0, dy=1.0, dt=0.05, mobil=1.0,
                             grcoef=2.0, gamma=1.5)
            slow = ob.gg_run(p, etas, 6)
            fast = ob.gg_run(p, etas, 6, fast=True)
            err = max(float(np.abs(a - b).max()) for a, b in zip(slow, fast))
            assert 0 < err <= 1e-14 or err == 0, (bc, stencil, err)
    phi0, T0 = ob.kob_init_disc(64, 64, 32, 32, 25.0)
    kp = ob.kob_params(64, 64, bc=1, kappa=1.6, theta0=0.2, noise=0.01, seed=3)
    a = ob.kob_run(kp, phi0, T0, 5)
    b = ob.kob_run(kp, phi0, T0, 5, fast=True)
    assert max(float(np.abs(x - y).max()) for x, y in zip(a, b)) <= 1e-12


def test_seeded_multigrain_start_matches_the_library():
    """The oracle's seeded start (eta_i ~ U[-amp, amp) keyed by seed, field,
    cell) equals the library's amps_init_host, so the CPU baseline and the
    GPU runs start from the same state."""
    import w3914777_gb300 as w
    p = w.Params.preset("graingrowth", 0, nx=64, ny=96, nfields=3)
    lib_state = w.init_host(p, w.INIT_SEEDED)
    orc_state = ob.gg_init_uniform(64, 96, 3, p.init_amp, p.seed)
    assert all(np.array_equal(lib_state[k], orc_state[k]) for k in range(3))
