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
