"""The CPU oracle against the reference's own plain kernels run on the CPU.

oracle/_ref/ holds the reference's snowflake/graingrowth/sintering kernels
compiled in place from the reference sources (oracle/Makefile, target `ref`).
When present, the oracle must reproduce them bit for bit.  Without it (a
machine without the reference tree) the committed golden fixtures, which were
generated from those same builds by tests/golden/make_golden.py, pin the
oracle instead (tests/test_oracle_golden.py).
"""
import os

import numpy as np
import pytest

import oracle_bind as ob

N = 512  # the reference's compile-time grid (snowflake/paras/total.h:20)


@pytest.mark.skipif(not ob.ref_available("snowflake"), reason="reference CPU build absent")
def test_kobayashi_bit_exact_vs_reference():
    R = ob.ref_lib("snowflake")
    phi = np.zeros((N, N)); T = np.zeros((N, N))
    R.ref_snowflake_init(ob.ptr(phi), ob.ptr(T))
    phi0, T0 = ob.kob_init_disc(N, N, N // 2 + 8, N // 2 + 8, 10.0)
    assert np.array_equal(phi, phi0) and np.array_equal(T, T0)
    R.ref_snowflake_steps(ob.ptr(phi), ob.ptr(T), 12)
    p2, T2 = ob.kob_run(ob.kob_params(N, N), phi0, T0, 12)
    assert np.array_equal(phi, p2)
    assert np.array_equal(T, T2)


@pytest.mark.skipif(not ob.ref_available("graingrowth"), reason="reference CPU build absent")
def test_graingrowth_bit_exact_vs_reference():
    R = ob.ref_lib("graingrowth")
    e1 = np.zeros((N, N)); e2 = np.zeros((N, N))
    R.ref_gg_init(ob.ptr(e1), ob.ptr(e2))
    a1, a2 = ob.gg_init_circle(N, N, 256, 256, 50)
    assert np.array_equal(e1, a1) and np.array_equal(e2, a2)
    R.ref_gg_steps(ob.ptr(e1), ob.ptr(e2), 12)
    b = ob.gg_run(ob.gg_params(N, N), [a1, a2], 12)
    assert np.array_equal(e1, b[0]) and np.array_equal(e2, b[1])


@pytest.mark.skipif(not ob.ref_available("sintering"), reason="reference CPU build absent")
def test_sintering_bit_exact_vs_reference():
    pr = ob.ref_params("sintering", 15)
    c, s1, s2 = ob.sint_init_two(N, N, pr[12], pr[13], pr[10], pr[14], pr[11])
    R = ob.ref_lib("sintering")
    c1, t1, t2 = c.copy(), s1.copy(), s2.copy()
    R.ref_sint_steps(ob.ptr(c1), ob.ptr(t1), ob.ptr(t2), 12)
    c2, (u1, u2) = ob.sint_run(ob.sint_params(N, N), c, [s1, s2], 12)
    assert np.array_equal(c1, c2) and np.array_equal(t1, u1) and np.array_equal(t2, u2)


def test_monitor_lattices():
    pts = (np.zeros(4, dtype=np.int32))
    import ctypes
    L = ob.lib()
    L.orc_sample_points(16, 1, pts.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    assert list(pts) == [0, 5, 10, 15]  # snowflake/tools.h:185
    L.orc_sample_points(16, 2, pts.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    assert list(pts) == [2, 6, 10, 14]  # snowflake/tools.h:203


def test_classify_is_non_periodic_five_point_max():
    m = np.zeros((4, 4))
    m[0, 0] = 1.0  # corner tile: neighbours (0,1) and (1,0) promoted, wrap-around ones not
    t = ob.classify(m, 0.5, 0.5)
    assert t[0, 0] == 2 and t[0, 1] == 2 and t[1, 0] == 2
    assert t[3, 0] == 0 and t[0, 3] == 0 and t[1, 1] == 0
    t3 = ob.classify(np.array([[0.0, 0.2], [0.6, 0.0]]), 0.1, 0.5)
    assert t3.tolist() == [[2, 1], [2, 2]]


@pytest.mark.parametrize("monitor,thr", [(2, 1e-4), (1, 0.5)])
def test_reference_mixed_golden_comes_from_the_reference_kernels(monitor, thr):
    """tests/golden/graingrowth_mix_ref.npz (the reference's AMSTENCIL runs,
    made by tests/golden/make_golden_mix.py): its first periods' tier maps
    are what the reference's kernels, compiled here for the CPU, produce."""
    import importlib.util
    if not os.path.exists(os.path.join(ob.REF_DIR, f"libref_ggmix_m{monitor}.so")):
        pytest.skip("oracle/_ref not built (no reference tree)")
    spec = importlib.util.spec_from_file_location(
        "make_golden_mix", os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_golden_mix.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "graingrowth_mix_ref.npz"))
    types, _, _ = mg.run_mix(monitor, thr, steps=30)
    assert np.array_equal(types, g[mg.key(monitor, thr) + "_types"][:3])
