"""The reference-named wrappers (include/amps_compat.h) driven exactly like the
reference's purehigh time loops (snowflake/purehigh.cu, graingrowth/purehigh.cu,
sintering/main.cu:137-146) reproduce the reference's own outputs
(tests/golden/), with the parity bars of the fused path: 1e-12 relative
(Kobayashi: at the early snapshot; after 40 steps the symmetric seed's
atan2 discontinuity allows 1e-3 / 1e-2, see test_gpu_parity.py).  The monitor
tools match the oracle's restatement exactly."""
import ctypes
import os

import numpy as np
import pytest
import torch

import oracle_bind as ob

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
P = ctypes.c_void_p


def w():
    import w3914777_gb300 as m
    return m


def lib():
    L = w().lib()
    dp = ctypes.POINTER(w().Params)
    for name, n in (("amps_snowflake_kernel1_pure", 8), ("amps_snowflake_kernel2_pure", 8),
                    ("amps_snowflake_dataprepare_high", 1), ("amps_graingrowth_kernel1_pure", 5),
                    ("amps_get_max_diff1", 2), ("amps_get_max_diff2", 3), ("amps_get_type", 3)):
        f = getattr(L, name)
        f.argtypes = [dp] + [P] * n + [P]
        f.restype = ctypes.c_int
    for name in ("amps_sintering_con1_pure",):
        getattr(L, name).argtypes = [dp] + [P] * 6 + [ctypes.c_int, P]
    for name in ("amps_sintering_con2_pure",):
        getattr(L, name).argtypes = [dp] + [P] * 5 + [ctypes.c_int, P]
    for name in ("amps_sintering_phi1_pure", "amps_sintering_phi2_pure"):
        getattr(L, name).argtypes = [dp] + [P] * 6 + [ctypes.c_int, P]
    return L


def ptr(t):
    return P(t.data_ptr())


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def zeros(p, k=1):
    return [torch.zeros((p.ny, p.nx), dtype=torch.float64, device="cuda") for _ in range(k)]


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_snowflake_kernels_match_reference_golden():
    L = lib()
    g = np.load(os.path.join(GOLD, "kobayashi_ref.npz"))
    p = w().Params.preset("kobayashi", 2, mode="purehigh")
    pp = ctypes.byref(p)
    phi, T = zeros(p, 2)
    phi_lap, T_lap, px, py, eps, epd = zeros(p, 6)
    assert L.amps_snowflake_dataprepare_high(pp, ptr(phi), None) == 0
    snaps = {}
    for i in range(int(g["steps"])):
        assert L.amps_snowflake_kernel1_pure(pp, ptr(phi), ptr(phi_lap), ptr(T), ptr(T_lap), ptr(px), ptr(py),
                                             ptr(eps), ptr(epd), None) == 0
        assert L.amps_snowflake_kernel2_pure(pp, ptr(phi), ptr(phi_lap), ptr(eps), ptr(epd), ptr(px), ptr(py),
                                             ptr(T), ptr(T_lap), None) == 0
        if i + 1 == int(g["early"]):
            snaps["early"] = (phi.cpu().numpy(), T.cpu().numpy())
    torch.cuda.synchronize()
    e8 = max(rel_err(snaps["early"][0], g["phi_early"]), rel_err(snaps["early"][1], g["T_early"]))
    e_phi, e_T = rel_err(phi.cpu().numpy(), g["phi"]), rel_err(T.cpu().numpy(), g["T"])
    print(f"snowflake wrappers vs reference: early {e8:.3e}, final phi {e_phi:.3e} T {e_T:.3e}")
    assert e8 <= 1e-12
    assert e_phi <= 1e-3 and e_T <= 1e-2


def test_graingrowth_kernel_matches_reference_golden():
    L = lib()
    g = np.load(os.path.join(GOLD, "graingrowth_ref.npz"))
    p = w().Params.preset("graingrowth", 1, mode="purehigh")
    pp = ctypes.byref(p)
    f0 = w().init_host(p, w().INIT_REFERENCE)
    e1, e2 = dev(f0[0]), dev(f0[1])
    o1, o2, l1, l2, d1, d2 = zeros(p, 6)
    for _ in range(int(g["steps"])):
        assert L.amps_graingrowth_kernel1_pure(pp, ptr(e1), ptr(e2), ptr(l1), ptr(d1), ptr(o1), None) == 0
        assert L.amps_graingrowth_kernel1_pure(pp, ptr(e2), ptr(e1), ptr(l2), ptr(d2), ptr(o2), None) == 0
        e1, o1 = o1, e1
        e2, o2 = o2, e2
    torch.cuda.synchronize()
    a, b = rel_err(e1.cpu().numpy(), g["eta1"]), rel_err(e2.cpu().numpy(), g["eta2"])
    print(f"graingrowth wrapper vs reference: {a:.3e} {b:.3e}")
    assert a <= 1e-12 and b <= 1e-12


def test_sintering_kernels_match_reference_golden():
    L = lib()
    g = np.load(os.path.join(GOLD, "sintering_ref.npz"))
    p = w().Params.preset("sintering", 5, mode="purehigh")
    pp = ctypes.byref(p)
    f0 = w().init_host(p, w().INIT_REFERENCE)
    con, e1, e2 = dev(f0[0]), dev(f0[1]), dev(f0[2])
    con_lap, dfdcon, dummy, dummy_lap, o1, o2, l1, l2, d1, d2 = zeros(p, 10)
    for i in range(int(g["steps"])):
        assert L.amps_sintering_con1_pure(pp, ptr(con), ptr(con_lap), ptr(e1), ptr(e2), ptr(dfdcon), ptr(dummy), i,
                                          None) == 0
        assert L.amps_sintering_con2_pure(pp, ptr(dummy), ptr(dummy_lap), ptr(con), ptr(e1), ptr(e2), i, None) == 0
        assert L.amps_sintering_phi1_pure(pp, ptr(e1), ptr(o1), ptr(e2), ptr(l1), ptr(d1), ptr(con), i, None) == 0
        assert L.amps_sintering_phi2_pure(pp, ptr(e2), ptr(o2), ptr(e1), ptr(l2), ptr(d2), ptr(con), i, None) == 0
        e1, o1 = o1, e1
        e2, o2 = o2, e2
    torch.cuda.synchronize()
    errs = [rel_err(con.cpu().numpy(), g["c"]), rel_err(e1.cpu().numpy(), g["eta1"]),
            rel_err(e2.cpu().numpy(), g["eta2"])]
    print("sintering wrappers vs reference:", errs)
    assert max(errs) <= 1e-12


@pytest.mark.parametrize("tile", [16, 32])
def test_monitor_tools_match_oracle(tile):
    L = lib()
    p = w().Params.preset("kobayashi", 2, mode="purehigh", nx=128, ny=96, tile=tile, thr_hi=0.35)
    pp = ctypes.byref(p)
    rng = np.random.default_rng(3)
    now = rng.uniform(0, 1, (p.ny, p.nx)) ** 3
    last = now + rng.normal(0, 0.01, now.shape)
    ntx, nty = p.nx // tile, p.ny // tile
    md1 = torch.zeros((nty, ntx), dtype=torch.float64, device="cuda")
    md2 = torch.zeros_like(md1)
    cur = torch.full((nty, ntx), 2, dtype=torch.int32, device="cuda")
    old = torch.zeros_like(cur)
    assert L.amps_get_max_diff1(pp, ptr(dev(now)), ptr(md1), None) == 0
    assert L.amps_get_max_diff2(pp, ptr(dev(last)), ptr(dev(now)), ptr(md2), None) == 0
    assert L.amps_get_type(pp, ptr(md1), ptr(old), ptr(cur), None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(md1.cpu().numpy(), ob.monitor_spa(now, tile).reshape(nty, ntx))
    np.testing.assert_array_equal(md2.cpu().numpy(), ob.monitor_tem(now, last, tile).reshape(nty, ntx))
    ref = ob.classify(md1.cpu().numpy(), p.thr_hi, p.thr_hi)
    np.testing.assert_array_equal(cur.cpu().numpy(), np.where(ref >= 2, 2, 1))
    assert (old.cpu().numpy() == 2).all()
