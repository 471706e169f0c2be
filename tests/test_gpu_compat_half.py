"""The reference-named binary16 wrappers (include/amps_compat.h: the all-half2
"purelow" steps of grain growth and the Kobayashi dendrite, their half2
preparation and gathering) driven exactly like the reference's purelow
programs (graingrowth/purelow.cu, snowflake/purelow.cu), against the
reference's own kernels run on the same GPU (baseline/_ref cubins; skipped
where they are not built).  Same arrays, same launch sequence: the half2
words at the end are compared bit for bit."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

refcuda = pytest.importorskip("baseline.refcuda")
P = ctypes.c_void_p


def w():
    import w3914777_gb300 as m
    return m


def lib():
    L = w().lib()
    dp = ctypes.POINTER(w().Params)
    for name, n in (("amps_graingrowth_kernel1_lowpure", 5), ("amps_graingrowth_dataprepare_half2", 2),
                    ("amps_snowflake_kernel1_purelow", 8), ("amps_snowflake_kernel2_purelow", 8),
                    ("amps_snowflake_dataprepare_half2", 1), ("amps_purelow2high_aftercomputing", 2)):
        f = getattr(L, name)
        f.argtypes = [dp] + [P] * n + [P]
        f.restype = ctypes.c_int
    return L


def need(name):
    if not refcuda.available(name):
        pytest.skip(f"baseline/_ref/{name}.cubin not built (needs the reference tree)")


def half2s(p, k):
    return [torch.zeros((p.ny, p.nx // 2), dtype=torch.int32, device="cuda") for _ in range(k)]


def ptr(t):
    return P(t.data_ptr())


def words(t):
    return t.cpu().numpy().view(np.uint32)


def ulps(a, b):
    """max distance in binary16 ulps (same sign assumed) between two half2 word arrays"""
    ha, hb = a.view(np.uint16).astype(np.int64), b.view(np.uint16).astype(np.int64)
    return int(np.max(np.abs(ha - hb)))


@pytest.mark.parametrize("steps", [1, 40, 300])
def test_graingrowth_lowpure_equals_the_reference_kernel(steps):
    need("graingrowth_purelow")
    L = lib()
    p = w().Params.preset("graingrowth", 1, mode="purelow")
    pp = ctypes.byref(p)
    e1, e2, o1, o2, l1, l2, d1, d2 = half2s(p, 8)
    assert L.amps_graingrowth_dataprepare_half2(pp, ptr(e1), ptr(e2), None) == 0
    for _ in range(steps):
        assert L.amps_graingrowth_kernel1_lowpure(pp, ptr(e1), ptr(e2), ptr(l1), ptr(d1), ptr(o1), None) == 0
        assert L.amps_graingrowth_kernel1_lowpure(pp, ptr(e2), ptr(e1), ptr(l2), ptr(d2), ptr(o2), None) == 0
        e1, o1 = o1, e1
        e2, o2 = o2, e2
    torch.cuda.synchronize()
    r1, r2, _ = refcuda.gg_purelow(steps)
    ours1, ours2 = words(e1), words(e2)
    print(f"grain growth purelow {steps} steps: words differing {int((ours1 != r1).sum() + (ours2 != r2).sum())}, "
          f"max {max(ulps(ours1, r1), ulps(ours2, r2))} ulp")
    assert np.array_equal(ours1, r1) and np.array_equal(ours2, r2)
    # the gathering tool: floats of the half2 pairs
    f = torch.zeros((p.ny, p.nx), dtype=torch.float32, device="cuda")
    assert L.amps_purelow2high_aftercomputing(pp, ptr(e2), ptr(f), None) == 0
    h = ours2.view(np.float16).astype(np.float32)
    assert np.array_equal(f.cpu().numpy(), h.reshape(p.ny, p.nx))


@pytest.mark.parametrize("steps", [1, 8, 100])
def test_snowflake_purelow_equals_the_reference_kernels(steps):
    need("snowflake_purelow")
    L = lib()
    p = w().Params.preset("kobayashi", 2, mode="purelow")
    pp = ctypes.byref(p)
    phi, T, pl, tl, px, py, eps, epd = half2s(p, 8)
    assert L.amps_snowflake_dataprepare_half2(pp, ptr(phi), None) == 0
    for _ in range(steps):
        assert L.amps_snowflake_kernel1_purelow(pp, ptr(phi), ptr(pl), ptr(T), ptr(tl), ptr(px), ptr(py), ptr(eps),
                                                ptr(epd), None) == 0
        assert L.amps_snowflake_kernel2_purelow(pp, ptr(phi), ptr(pl), ptr(eps), ptr(epd), ptr(px), ptr(py), ptr(T),
                                                ptr(tl), None) == 0
    torch.cuda.synchronize()
    rp, rt, _ = refcuda.kob_purelow(steps)
    ours_p, ours_t = words(phi), words(T)
    print(f"kobayashi purelow {steps} steps: words differing {int((ours_p != rp).sum() + (ours_t != rt).sum())}")
    assert np.array_equal(ours_p, rp) and np.array_equal(ours_t, rt)


def test_half2_wrappers_reject_what_the_reference_cannot_run():
    L = lib()
    z = half2s(w().Params.preset("graingrowth", 1), 5)
    bad = w().Params.preset("graingrowth", 1, bc=w().BC_NOFLUX)
    assert L.amps_graingrowth_kernel1_lowpure(ctypes.byref(bad), *[ptr(t) for t in z], None) != 0
    odd = w().Params.preset("graingrowth", 1, nx=511)
    assert L.amps_graingrowth_kernel1_lowpure(ctypes.byref(odd), *[ptr(t) for t in z], None) != 0


def mix_lib():
    L = lib()
    dp = ctypes.POINTER(w().Params)
    I = ctypes.c_int
    sig = {
        "amps_graingrowth_kernel1_mix": [P] * 11 + [P, I, I],
        "amps_graingrowth_dataprepare_high": [P, P],
        "amps_graingrowth_data_sychro_duringcomputation": [P] * 6,
        "amps_graingrowth_data_sychro_aftercomputation": [P] * 3,
        "amps_graingrowth_highdata_to_low": [P, P],
        "amps_graingrowth_kernel1_conversion": [P, P, P, I],
        "amps_graingrowth_monitor2_lastdata_store": [P, P],
        "amps_get_max_diff1": [P, P],
        "amps_get_max_diff2": [P, P, P],
        "amps_get_type": [P, P, P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = [dp] + args + [P]
        f.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("monitor,thr,steps", [(1, 0.5, 200), (2, 1e-4, 200), (2, 1e-2, 120), (1, 0.1, 120)])
def test_graingrowth_mixed_loop_equals_the_reference_kernels(monitor, thr, steps):
    """graingrowth/end2end_mix.cu's loop (AMSTENCIL, Monitor1/2) through the
    reference-named wrappers: the initial circle, per period get_max_diff /
    get_type / data_sychro_duringcomputation, two kernel1_mix a step, the
    final data_sychro_aftercomputation -- against the reference's own
    kernels driven the same way: the tile types of every period and the
    final fields, bit for bit."""
    need(f"graingrowth_mix_m{monitor}")
    L = mix_lib()
    p = w().Params.preset("graingrowth", 1, mode="end2end_mix", monitor=monitor, thr_lo=thr, thr_hi=thr)
    with refcuda.Module(f"graingrowth_mix_m{monitor}") as m:
        assert (m.nx, m.ny, m.ux, m.uy) == (p.nx, p.ny, p.tile, p.tile)
    pp = ctypes.byref(p)
    nx, ny, T = p.nx, p.ny, p.tile
    tiles = (nx // T) * (ny // T)
    f64 = lambda: torch.zeros((ny, nx), dtype=torch.float64, device="cuda")
    e1, e2, o1, o2, l1, l2, d1, d2, last = (f64() for _ in range(9))
    h1, h2, ho1, ho2, hl1, hl2, hd1, hd2 = half2s(p, 8)
    tcur = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    told = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    md = torch.zeros(tiles, dtype=torch.float64, device="cuda")
    assert L.amps_graingrowth_dataprepare_high(pp, ptr(e1), ptr(e2), None) == 0
    assert L.amps_graingrowth_dataprepare_half2(pp, ptr(h1), ptr(h2), None) == 0
    if monitor == 2:  # end2end_mix.cu:43-47
        last.copy_((e2 == 0).double())
    types = []
    for i in range(steps):
        if i % 10 == 0:
            if monitor == 1:
                assert L.amps_get_max_diff1(pp, ptr(e2), ptr(md), None) == 0
            else:
                assert L.amps_get_max_diff2(pp, ptr(last), ptr(e2), ptr(md), None) == 0
            assert L.amps_get_type(pp, ptr(md), ptr(told), ptr(tcur), None) == 0
            assert L.amps_graingrowth_data_sychro_duringcomputation(pp, ptr(e1), ptr(e2), ptr(h1), ptr(h2),
                                                                    ptr(told), ptr(tcur), None) == 0
            types.append(tcur.cpu().numpy().astype(np.uint8))
        assert L.amps_graingrowth_kernel1_mix(pp, ptr(e1), ptr(last), ptr(e2), ptr(l1), ptr(d1), ptr(o1), ptr(h1),
                                              ptr(h2), ptr(hl1), ptr(hd1), ptr(ho1), ptr(tcur), i, 1, None) == 0
        assert L.amps_graingrowth_kernel1_mix(pp, ptr(e2), ptr(last), ptr(e1), ptr(l2), ptr(d2), ptr(o2), ptr(h2),
                                              ptr(h1), ptr(hl2), ptr(hd2), ptr(ho2), ptr(tcur), i, 2, None) == 0
        e1, o1, e2, o2 = o1, e1, o2, e2
        h1, ho1, h2, ho2 = ho1, h1, ho2, h2
    assert L.amps_graingrowth_data_sychro_aftercomputation(pp, ptr(e1), ptr(h1), ptr(tcur), None) == 0
    assert L.amps_graingrowth_data_sychro_aftercomputation(pp, ptr(e2), ptr(h2), ptr(tcur), None) == 0
    torch.cuda.synchronize()
    r1, r2, rtypes, _ = refcuda.gg_mix(steps, thr, monitor)
    ours = np.stack(types)
    both = ours.ravel()
    mix = np.bincount(both, minlength=3)[1:] / both.size
    bad = [k for k in range(rtypes.shape[0]) if not np.array_equal(ours[k], rtypes[k])]
    f1, f2 = e1.cpu().numpy(), e2.cpu().numpy()
    d = max(float(np.abs(f1 - r1).max()), float(np.abs(f2 - r2).max()))
    print(f"grain growth mixed loop, monitor {monitor} {thr:g}, {steps} steps: tile types half/FP64 {mix}, "
          f"periods differing {bad[:5]}, fields max |diff| {d:.3e}")
    assert not bad
    assert np.array_equal(f1, r1) and np.array_equal(f2, r2)


def test_graingrowth_mix_tools():
    """highdata_to_low, kernel1_conversion and monitor2_lastdata_store
    against numpy statements of graingrowth/tools.h:158-171 and
    function.h:311-341 on random data and types."""
    L = mix_lib()
    p = w().Params.preset("graingrowth", 1, mode="end2end_mix")
    pp = ctypes.byref(p)
    nx, ny, T = p.nx, p.ny, p.tile
    rng = np.random.default_rng(3)
    hi = rng.uniform(-1, 1, (ny, nx))
    dh = torch.tensor(hi, device="cuda")
    lo, = half2s(p, 1)
    assert L.amps_graingrowth_highdata_to_low(pp, ptr(dh), ptr(lo), None) == 0
    want = hi.astype(np.float32).astype(np.float16)
    assert np.array_equal(lo.cpu().numpy().view(np.float16), want)
    last = torch.zeros_like(dh)
    assert L.amps_graingrowth_monitor2_lastdata_store(pp, ptr(dh), ptr(last), None) == 0
    assert np.array_equal(last.cpu().numpy(), hi)
    ty = rng.integers(1, 3, (ny // T, nx // T)).astype(np.int32)
    dty = torch.tensor(ty, device="cuda")
    for step in (3, 9):
        out = torch.full_like(dh, 7.0)
        assert L.amps_graingrowth_kernel1_conversion(pp, ptr(out), ptr(lo), ptr(dty), step, None) == 0
        exp = np.full((ny, nx), 7.0)
        cell = want.astype(np.float64)
        yy, xx = np.mgrid[0:ny, 0:nx]
        low_tile = ty[yy // T, xx // T] == 1
        yo, xo = yy % T, xx % T
        conv = low_tile & ((yo == 0) | (yo == T - 1) | ((step + 1) % 10 == 0) | (xo == 0) | (xo == T - 1))
        exp[conv] = cell[conv]
        assert np.array_equal(out.cpu().numpy(), exp), step


def kob_mix_lib():
    L = mix_lib()
    dp = ctypes.POINTER(w().Params)
    I = ctypes.c_int
    sig = {
        "amps_snowflake_kernel1_mix": [P] * 18 + [I],
        "amps_snowflake_mix_kernel2": [P] * 17 + [I],
        "amps_snowflake_dataprepare_high": [P],
        "amps_snowflake_data_sychro_duringcomputation": [P] * 6,
        "amps_snowflake_data_sychro_aftercomputation": [P] * 3,
        "amps_snowflake_kernel2_conversion": [P] * 5 + [I],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = [dp] + args + [P]
        f.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("monitor,thr,steps", [(1, 0.5, 200), (1, 0.1, 120), (2, 1e-4, 200), (2, 1e-2, 120)])
def test_kobayashi_mixed_loop_equals_the_reference_kernels(monitor, thr, steps):
    """snowflake/end2end_mix.cu's loop (AMSTENCIL, Monitor1/2) through the
    reference-named wrappers -- the seed disc, per period get_max_diff /
    get_type / data_sychro_duringcomputation, kernel1_mix and mix_kernel2 a
    step, the final data_sychro_aftercomputation -- against the reference's
    own kernels driven the same way: tile types of every period and the
    final phi and tempr, bit for bit."""
    need(f"snowflake_mix_m{monitor}")
    L = kob_mix_lib()
    p = w().Params.preset("kobayashi", 2, mode="end2end_mix", monitor=monitor, thr_lo=thr, thr_hi=thr)
    with refcuda.Module(f"snowflake_mix_m{monitor}") as m:
        assert (m.nx, m.ny, m.ux, m.uy) == (p.nx, p.ny, p.tile, p.tile)
    pp = ctypes.byref(p)
    nx, ny, T = p.nx, p.ny, p.tile
    tiles = (nx // T) * (ny // T)
    f64 = lambda: torch.zeros((ny, nx), dtype=torch.float64, device="cuda")
    phi, plap, eps, epsd, pdx, pdy, tem, tlap, last = (f64() for _ in range(9))
    hphi, hplap, htem, htlap, hpdx, hpdy, heps, hepsd = half2s(p, 8)
    tcur = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    told = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    md = torch.zeros(tiles, dtype=torch.float64, device="cuda")
    assert L.amps_snowflake_dataprepare_high(pp, ptr(phi), None) == 0
    assert L.amps_snowflake_dataprepare_half2(pp, ptr(hphi), None) == 0
    if monitor == 2:  # end2end_mix.cu:42-46
        last.copy_((phi == 0).double())
    types = []
    for i in range(steps):
        if i % 10 == 0:
            if monitor == 1:
                assert L.amps_get_max_diff1(pp, ptr(phi), ptr(md), None) == 0
            else:
                assert L.amps_get_max_diff2(pp, ptr(last), ptr(phi), ptr(md), None) == 0
            assert L.amps_get_type(pp, ptr(md), ptr(told), ptr(tcur), None) == 0
            assert L.amps_snowflake_data_sychro_duringcomputation(pp, ptr(phi), ptr(tem), ptr(hphi), ptr(htem),
                                                                  ptr(told), ptr(tcur), None) == 0
            types.append(tcur.cpu().numpy().astype(np.uint8))
        assert L.amps_snowflake_kernel1_mix(pp, ptr(phi), ptr(last), ptr(plap), ptr(eps), ptr(epsd), ptr(pdx),
                                            ptr(pdy), ptr(tem), ptr(tlap), ptr(hphi), ptr(hplap), ptr(htem),
                                            ptr(htlap), ptr(hpdx), ptr(hpdy), ptr(heps), ptr(hepsd), ptr(tcur), i,
                                            None) == 0
        assert L.amps_snowflake_mix_kernel2(pp, ptr(phi), ptr(plap), ptr(eps), ptr(epsd), ptr(pdx), ptr(pdy),
                                            ptr(tem), ptr(tlap), ptr(hphi), ptr(hplap), ptr(heps), ptr(hepsd),
                                            ptr(hpdx), ptr(hpdy), ptr(htem), ptr(htlap), ptr(tcur), i, None) == 0
    assert L.amps_snowflake_data_sychro_aftercomputation(pp, ptr(phi), ptr(hphi), ptr(tcur), None) == 0
    assert L.amps_snowflake_data_sychro_aftercomputation(pp, ptr(tem), ptr(htem), ptr(tcur), None) == 0
    torch.cuda.synchronize()
    rp, rt, rtypes, _ = refcuda.kob_mix(steps, thr, monitor)
    ours = np.stack(types)
    mix = np.bincount(ours.ravel(), minlength=3)[1:] / ours.size
    bad = [k for k in range(rtypes.shape[0]) if not np.array_equal(ours[k], rtypes[k])]
    fp, ft = phi.cpu().numpy(), tem.cpu().numpy()
    d = max(float(np.abs(fp - rp).max()), float(np.abs(ft - rt).max()))
    print(f"kobayashi mixed loop, monitor {monitor} {thr:g}, {steps} steps: tile types half/FP64 {mix}, "
          f"periods differing {bad[:5]}, fields max |diff| {d:.3e}")
    assert not bad
    assert np.array_equal(fp, rp) and np.array_equal(ft, rt)


def test_kobayashi_kernel2_conversion():
    """kernel2_conversion against a numpy statement of
    snowflake/function.h:760-790 on random half2 data and tile types."""
    L = kob_mix_lib()
    p = w().Params.preset("kobayashi", 2, mode="end2end_mix")
    pp = ctypes.byref(p)
    nx, ny, T = p.nx, p.ny, p.tile
    rng = np.random.default_rng(4)
    hp = rng.uniform(-1, 1, (ny, nx)).astype(np.float16)
    ht = rng.uniform(-1, 1, (ny, nx)).astype(np.float16)
    dhp = torch.tensor(hp.view(np.int32), device="cuda")
    dht = torch.tensor(ht.view(np.int32), device="cuda")
    ty = rng.integers(1, 3, (ny // T, nx // T)).astype(np.int32)
    dty = torch.tensor(ty, device="cuda")
    for step in (3, 9):
        fp = torch.full((ny, nx), 7.0, dtype=torch.float64, device="cuda")
        ft = torch.full((ny, nx), 7.0, dtype=torch.float64, device="cuda")
        assert L.amps_snowflake_kernel2_conversion(pp, ptr(fp), ptr(ft), ptr(dhp), ptr(dht), ptr(dty), step,
                                                   None) == 0
        yy, xx = np.mgrid[0:ny, 0:nx]
        yo, xo = yy % T, (xx % T) // 2
        band = (ty[yy // T, xx // T] == 1) & ((yo < 2) | (yo + 2 > T - 1) | (xo == 0) | (xo == T // 2 - 1) |
                                              ((step + 1) % 10 == 0))
        for got, src in ((fp, hp), (ft, ht)):
            exp = np.full((ny, nx), 7.0)
            exp[band] = src.astype(np.float64)[band]
            assert np.array_equal(got.cpu().numpy(), exp), step


def sint_mix_lib():
    L = mix_lib()
    dp = ctypes.POINTER(w().Params)
    I = ctypes.c_int
    sig = {
        "amps_sintering_con1_mix": [P] * 14 + [I],
        "amps_sintering_con2_mix": [P] * 11 + [I],
        "amps_sintering_phi1_mix": [P] * 13 + [I],
        "amps_sintering_phi2_mix": [P] * 13 + [I],
        "amps_sintering_data_sychro_duringcomputation": [P] * 8,
        "amps_sintering_dataprepare": [P, P],
        "amps_sintering_data_sychro_aftercomputation": [P] * 3,
        "amps_sintering_con2_conversion": [P, P, P, I],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = [dp] + args + [P]
        f.restype = ctypes.c_int
    return L


@pytest.mark.parametrize("monitor,thr,steps", [(1, 0.5, 200), (2, 1e-4, 200), (2, 1e-2, 120), (1, 0.1, 120)])
def test_sintering_mixed_loop_equals_the_reference_kernels(monitor, thr, steps):
    """sintering/main.cu's AMSTENCIL loop (Monitor1/2) through the
    reference-named wrappers -- dataprepare of the two-particle start, per
    period get_max_diff / get_type / data_sychro_duringcomputation,
    con1/con2/phi1/phi2_mix a step, the final data_sychro_aftercomputation
    -- against the reference's own kernels driven the same way: tile types
    of every period and the final con, eta1, eta2, bit for bit."""
    need("sintering_mix")
    L = sint_mix_lib()
    p = w().Params.preset("sintering", 5, mode="end2end_mix", monitor=monitor, thr_lo=thr, thr_hi=thr)
    with refcuda.Module("sintering_mix") as m:
        assert (m.nx, m.ny, m.ux, m.uy) == (p.nx, p.ny, p.tile, p.tile)
    f0 = w().init_host(p.replace(ref_order=1), w().INIT_REFERENCE)
    pp = ctypes.byref(p)
    nx, ny, T = p.nx, p.ny, p.tile
    tiles = (nx // T) * (ny // T)
    f64 = lambda: torch.zeros((ny, nx), dtype=torch.float64, device="cuda")
    con, e1, e2 = (torch.tensor(np.ascontiguousarray(f0[k]), dtype=torch.float64, device="cuda") for k in range(3))
    last = (con == 0).double()  # main.cu:61-64
    e1o, e2o, clap, l1, l2, mu, mulap, dfc, d1, d2 = (f64() for _ in range(10))
    hc, h1, h2, h1o, h2o, hclap, hl1, hl2, hmu, hmulap, hdfc, hd1, hd2 = half2s(p, 13)
    tcur = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    told = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    md = torch.zeros(tiles, dtype=torch.float64, device="cuda")
    for f, h in ((con, hc), (e1, h1), (e2, h2)):
        assert L.amps_sintering_dataprepare(pp, ptr(f), ptr(h), None) == 0
    types = []
    for i in range(steps):
        if i % 10 == 0:
            if monitor == 1:
                assert L.amps_get_max_diff1(pp, ptr(con), ptr(md), None) == 0
            else:
                assert L.amps_get_max_diff2(pp, ptr(last), ptr(con), ptr(md), None) == 0
            assert L.amps_get_type(pp, ptr(md), ptr(told), ptr(tcur), None) == 0
            assert L.amps_sintering_data_sychro_duringcomputation(pp, ptr(con), ptr(e1), ptr(e2), ptr(hc), ptr(h1),
                                                                  ptr(h2), ptr(told), ptr(tcur), None) == 0
            types.append(tcur.cpu().numpy().astype(np.uint8))
        assert L.amps_sintering_con1_mix(pp, ptr(tcur), ptr(con), ptr(last), ptr(clap), ptr(e1), ptr(e2), ptr(dfc),
                                         ptr(mu), ptr(hc), ptr(hclap), ptr(h1), ptr(h2), ptr(hdfc), ptr(hmu), i,
                                         None) == 0
        assert L.amps_sintering_con2_mix(pp, ptr(tcur), ptr(mu), ptr(mulap), ptr(con), ptr(e1), ptr(e2), ptr(hmu),
                                         ptr(hmulap), ptr(hc), ptr(h1), ptr(h2), i, None) == 0
        assert L.amps_sintering_phi1_mix(pp, ptr(tcur), ptr(e1), ptr(e1o), ptr(e2), ptr(l1), ptr(d1), ptr(con),
                                         ptr(h1), ptr(h1o), ptr(h2), ptr(hl1), ptr(hd1), ptr(hc), i, None) == 0
        assert L.amps_sintering_phi2_mix(pp, ptr(tcur), ptr(e2), ptr(e2o), ptr(e1), ptr(l2), ptr(d2), ptr(con),
                                         ptr(h2), ptr(h2o), ptr(h1), ptr(hl2), ptr(hd2), ptr(hc), i, None) == 0
        e1, e1o, e2, e2o = e1o, e1, e2o, e2
        h1, h1o, h2, h2o = h1o, h1, h2o, h2
    for f, h in ((con, hc), (e1, h1), (e2, h2)):
        assert L.amps_sintering_data_sychro_aftercomputation(pp, ptr(f), ptr(h), ptr(tcur), None) == 0
    torch.cuda.synchronize()
    rc, r1, r2, rtypes, _ = refcuda.sint_mix(steps, thr, monitor, f0[0], f0[1], f0[2])
    ours = np.stack(types)
    mix = np.bincount(ours.ravel(), minlength=3)[1:] / ours.size
    bad = [k for k in range(rtypes.shape[0]) if not np.array_equal(ours[k], rtypes[k])]
    fc, f1, f2 = con.cpu().numpy(), e1.cpu().numpy(), e2.cpu().numpy()
    d = max(float(np.abs(a - b).max()) for a, b in ((fc, rc), (f1, r1), (f2, r2)))
    print(f"sintering mixed loop, monitor {monitor} {thr:g}, {steps} steps: tile types half/FP64 {mix}, "
          f"periods differing {bad[:5]}, fields max |diff| {d:.3e}")
    assert not bad
    assert np.array_equal(fc, rc) and np.array_equal(f1, r1) and np.array_equal(f2, r2)


def test_sintering_con2_conversion():
    """con2_conversion against a numpy statement of
    sintering/function.h:824-853: type-1 tiles' edge cells (all of them at a
    period's last step) into the FP64 array, type-2 tiles' first and last
    columns into the half2 array, in sintering's tile-halves packing."""
    L = sint_mix_lib()
    p = w().Params.preset("sintering", 5, mode="end2end_mix")
    pp = ctypes.byref(p)
    nx, ny, T = p.nx, p.ny, p.tile
    th = T // 2
    rng = np.random.default_rng(6)
    hv = rng.uniform(0, 1, (ny, nx)).astype(np.float16)  # pair-major: [y][pair][low, high]
    fv = rng.uniform(0, 1, (ny, nx))
    ty = rng.integers(1, 3, (ny // T, nx // T)).astype(np.int32)
    dty = torch.tensor(ty, device="cuda")
    yy, pp_ = np.mgrid[0:ny, 0:nx // 2]
    tx, xo = pp_ // th, pp_ % th
    lo_cell, hi_cell = tx * T + xo, tx * T + xo + th
    for step in (3, 9):
        dh = torch.tensor(hv.view(np.int32).copy(), device="cuda")
        df = torch.tensor(fv, device="cuda")
        assert L.amps_sintering_con2_conversion(pp, ptr(dty), ptr(df), ptr(dh), step, None) == 0
        ef, eh = fv.copy(), hv.copy().reshape(ny, nx // 2, 2)
        low = ty[yy // T, tx] == 1
        yo = yy % T
        full = low & ((yo == 0) | (yo == T - 1) | ((step + 1) % 10 == 0))
        pairs = hv.reshape(ny, nx // 2, 2).astype(np.float64)
        for mask, cell, half in ((full | (low & (xo == 0)), lo_cell, 0), (full | (low & (xo == th - 1)), hi_cell, 1)):
            ef[yy[mask], cell[mask]] = pairs[..., half][mask]
        high = ~low
        first = high & (xo == 0)
        eh[yy[first], pp_[first], 0] = fv[yy[first], lo_cell[first]].astype(np.float32).astype(np.float16)
        last = high & (xo == th - 1)
        eh[yy[last], pp_[last], 1] = fv[yy[last], hi_cell[last]].astype(np.float32).astype(np.float16)
        assert np.array_equal(df.cpu().numpy(), ef), step
        assert np.array_equal(dh.cpu().numpy().view(np.float16).reshape(ny, nx // 2, 2), eh), step
