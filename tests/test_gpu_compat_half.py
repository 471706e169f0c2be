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
