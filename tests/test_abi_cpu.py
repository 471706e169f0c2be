"""The C ABI without a GPU: the library loads, exports every symbol the
header declares, and its host-only entry points (presets, validation,
initial states) agree with the reference-derived oracle."""
import os
import re

import numpy as np
import pytest

import oracle_bind as ob

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def amps():
    import w3914777_gb300 as w
    return w


def declared_symbols():
    src = "".join(open(os.path.join(ROOT, "include", h)).read() for h in ("amps.h", "amps_compat.h"))
    return sorted(set(re.findall(r"AMPS_API[^;(]*?\b(amps_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    w = amps()
    L = w.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert L.amps_abi_version() == 2


def test_status_strings_and_errors_never_exit():
    w = amps()
    L = w.lib()
    assert L.amps_status_string(0) == b"ok"
    assert b"invalid" in L.amps_status_string(1)
    p = w.Params.preset("kobayashi", 2, nx=100)  # not a multiple of the tile
    rc, msg = p.check()
    assert rc == 1 and "multiples" in msg
    with pytest.raises(w.AmpsError) as e:
        w.Simulation(p)
    assert e.value.status == 1


def test_ragged_sides_grain_growth_only():
    """Sides that are not multiples of the tile: grain growth computes the
    partial edge tiles' valid cells; Kobayashi and sintering, the binary16
    half-tile arithmetic and the reference's snapshot rule need whole tiles."""
    w = amps()
    gg = w.Params.preset("graingrowth", 0, nx=100, ny=77, nfields=4)
    assert gg.check()[0] == 0
    assert gg.replace(nx=33, ny=33, tile=32).check()[0] == 0
    assert gg.replace(nx=31).check()[0] == 1                    # below one tile
    assert gg.replace(half_arith=w.HALF_REF).check()[0] == 1
    assert gg.replace(half_arith=w.HALF_HFMA2).check()[0] == 1
    assert gg.replace(ref_snapshot=1).check()[0] == 1
    assert gg.replace(nx=96, ny=64, half_arith=w.HALF_REF).check()[0] == 0
    assert w.Params.preset("sintering", 0, nx=100, ny=96).check()[0] == 1
    # the tile limit counts the partial tiles
    rc, msg = w.Params.preset("graingrowth", 1, nx=23169, ny=23168, tile=16).check()
    assert rc == 1 and "too many tiles" in msg


def test_tile_count_limit():
    """The classification's packed counters hold 21 bits per tier, so a grid
    of more than 0x1FFFFF tiles is rejected before any allocation."""
    w = amps()
    # 16^2 tiles: 23168^2 / 256 = 2,096,704 tiles fits; 23184^2 (2,099,601) does not
    ok = w.Params.preset("graingrowth", 1, nx=23168, ny=23168, tile=16)
    assert ok.check()[0] == 0
    big = w.Params.preset("graingrowth", 1, nx=23184, ny=23184, tile=16)
    rc, msg = big.check()
    assert rc == 1 and "too many tiles" in msg
    # the same grid with 32^2 tiles is a quarter of the count and is accepted
    assert big.replace(tile=32, nx=23200, ny=23200).check()[0] == 0


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_presets_mirror_reference_parameter_files(k):
    w = amps()
    kob = w.Params.preset("kobayashi", k)
    assert (kob.nx, kob.ny, kob.tile, kob.cadence) == (512, 512, 16, 10)  # snowflake/paras/total.h:20-21
    assert kob.aniso == [4.0, 6.0, 5.0, 6.0, 4.0][k - 1]                # snowflake/paras/para*.h
    assert kob.theta0 == [0.0, 0.0, 0.0, 0.4, 0.25][k - 1]
    gg = w.Params.preset("graingrowth", k)
    assert gg.mobil == [5.0, 10.0, 5.0, 5.0, 20.0][k - 1] and gg.dt == 0.005  # graingrowth/paras/para*.h
    si = w.Params.preset("sintering", k)
    assert si.coefm == [5.0, 5.0, 20.0, 20.0, 20.0][k - 1] and si.dsur == [32, 64, 16, 16, 64][k - 1]
    if ob.ref_available("snowflake") and k == 2:
        rp = ob.ref_params("snowflake", 14)
        assert [kob.dx, kob.dy, kob.tau, kob.epsb, kob.kappa, kob.delta, kob.aniso, kob.alpha, kob.gama,
                kob.teq, kob.theta0, kob.dt, kob.pi] == list(rp[:13])


def test_reference_initial_states_match_oracle():
    w = amps()
    f = w.init_host(w.Params.preset("kobayashi", 2), w.INIT_REFERENCE)
    a, _ = ob.kob_init_disc(512, 512, 264, 264, 10.0)
    assert np.array_equal(f[0], a) and not f[1].any()
    f = w.init_host(w.Params.preset("graingrowth", 1), w.INIT_REFERENCE)
    a, b = ob.gg_init_circle(512, 512, 256, 256, 50)
    assert np.array_equal(f[0], a) and np.array_equal(f[1], b)
    f = w.init_host(w.Params.preset("sintering", 5), w.INIT_REFERENCE)
    c, e1, e2 = ob.sint_init_two(512, 512, 264, 240, 20, 270, 10)
    assert np.array_equal(f[0], c) and np.array_equal(f[1], e1) and np.array_equal(f[2], e2)


def test_seeded_states():
    w = amps()
    p = w.Params.preset("graingrowth", 0, nx=128, ny=64)
    f = w.init_host(p, w.INIT_SEEDED)
    assert f.shape == (8, 64, 128) and np.abs(f).max() <= 1e-3 and abs(f.mean()) < 5e-5
    # same RNG as the oracle's counter-based generator
    u = ob.lib().orc_uniform01(p.seed, 3, 77)
    assert f[3].ravel()[77] == p.init_amp * (2 * u - 1)
    s = w.Params.preset("sintering", 0)
    g = w.init_host(s, w.INIT_SEEDED)
    assert g.shape == (17, 1024, 1024)
    eta = g[1:]
    assert set(np.unique(eta)) <= {0.0, 1.0} and eta.sum(0).max() == 1.0   # one particle per cell
    assert np.array_equal(g[0], eta.sum(0))                                # c = 1 inside particles
    assert all(eta[k].sum() > 1000 for k in range(16))                     # all 16 placed, r >= 20
    assert np.array_equal(g, w.init_host(s, w.INIT_SEEDED))                # deterministic


def test_stochastic_half_rounding_is_a_kobayashi_option():
    w = amps()
    assert w.Params.preset("kobayashi", 2, mode="end2end_mix", half_arith=w.HALF_SR).check()[0] == 0
    assert w.Params.preset("graingrowth", 0, half_arith=w.HALF_SR).check()[0] == 1
    assert w.Params.preset("sintering", 0, half_arith=w.HALF_SR).check()[0] == 1
    assert w.Params.preset("kobayashi", 2, half_arith=4).check()[0] == 1


# the reference-named half2 and adaptive wrappers: (name, pointer arguments, trailing ints)
_WRAPPERS = [
    ("amps_graingrowth_kernel1_lowpure", 5, 0), ("amps_graingrowth_dataprepare_half2", 2, 0),
    ("amps_snowflake_kernel1_purelow", 8, 0), ("amps_snowflake_kernel2_purelow", 8, 0),
    ("amps_graingrowth_kernel1_mix", 12, 2), ("amps_graingrowth_data_sychro_duringcomputation", 6, 0),
    ("amps_graingrowth_data_sychro_aftercomputation", 3, 0), ("amps_graingrowth_highdata_to_low", 2, 0),
    ("amps_graingrowth_kernel1_conversion", 3, 1), ("amps_graingrowth_monitor2_lastdata_store", 2, 0),
    ("amps_snowflake_kernel1_mix", 18, 1), ("amps_snowflake_mix_kernel2", 17, 1),
    ("amps_snowflake_kernel2_conversion", 5, 1),
    ("amps_sintering_con1_mix", 14, 1), ("amps_sintering_con2_mix", 11, 1), ("amps_sintering_phi1_mix", 13, 1),
    ("amps_sintering_phi2_mix", 13, 1), ("amps_sintering_con2_conversion", 3, 1),
    ("amps_sintering_data_sychro_duringcomputation", 8, 0), ("amps_sintering_dataprepare", 2, 0),
    ("amps_sintering_data_sychro_aftercomputation", 3, 0),
]


@pytest.mark.parametrize("name,nptr,nint", _WRAPPERS)
def test_reference_named_wrappers_validate_before_any_launch(name, nptr, nint):
    """Every half2 / adaptive wrapper refuses, before touching the device, a
    grid it cannot run (odd nx, zero-flux, a tile that does not divide the
    sides or is above 32) and a null array: AMPS_ERR_INVALID (1)."""
    import ctypes
    w = amps()
    f = getattr(w.lib(), name)
    f.argtypes = [ctypes.POINTER(w.Params)] + [ctypes.c_void_p] * nptr + [ctypes.c_int] * nint + [ctypes.c_void_p]
    f.restype = ctypes.c_int
    model = "sintering" if "sintering" in name else ("kobayashi" if "snowflake" in name else "graingrowth")
    preset = {"sintering": 5, "kobayashi": 2, "graingrowth": 1}[model]
    fake = [ctypes.c_void_p(256 * (k + 1)) for k in range(nptr)]  # never dereferenced on the host
    ints = [0] * nint
    bad = [dict(nx=510), dict(nx=511), dict(bc=w.BC_NOFLUX), dict(tile=12), dict(tile=64)]
    if "lowpure" in name or "purelow" in name or "half2" in name:
        bad = [dict(nx=511), dict(bc=w.BC_NOFLUX)]  # untiled: any even periodic grid
    for kw in bad:
        p = w.Params.preset(model, preset, **kw)
        assert f(ctypes.byref(p), *fake, *ints, None) == 1, kw
    p = w.Params.preset(model, preset)
    for k in range(nptr):
        if name in ("amps_graingrowth_kernel1_mix", "amps_snowflake_kernel1_mix", "amps_sintering_con1_mix") and k == (
                1 if "sintering" not in name else 2):
            continue  # the snapshot array may be null unless the temporal monitor is on
        args = list(fake)
        args[k] = None
        assert f(ctypes.byref(p), *args, *ints, None) == 1, (name, k)
