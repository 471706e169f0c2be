"""ctypes bindings to the CPU FP64 oracle (oracle/liboracle.so) and to the
reference's own plain kernels compiled for the CPU (oracle/_ref/*.so).

Test infrastructure only: the oracle is the checker, never the product.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")

_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class KobParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("bc", ctypes.c_int)] + [
        (n, ctypes.c_double)
        for n in ("dx", "dy", "tau", "epsb", "kappa", "delta", "aniso", "alpha", "gama", "teq",
                  "theta0", "dt", "pi", "noise")
    ] + [("seed", ctypes.c_uint64)]


class GGParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("bc", ctypes.c_int), ("q", ctypes.c_int),
                ("stencil", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("dx", "dy", "dt", "mobil", "grcoef", "gamma")]


class SintParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("bc", ctypes.c_int), ("n", ctypes.c_int)] + [
        (n, ctypes.c_double)
        for n in ("dx", "dy", "dt", "coefm", "coefk", "coefl", "dvol", "dvap", "dsur", "dgrb", "A", "B")]


def ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def ptr_array(arrs):
    t = (_dp * len(arrs))(*[ptr(a) for a in arrs])
    return t


_libs = {}


def build_oracle(target="liboracle.so"):
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, target], check=True)


def lib(fast=False):
    """The oracle library.  fast=False: the checker (-O2, no fused
    multiply-add: the reference's rounding); fast=True: the same source at -O3
    with fused multiply-add, the timed CPU baseline (never a checker)."""
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name not in _libs:
        path = os.path.join(ORACLE_DIR, name)
        if not os.path.exists(path):
            build_oracle(name)
        L = ctypes.CDLL(path)
        L.orc_kob_step.argtypes = [ctypes.POINTER(KobParams), _dp, _dp, _dp, ctypes.c_int64]
        L.orc_kob_init_disc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, _dp, _dp]
        L.orc_gg_step.argtypes = [ctypes.POINTER(GGParams), ctypes.c_void_p, ctypes.c_void_p]
        L.orc_gg_step_fast.argtypes = [ctypes.POINTER(GGParams), ctypes.c_void_p, ctypes.c_void_p]
        L.orc_gg_init_circle.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, _dp, _dp]
        L.orc_sint_step.argtypes = [ctypes.POINTER(SintParams), _dp, ctypes.c_void_p, ctypes.c_void_p, _dp]
        L.orc_sint_init_two.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 5 + [_dp, _dp, _dp]
        L.orc_monitor_spa.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]
        L.orc_monitor_tem.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]
        L.orc_monitor_rate.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, _dp]
        L.orc_classify.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _u8p]
        L.orc_uniform01.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_uniform01.restype = ctypes.c_double
        L.orc_hash3.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_hash3.restype = ctypes.c_uint64
        L.orc_gg_init_uniform.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_uint64, ctypes.c_void_p]
        _libs[name] = L
    return _libs[name]


# ------------------------------------------------------------ Kobayashi ----
def kob_params(nx, ny, bc=0, **kw):
    """Reference para2 (snowflake/paras/para2.h) unless overridden."""
    d = dict(dx=0.03, dy=0.03, tau=0.0003, epsb=0.01, kappa=1.8, delta=0.02, aniso=6.0, alpha=0.9,
             gama=10.0, teq=1.0, theta0=0.0, dt=1.0e-4, pi=3.1415926, noise=0.0, seed=0)
    d.update(kw)
    return KobParams(nx=nx, ny=ny, bc=bc, **d)


def kob_run(p, phi, T, steps, step0=0, fast=False):
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    T = np.ascontiguousarray(T, dtype=np.float64).copy()
    s = np.zeros(6 * p.nx * p.ny)
    L = lib(fast)
    for k in range(steps):
        L.orc_kob_step(ctypes.byref(p), ptr(phi), ptr(T), ptr(s), step0 + k)
    return phi, T


def kob_init_disc(nx, ny, cx, cy, r2):
    phi = np.zeros((ny, nx))
    T = np.zeros((ny, nx))
    lib().orc_kob_init_disc(nx, ny, cx, cy, r2, ptr(phi), ptr(T))
    return phi, T


# --------------------------------------------------------- grain growth ----
def gg_params(nx, ny, q=2, bc=0, stencil=0, **kw):
    """Reference para1 (graingrowth/paras/para1.h) unless overridden."""
    d = dict(dx=0.5, dy=0.5, dt=0.005, mobil=5.0, grcoef=0.1, gamma=1.0)
    d.update(kw)
    return GGParams(nx=nx, ny=ny, bc=bc, q=q, stencil=stencil, **d)


def gg_run(p, etas, steps, fast=False):
    """steps of the grain-growth update; fast=True: the timed baseline's
    restructured loop in the -O3 build (equal to the checker to rounding)."""
    cur = [np.ascontiguousarray(e, dtype=np.float64).copy() for e in etas]
    nxt = [np.empty_like(e) for e in cur]
    L = lib(fast)
    step = L.orc_gg_step_fast if fast else L.orc_gg_step
    for _ in range(steps):
        step(ctypes.byref(p), ctypes.cast(ptr_array(cur), ctypes.c_void_p), ctypes.cast(ptr_array(nxt), ctypes.c_void_p))
        cur, nxt = nxt, cur
    return cur


def gg_init_uniform(nx, ny, q, amp, seed):
    """The seeded multi-grain start: eta_i ~ U[-amp, amp) from (seed, i, cell)."""
    etas = [np.zeros((ny, nx)) for _ in range(q)]
    lib().orc_gg_init_uniform(nx, ny, q, amp, seed, ctypes.cast(ptr_array(etas), ctypes.c_void_p))
    return etas


def gg_init_circle(nx, ny, rx, ry, r):
    e1 = np.zeros((ny, nx))
    e2 = np.zeros((ny, nx))
    lib().orc_gg_init_circle(nx, ny, rx, ry, r, ptr(e1), ptr(e2))
    return e1, e2


# ------------------------------------------------------------ sintering ----
def sint_params(nx, ny, n=2, bc=0, **kw):
    """Reference para5 (sintering/paras/para5.h) unless overridden."""
    d = dict(dx=0.5, dy=0.5, dt=1.0e-4, coefm=20.0, coefk=2.0, coefl=5.0, dvol=0.040, dvap=0.002,
             dsur=64.0, dgrb=1.6, A=16.0, B=1.0)
    d.update(kw)
    return SintParams(nx=nx, ny=ny, bc=bc, n=n, **d)


def sint_run(p, c, etas, steps):
    c = np.ascontiguousarray(c, dtype=np.float64).copy()
    cur = [np.ascontiguousarray(e, dtype=np.float64).copy() for e in etas]
    nxt = [np.empty_like(e) for e in cur]
    s = np.zeros(3 * p.nx * p.ny)
    for _ in range(steps):
        lib().orc_sint_step(ctypes.byref(p), ptr(c), ctypes.cast(ptr_array(cur), ctypes.c_void_p),
                            ctypes.cast(ptr_array(nxt), ctypes.c_void_p), ptr(s))
        cur, nxt = nxt, cur
    return c, cur


def sint_init_two(nx, ny, rx1, ry1, r1, ry2, r2):
    c = np.zeros((ny, nx))
    e1 = np.zeros((ny, nx))
    e2 = np.zeros((ny, nx))
    lib().orc_sint_init_two(nx, ny, rx1, ry1, r1, ry2, r2, ptr(c), ptr(e1), ptr(e2))
    return c, e1, e2


# -------------------------------------------------------------- monitor ----
def _ntiles(nx, ny, tile):
    return -(-ny // tile), -(-nx // tile)  # partial edge tiles on ragged sides


def monitor_spa(f, tile, samples=0):
    ny, nx = f.shape
    m = np.zeros(_ntiles(nx, ny, tile))
    lib().orc_monitor_spa(ptr(np.ascontiguousarray(f)), nx, ny, tile, samples, ptr(m))
    return m


def monitor_tem(f, last, tile, samples=0):
    ny, nx = f.shape
    m = np.zeros(_ntiles(nx, ny, tile))
    lib().orc_monitor_tem(ptr(np.ascontiguousarray(f)), ptr(np.ascontiguousarray(last)), nx, ny, tile,
                          samples, ptr(m))
    return m


def monitor_rate(f, prev, tile, cadence, samples=0):
    ny, nx = f.shape
    m = np.zeros(_ntiles(nx, ny, tile))
    lib().orc_monitor_rate(ptr(np.ascontiguousarray(f)), ptr(np.ascontiguousarray(prev)), nx, ny, tile, samples,
                           cadence, ptr(m))
    return m


def classify(metric, thr_lo, thr_hi):
    nty, ntx = metric.shape
    out = np.zeros(nty * ntx, dtype=np.uint8)
    lib().orc_classify(ptr(np.ascontiguousarray(metric, dtype=np.float64)), ntx, nty, thr_lo, thr_hi,
                       out.ctypes.data_as(_u8p))
    return out.reshape(nty, ntx)


# ------------------------------------------------- reference on the CPU ----
def ref_available(name):
    return os.path.exists(os.path.join(REF_DIR, f"libref_{name}.so"))


def ref_lib(name):
    L = ctypes.CDLL(os.path.join(REF_DIR, f"libref_{name}.so"))
    return L


def ref_params(name, count):
    L = ref_lib(name)
    out = np.zeros(count)
    getattr(L, {"snowflake": "ref_snowflake_params", "graingrowth": "ref_gg_params",
                "sintering": "ref_sint_params"}[name])(ptr(out))
    return out
