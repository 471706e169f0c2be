"""The reference's own CUDA kernels on the GPU (baseline/_ref/): its device
code built in place from the reference tree into cubins, driven by
baseline/ref_cuda.cpp's restatement of its host time loops.  Used to time the
reference beside the library on the same GPU and to compare its results; not
part of the library.

Each cubin fixes the reference's compile-time sizes and constants (its
parameter file): graingrowth_pure / graingrowth_mix_m{1,2} are
graingrowth/paras/para1.h (512 x 512, 16 x 16 tiles, Q = 2), snowflake_pure /
snowflake_mix_m{1,2} snowflake/paras/para2.h (512 x 512, 16 x 16 tiles),
sintering_pure / sintering_mix sintering/paras/para5.h (512 x 512, 16 x 16
tiles, two particles; the initial state comes from the caller);
graingrowth_purelow / snowflake_purelow the shipped header state (HALF2,
float constants) with para1 / para2."""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
_lib = None


def available(name):
    """The cubin `name` (e.g. "graingrowth_pure") and the host driver are built."""
    return os.path.exists(os.path.join(REF, name + ".cubin")) and os.path.exists(os.path.join(REF, "libref_cuda.so"))


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(os.path.join(REF, "libref_cuda.so"))
        L.refcuda_error.restype = ctypes.c_char_p
        L.refcuda_open.restype = ctypes.c_void_p
        L.refcuda_open.argtypes = [ctypes.c_char_p]
        L.refcuda_close.argtypes = [ctypes.c_void_p]
        L.refcuda_dims.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.refcuda_gg_pure.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, fp]
        L.refcuda_gg_mix.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp,
                                     ctypes.c_void_p, fp]
        L.refcuda_kob_pure.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, fp]
        L.refcuda_kob_mix.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp,
                                      ctypes.c_void_p, fp]
        L.refcuda_sint_pure.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, fp]
        L.refcuda_sint_mix.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp, dp,
                                       ctypes.c_void_p, fp]
        up = ctypes.POINTER(ctypes.c_uint32)
        L.refcuda_gg_purelow.argtypes = [ctypes.c_void_p, ctypes.c_int, up, up, fp]
        L.refcuda_kob_purelow.argtypes = [ctypes.c_void_p, ctypes.c_int, up, up, fp]
        _lib = L
    return _lib


class Module:
    """One of the reference's cubins, loaded into the device's primary context."""

    def __init__(self, name):
        self.h = lib().refcuda_open(os.path.join(REF, name + ".cubin").encode())
        if not self.h:
            raise RuntimeError(f"{name}: {lib().refcuda_error().decode()}")
        d = np.zeros(4, dtype=np.int32)
        lib().refcuda_dims(self.h, d.ctypes.data)
        self.nx, self.ny, self.ux, self.uy = (int(v) for v in d)
        self.tiles = (self.nx // self.ux) * (self.ny // self.uy)

    def close(self):
        if self.h:
            lib().refcuda_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc, what):
        if rc:
            raise RuntimeError(f"{what}: {lib().refcuda_error().decode()}")


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def gg_pure(steps):
    """graingrowth/purehigh.cu for `steps` steps: (eta1, eta2, ms from step 5)."""
    with Module("graingrowth_pure") as m:
        e1, e2 = np.zeros((m.ny, m.nx)), np.zeros((m.ny, m.nx))
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_gg_pure(m.h, steps, _p(e1), _p(e2), ctypes.byref(ms)), "refcuda_gg_pure")
        return e1, e2, float(ms.value)


def gg_mix(steps, thr, monitor):
    """graingrowth/end2end_mix.cu (AMSTENCIL, Monitor1/2) for `steps` steps at
    threshold `thr`: (eta1, eta2, types [periods][tiles] (1 half2, 2 high),
    ms from step 5)."""
    with Module(f"graingrowth_mix_m{monitor}") as m:
        e1, e2 = np.zeros((m.ny, m.nx)), np.zeros((m.ny, m.nx))
        types = np.zeros(((steps + 9) // 10, m.tiles), dtype=np.uint8)
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_gg_mix(m.h, steps, thr, monitor, _p(e1), _p(e2), types.ctypes.data, ctypes.byref(ms)),
              "refcuda_gg_mix")
        return e1, e2, types, float(ms.value)


def kob_pure(steps):
    """snowflake/purehigh.cu for `steps` steps: (phi, T, ms from step 5)."""
    with Module("snowflake_pure") as m:
        phi, t = np.zeros((m.ny, m.nx)), np.zeros((m.ny, m.nx))
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_kob_pure(m.h, steps, _p(phi), _p(t), ctypes.byref(ms)), "refcuda_kob_pure")
        return phi, t, float(ms.value)


def kob_mix(steps, thr, monitor):
    """snowflake/end2end_mix.cu (AMSTENCIL, Monitor1/2) for `steps` steps at
    threshold `thr`: (phi, T, types [periods][tiles] (1 half2, 2 high), ms
    from step 5)."""
    with Module(f"snowflake_mix_m{monitor}") as m:
        phi, t = np.zeros((m.ny, m.nx)), np.zeros((m.ny, m.nx))
        types = np.zeros(((steps + 9) // 10, m.tiles), dtype=np.uint8)
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_kob_mix(m.h, steps, thr, monitor, _p(phi), _p(t), types.ctypes.data, ctypes.byref(ms)),
              "refcuda_kob_mix")
        return phi, t, types, float(ms.value)


def sint_pure(steps, c, e1, e2):
    """sintering/main.cu (PURE) for `steps` steps from (c, e1, e2):
    (c, e1, e2, ms from step 5)."""
    with Module("sintering_pure") as m:
        c, e1, e2 = (np.array(a, dtype=np.float64, copy=True, order="C") for a in (c, e1, e2))
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_sint_pure(m.h, steps, _p(c), _p(e1), _p(e2), ctypes.byref(ms)), "refcuda_sint_pure")
        return c, e1, e2, float(ms.value)


def sint_mix(steps, thr, monitor, c, e1, e2):
    """sintering/main.cu (AMSTENCIL, Monitor1/2) for `steps` steps from
    (c, e1, e2) at threshold `thr`: (c, e1, e2, types [periods][tiles]
    (1 half2, 2 high), ms from step 5)."""
    with Module("sintering_mix") as m:
        c, e1, e2 = (np.array(a, dtype=np.float64, copy=True, order="C") for a in (c, e1, e2))
        types = np.zeros(((steps + 9) // 10, m.tiles), dtype=np.uint8)
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_sint_mix(m.h, steps, thr, monitor, _p(c), _p(e1), _p(e2), types.ctypes.data,
                                     ctypes.byref(ms)), "refcuda_sint_mix")
        return c, e1, e2, types, float(ms.value)


def _u(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def gg_purelow(steps):
    """graingrowth/purelow.cu (HALF2) for `steps` steps: (eta1, eta2 as
    uint32 [ny][nx/2] half2 words, ms from step 5)."""
    with Module("graingrowth_purelow") as m:
        e1, e2 = np.zeros((m.ny, m.nx // 2), np.uint32), np.zeros((m.ny, m.nx // 2), np.uint32)
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_gg_purelow(m.h, steps, _u(e1), _u(e2), ctypes.byref(ms)), "refcuda_gg_purelow")
        return e1, e2, float(ms.value)


def kob_purelow(steps):
    """snowflake/purelow.cu (HALF2) for `steps` steps: (phi, T as uint32
    [ny][nx/2] half2 words, ms from step 5)."""
    with Module("snowflake_purelow") as m:
        phi, t = np.zeros((m.ny, m.nx // 2), np.uint32), np.zeros((m.ny, m.nx // 2), np.uint32)
        ms = ctypes.c_float(0)
        m._ck(lib().refcuda_kob_purelow(m.h, steps, _u(phi), _u(t), ctypes.byref(ms)), "refcuda_kob_purelow")
        return phi, t, float(ms.value)
