"""Python mirror of the libamps C ABI (include/amps.h).

The reference's user-facing surface is its per-app driver programs
(snowflake/purehigh.cu, snowflake/purelow.cu, snowflake/end2end_mix.cu and
their graingrowth/sintering twins) plus compile-time parameter headers
(snowflake/paras/*.h).  Here the same path is a `Simulation` object over a
libamps handle: `Params.preset(model, k)` stands for paras/paraK.h,
`Simulation.init()` for the dataprepare_* kernels, `run(n)` for the driver's
time loop, `field(i)` for the CSV read-back.

There is no fallback: if libamps.so has not been built, importing the
library raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libamps.so")

KOBAYASHI, GRAINGROWTH, SINTERING = 0, 1, 2
PUREHIGH, PURELOW, END2END_MIX, GRAM1, GRAM2 = 0, 1, 2, 3, 4
TIER_HALF, TIER_FP32, TIER_FP64 = 0, 1, 2
BC_PERIODIC, BC_NOFLUX = 0, 1
MONITOR_SPA, MONITOR_TEM, MONITOR_RATE = 1, 2, 3
HALF_FP32, HALF_REF, HALF_HFMA2, HALF_SR = 0, 1, 2, 3
F64, F32 = 0, 1
INIT_REFERENCE, INIT_SEEDED = 0, 1
REDUCE_SUM, REDUCE_MIN, REDUCE_MAX, REDUCE_SUMSQ = 0, 1, 2, 3

MODEL_NAMES = {"kobayashi": KOBAYASHI, "snowflake": KOBAYASHI, "graingrowth": GRAINGROWTH,
               "sintering": SINTERING}
MODE_NAMES = {"purehigh": PUREHIGH, "purelow": PURELOW, "end2end_mix": END2END_MIX, "gram1": GRAM1,
              "gram2": GRAM2}

_INT_FIELDS = ["model", "mode", "nx", "ny", "nfields", "bc", "tile", "high_tier", "monitor", "monitor_samples",
               "monitor_field", "cadence", "stencil", "ref_order", "mu_lap_fp64", "max_log"]
_DBL_FIELDS = ["thr_lo", "thr_hi", "gram_ratio", "dx", "dy", "dt", "tau", "epsb", "kappa", "delta", "aniso",
               "alpha", "gama", "teq", "theta0", "pi", "noise", "mobil", "grcoef", "gamma", "coefm", "coefk",
               "coefl", "dvol", "dvap", "dsur", "dgrb", "A", "B", "init_r2", "init_r", "rmin", "rmax",
               "init_amp"]


class Params(ctypes.Structure):
    """amps_params (include/amps.h)."""
    _fields_ = ([(n, ctypes.c_int) for n in _INT_FIELDS] + [(n, ctypes.c_double) for n in _DBL_FIELDS]
                + [("init_offset", ctypes.c_int), ("seed", ctypes.c_uint64), ("half_arith", ctypes.c_int),
                   ("ref_snapshot", ctypes.c_int)])

    @classmethod
    def preset(cls, model, preset=0, **overrides):
        if isinstance(model, str):
            model = MODEL_NAMES[model]
        p = cls()
        _check(lib().amps_preset(model, preset, ctypes.byref(p)), None, "amps_preset")
        for k, v in overrides.items():
            if k == "mode" and isinstance(v, str):
                v = MODE_NAMES[v]
            if not hasattr(p, k):
                raise AttributeError(f"amps_params has no field {k!r}")
            setattr(p, k, v)
        return p

    def replace(self, **kw):
        q = Params()
        ctypes.pointer(q)[0] = self
        for k, v in kw.items():
            if k == "mode" and isinstance(v, str):
                v = MODE_NAMES[v]
            setattr(q, k, v)
        return q

    def check(self):
        buf = ctypes.create_string_buffer(256)
        rc = lib().amps_check_params(ctypes.byref(self), buf, 256)
        return rc, buf.value.decode()

    @property
    def num_fields(self):
        return lib().amps_num_fields(ctypes.byref(self))

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("tile_steps", ctypes.c_int64 * 3), ("monitor_evals", ctypes.c_int64),
                ("promotions", ctypes.c_int64), ("demotions", ctypes.c_int64), ("tiles", ctypes.c_int32),
                ("numeric_error", ctypes.c_int32), ("kernel_launches", ctypes.c_int64)]

    def as_dict(self):
        return {"steps": self.steps, "tile_steps": list(self.tile_steps), "monitor_evals": self.monitor_evals,
                "promotions": self.promotions, "demotions": self.demotions, "tiles": self.tiles,
                "numeric_error": self.numeric_error}


class AmpsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None


def lib():
    """The loaded libamps.so; raises if it was never built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m w3914777_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        P = ctypes.POINTER(Params)
        sig = {
            "amps_abi_version": ([], ip), "amps_status_string": ([ip], ctypes.c_char_p),
            "amps_last_error": ([vp], ctypes.c_char_p), "amps_preset": ([ip, ip, P], ip),
            "amps_check_params": ([P, ctypes.c_char_p, ctypes.c_size_t], ip), "amps_num_fields": ([P], ip),
            "amps_create": ([P, ctypes.POINTER(vp)], ip), "amps_destroy": ([vp], ip),
            "amps_set_stream": ([vp, vp], ip), "amps_synchronize": ([vp], ip), "amps_init": ([vp, ip], ip),
            "amps_init_host": ([P, ip, vp], ip), "amps_set_field": ([vp, ip, vp, ip, ip], ip),
            "amps_get_field": ([vp, ip, vp, ip, ip], ip), "amps_set_fields": ([vp, vp, ip, ip], ip),
            "amps_get_fields": ([vp, vp, ip, ip], ip), "amps_run": ([vp, ip], ip), "amps_set_graphs": ([vp, ip], ip),
            "amps_get_tile_tiers": ([vp, vp], ip), "amps_get_decision_log": ([vp, vp, ip, ctypes.POINTER(ip)], ip),
            "amps_get_tile_types": ([vp, vp], ip),
            "amps_get_tile_metric": ([vp, vp], ip), "amps_get_stats": ([vp, ctypes.POINTER(Stats)], ip),
            "amps_set_tier_schedule": ([vp, vp, ip], ip), "amps_set_tile_tiers": ([vp, vp], ip),
            "amps_measure_tiles": ([vp, ip, vp], ip),
            "amps_reduce": ([vp, ip, ip, ctypes.POINTER(dp)], ip),
            "amps_compare": ([vp, ip, vp, ip, ctypes.POINTER(dp), ctypes.POINTER(dp)], ip),
            "amps_set_profiling": ([vp, ip], ip),
            "amps_get_kernel_times": ([vp, ctypes.POINTER(dp), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64)], ip),
            "amps_step_forward": ([P, ip, vp, vp, ctypes.c_int64, vp], ip),
            "amps_step_adjoint": ([P, ip, vp, vp, vp, vp, ctypes.c_int64, vp], ip),
            "amps_adjoint_memory_bytes": ([P, ip, ip, ip], ctypes.c_size_t),
            "amps_adjoint_create": ([P, ip, ip, ip, ctypes.POINTER(vp)], ip),
            "amps_adjoint_destroy": ([vp], ip), "amps_adjoint_set_stream": ([vp, vp], ip),
            "amps_adjoint_set_graphs": ([vp, ip], ip), "amps_adjoint_segment": ([vp], ip),
            "amps_adjoint_last_error": ([vp], ctypes.c_char_p),
            "amps_adjoint_forward": ([vp, ctypes.POINTER(dp), vp, vp, ctypes.c_int64], ip),
            "amps_adjoint_backward": ([vp, vp, vp, vp], ip),
            "amps_compare_all": ([vp, ip, vp, ip, ctypes.POINTER(dp)], ip),
            "amps_interface": ([vp, ip, dp, ctypes.POINTER(dp)], ip),
            "amps_grains": ([vp, dp, dp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(dp)], ip),
            "amps_boundary_lengths": ([vp, dp, ctypes.POINTER(dp)], ip),
            "amps_ensemble_create": ([ctypes.POINTER(vp), ip, ctypes.POINTER(vp)], ip),
            "amps_ensemble_destroy": ([vp], ip), "amps_ensemble_set_stream": ([vp, vp], ip),
            "amps_ensemble_set_graphs": ([vp, ip], ip), "amps_ensemble_run": ([vp, ip], ip),
            "amps_ensemble_synchronize": ([vp], ip), "amps_ensemble_last_error": ([vp], ctypes.c_char_p),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _check(rc, handle, what):
    if rc != 0:
        msg = lib().amps_last_error(handle).decode() if handle is not None or what == "amps_create" else what
        raise AmpsError(rc, f"{what}: {msg or lib().amps_status_string(rc).decode()}")


def init_host(params, kind=INIT_REFERENCE):
    """Initial state of `params` computed on the host: array [nfields, ny, nx] (float64)."""
    nf = params.num_fields
    out = np.zeros((nf, params.ny, params.nx))
    ptrs = (ctypes.c_void_p * nf)(*[out[k].ctypes.data for k in range(nf)])
    _check(lib().amps_init_host(ctypes.byref(params), kind, ptrs), None, "amps_init_host")
    return out


class Simulation:
    """One libamps handle: a grid, its fields and its time loop."""

    def __init__(self, params, init=None, graphs=True):
        self.params = params
        h = ctypes.c_void_p()
        rc = lib().amps_create(ctypes.byref(params), ctypes.byref(h))
        if rc != 0:
            raise AmpsError(rc, "amps_create: " + lib().amps_last_error(None).decode())
        self.h = h
        self.nf = params.num_fields
        self.shape = (params.ny, params.nx)
        self.ntiles = (-(-params.ny // params.tile), -(-params.nx // params.tile))  # ragged sides: partial edge tiles
        if not graphs:
            lib().amps_set_graphs(self.h, 0)
        if init is not None:
            self.init(init)

    def close(self):
        if self.h:
            lib().amps_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        _check(rc, self.h, what)

    def init(self, kind=INIT_REFERENCE):
        self._ck(lib().amps_init(self.h, kind), "amps_init")
        return self

    def set_stream(self, stream_ptr):
        self._ck(lib().amps_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "amps_set_stream")

    def run(self, nsteps):
        self._ck(lib().amps_run(self.h, int(nsteps)), "amps_run")
        return self

    def synchronize(self):
        self._ck(lib().amps_synchronize(self.h), "amps_synchronize")

    def field(self, k, dtype=np.float64):
        out = np.empty(self.shape, dtype=dtype)
        self._ck(lib().amps_get_field(self.h, k, out.ctypes.data, F64 if dtype == np.float64 else F32, 0),
                 "amps_get_field")
        return out

    def fields(self, dtype=np.float64):
        out = np.empty((self.nf,) + self.shape, dtype=dtype)
        self._ck(lib().amps_get_fields(self.h, out.ctypes.data, F64 if dtype == np.float64 else F32, 0),
                 "amps_get_fields")
        return out

    def set_field(self, k, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.shape
        self._ck(lib().amps_set_field(self.h, k, a.ctypes.data, F64, 0), "amps_set_field")

    def set_fields(self, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == (self.nf,) + self.shape
        self._ck(lib().amps_set_fields(self.h, a.ctypes.data, F64, 0), "amps_set_fields")

    # device pointers (e.g. torch tensors' data_ptr()) -- no host round trip
    def set_fields_device(self, ptr, dtype=F64):
        self._ck(lib().amps_set_fields(self.h, ctypes.c_void_p(ptr), dtype, 1), "amps_set_fields")

    def get_fields_device(self, ptr, dtype=F64):
        self._ck(lib().amps_get_fields(self.h, ctypes.c_void_p(ptr), dtype, 1), "amps_get_fields")

    def tiers(self):
        out = np.empty(self.ntiles, dtype=np.uint8)
        self._ck(lib().amps_get_tile_tiers(self.h, out.ctypes.data), "amps_get_tile_tiers")
        return out

    def tile_types(self):
        """The tier map in the reference's type_curr encoding (1 half2, 2 high, 3 FP32)."""
        out = np.empty(self.ntiles, dtype=np.uint8)
        self._ck(lib().amps_get_tile_types(self.h, out.ctypes.data), "amps_get_tile_types")
        return out

    def metric(self):
        out = np.empty(self.ntiles, dtype=np.float64)
        self._ck(lib().amps_get_tile_metric(self.h, out.ctypes.data), "amps_get_tile_metric")
        return out

    def decision_log(self, max_entries=None):
        max_entries = max_entries or max(self.params.max_log, 0)
        out = np.empty((max(max_entries, 1),) + self.ntiles, dtype=np.uint8)
        n = ctypes.c_int(0)
        self._ck(lib().amps_get_decision_log(self.h, out.ctypes.data, max_entries, ctypes.byref(n)),
                 "amps_get_decision_log")
        return out[: n.value]

    def set_tier_schedule(self, maps):
        """Adaptive runs: take the tier maps of successive classifications from
        `maps` (e.g. another run's decision_log()) instead of the monitor, with
        no monitor epilogue; None or an empty array restores the monitor."""
        if maps is None or len(maps) == 0:
            self._ck(lib().amps_set_tier_schedule(self.h, None, 0), "amps_set_tier_schedule")
            return
        m = np.ascontiguousarray(maps, dtype=np.uint8).reshape((-1,) + self.ntiles)
        self._ck(lib().amps_set_tier_schedule(self.h, m.ctypes.data, m.shape[0]), "amps_set_tier_schedule")

    def set_tiers(self, tiers):
        """Static modes (purehigh, purelow, GRAM1, GRAM2): store the state at
        the tile tiers `tiers` ([nty][ntx], AMPS_TIER_*) from now on."""
        t = np.ascontiguousarray(tiers, dtype=np.uint8).reshape(self.ntiles)
        self._ck(lib().amps_set_tile_tiers(self.h, t.ctypes.data), "amps_set_tile_tiers")

    def measure_tiles(self, kind=MONITOR_SPA):
        """The monitor metric of the current state per tile ([nty][ntx]); for
        MONITOR_TEM against the state stored by store_temporal_reference()."""
        out = np.empty(self.ntiles, dtype=np.float64)
        self._ck(lib().amps_measure_tiles(self.h, int(kind), out.ctypes.data), "amps_measure_tiles")
        return out

    def store_temporal_reference(self):
        """Keep the current monitor samples as the reference of measure_tiles(MONITOR_TEM)."""
        self._ck(lib().amps_measure_tiles(self.h, MONITOR_TEM, None), "amps_measure_tiles")

    def stats(self):
        s = Stats()
        self._ck(lib().amps_get_stats(self.h, ctypes.byref(s)), "amps_get_stats")
        return s.as_dict()

    def kernel_launches(self):
        """Kernels amps_run has launched on this handle (steps, classifications)."""
        s = Stats()
        self._ck(lib().amps_get_stats(self.h, ctypes.byref(s)), "amps_get_stats")
        return s.kernel_launches

    def reduce(self, k, kind=REDUCE_SUM):
        v = ctypes.c_double()
        self._ck(lib().amps_reduce(self.h, k, kind, ctypes.byref(v)), "amps_reduce")
        return v.value

    def compare(self, k, other):
        a = np.ascontiguousarray(other, dtype=np.float64)
        mx, rms = ctypes.c_double(), ctypes.c_double()
        self._ck(lib().amps_compare(self.h, k, a.ctypes.data, 0, ctypes.byref(mx), ctypes.byref(rms)),
                 "amps_compare")
        return mx.value, rms.value

    def compare_all(self, k, other):
        """{max_abs, rms, mean_abs} of field k against `other` (the mean absolute
        difference is the reference's error metric)."""
        a = np.ascontiguousarray(other, dtype=np.float64)
        out = (ctypes.c_double * 3)()
        self._ck(lib().amps_compare_all(self.h, k, a.ctypes.data, 0, out), "amps_compare_all")
        return {"max_abs": out[0], "rms": out[1], "mean_abs": out[2]}

    def interface(self, k, level=0.5):
        """Level set {field k >= level}: cells, area, perimeter, bounding box."""
        out = (ctypes.c_double * 7)()
        self._ck(lib().amps_interface(self.h, k, float(level), out), "amps_interface")
        return {"cells": int(out[0]), "area": out[1], "perimeter": out[2],
                "xmin": int(out[3]), "xmax": int(out[4]), "ymin": int(out[5]), "ymax": int(out[6])}

    def grains(self, threshold=0.5, level=0.5):
        """Connected grains of the dominant order parameter: count, labelled cells, mean area."""
        out = (ctypes.c_int64 * 2)()
        area = ctypes.c_double()
        self._ck(lib().amps_grains(self.h, float(threshold), float(level), out, ctypes.byref(area)), "amps_grains")
        return {"grains": out[0], "cells": out[1], "mean_area": area.value}

    def boundary_lengths(self, level=0.5):
        """Boundary length between every pair of order parameters (q x q)."""
        q = self.nf - (1 if self.params.model == SINTERING else 0)
        out = np.zeros((q, q))
        self._ck(lib().amps_boundary_lengths(self.h, float(level), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                 "amps_boundary_lengths")
        return out

    def set_profiling(self, enable=True):
        self._ck(lib().amps_set_profiling(self.h, int(enable)), "amps_set_profiling")

    def kernel_times(self):
        """[half, fp32, fp64 per-tier kernels, fused all-tier kernel]: summed device ms and launches;
        tile-steps per tier (index 3: total) since profiling began."""
        ms = (ctypes.c_double * 4)()
        la = (ctypes.c_int64 * 4)()
        ts = (ctypes.c_int64 * 4)()
        self._ck(lib().amps_get_kernel_times(self.h, ms, la, ts), "amps_get_kernel_times")
        return list(ms), list(la), list(ts)


class Ensemble:
    """Grain-growth `Simulation`s advanced in lockstep, one launch per group
    of members a step (amps_ensemble_*).  The members stay usable for reads
    (fields, tiers, stats) and must outlive the ensemble."""

    def __init__(self, members, graphs=True):
        self.members = list(members)
        arr = (ctypes.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h = ctypes.c_void_p()
        rc = lib().amps_ensemble_create(arr, len(self.members), ctypes.byref(h))
        if rc != 0:
            raise AmpsError(rc, "amps_ensemble_create: " + lib().amps_ensemble_last_error(None).decode())
        self.h = h
        if not graphs:
            lib().amps_ensemble_set_graphs(self.h, 0)

    def _ck(self, rc, what):
        if rc != 0:
            raise AmpsError(rc, f"{what}: {lib().amps_ensemble_last_error(self.h).decode()}")

    def set_stream(self, stream_ptr):
        self._ck(lib().amps_ensemble_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "amps_ensemble_set_stream")

    def run(self, nsteps):
        self._ck(lib().amps_ensemble_run(self.h, int(nsteps)), "amps_ensemble_run")
        return self

    def synchronize(self):
        self._ck(lib().amps_ensemble_synchronize(self.h), "amps_ensemble_synchronize")

    def close(self):
        if getattr(self, "h", None):
            lib().amps_ensemble_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
