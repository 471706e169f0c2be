"""Generate tests/golden/graingrowth_mix_ref.npz and sintering_mix_ref.npz:
the reference's own adaptive mixed-precision runs (AMSTENCIL: half2 low tier,
double high tier), executed on the CPU from oracle/_ref/libref_ggmix_m*.so
and libref_sintmix_m*.so (built by `make -C oracle ref` from the reference
tree), for a few of the sweep scripts' thresholds of each monitor
(graingrowth/end2end_mix.py:19-23, sintering/end2end_run1.py:37-41), 500
steps as the scripts set `timesteps`:
  grain growth: graingrowth/end2end_mix.cu with graingrowth/function.h:33-277
    and graingrowth/tools.h, parameter set para1 (512x512, 16x16 tiles);
  sintering: sintering/main.cu:45-206 with sintering/function.h:161-774 and
    sintering/tools.h, the shipped parameter set para5 (512x512), built with
    SHIM_CUBE_RN: pow(x, 3) is the correctly rounded cube, on both sides of
    every comparison.  This run is chaotic at the ulp level (a one-ulp change
    grows about 1.5x per step; the two particles dissolve into clamped cells),
    and the last bit of pow(x, 3) differs between the C library, CUDA and a
    correctly rounded cube, so a bit-level pin needs one cube everywhere.

Per run (key prefix m<monitor>_<threshold>):
  types   [periods][1024] uint8: type_curr after each classification
          (1 = half2, 2 = high), one map per 10 steps
  eta1, eta2  final fields (high arrays after data_sychro_aftercomputation),
          for the runs in FIELD_RUNS (sintering: c, eta1, eta2)
  err     the run against the reference's plain FP64 run of the same steps:
          mean |d f| of every field, then max |d f| of every field; the mean
          over the grid is the reference's error metric
          (graingrowth/end2enderror.py:34, sintering/end2enderror.py:36)

Run from the repository root (a few minutes each, runs in parallel):
    python tests/golden/make_golden_mix.py [graingrowth|sintering|all]
"""
import ctypes
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_bind as ob  # noqa: E402

STEPS = 500
RUNS = [(2, 1e-6), (2, 1e-4), (2, 1e-2), (1, 1e-3), (1, 0.1), (1, 0.5)]
FIELD_RUNS = [(2, 1e-4), (2, 1e-2), (1, 0.5)]  # final fields kept for these (the fixture stays small)


def key(monitor, thr):
    return f"m{monitor}_{thr:g}"


def run_mix(monitor, thr, steps=STEPS):
    """One reference AMSTENCIL run: (types, eta1, eta2)."""
    L = ctypes.CDLL(os.path.join(ob.REF_DIR, f"libref_ggmix_m{monitor}.so"))
    n, nt = L.ref_ggmix_dims(), L.ref_ggmix_tiles()
    periods = (steps + 9) // 10
    e1, e2 = np.zeros((n, n)), np.zeros((n, n))
    types = np.zeros((periods, nt), np.uint8)
    dp = ctypes.POINTER(ctypes.c_double)
    L.ref_ggmix_run.argtypes = [ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_void_p, dp]
    L.ref_ggmix_run(steps, thr, ob.ptr(e1), ob.ptr(e2), types.ctypes.data, None)
    return types, e1, e2


def _job(args):
    return args, run_mix(*args)


def run_pure(steps=STEPS):
    R = ob.ref_lib("graingrowth")
    n = R.ref_gg_dims()
    e1, e2 = np.zeros((n, n)), np.zeros((n, n))
    R.ref_gg_init(ob.ptr(e1), ob.ptr(e2))
    R.ref_gg_steps(ob.ptr(e1), ob.ptr(e2), steps)
    return e1, e2


def run_sint_mix(monitor, thr, steps=STEPS):
    """One reference AMSTENCIL sintering run: (types, c, eta1, eta2)."""
    L = ctypes.CDLL(os.path.join(ob.REF_DIR, f"libref_sintmix_m{monitor}.so"))
    n, nt = L.ref_sintmix_dims(), L.ref_sintmix_tiles()
    periods = (steps + 9) // 10
    c, e1, e2 = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    types = np.zeros((periods, nt), np.uint8)
    dp = ctypes.POINTER(ctypes.c_double)
    L.ref_sintmix_run.argtypes = [ctypes.c_int, ctypes.c_double, dp, dp, dp, ctypes.c_void_p]
    L.ref_sintmix_run(steps, thr, ob.ptr(c), ob.ptr(e1), ob.ptr(e2), types.ctypes.data)
    return types, c, e1, e2


def _sint_job(args):
    return args, run_sint_mix(*args)


def run_sint_pure(steps=STEPS):
    """The reference's plain sintering, built like the mixed runs with pow(x, 3)
    as the correctly rounded cube (libref_sintering_rn.so)."""
    R = ob.ref_lib("sintering_rn")
    n = R.ref_sint_dims()
    pr = ob.ref_params("sintering", 15)
    c, e1, e2 = ob.sint_init_two(n, n, pr[12], pr[13], pr[10], pr[14], pr[11])
    R.ref_sint_steps(ob.ptr(c), ob.ptr(e1), ob.ptr(e2), steps)
    return c, e1, e2


def make_sintering():
    for m in (1, 2):
        if not os.path.exists(os.path.join(ob.REF_DIR, f"libref_sintmix_m{m}.so")) or \
                not os.path.exists(os.path.join(ob.REF_DIR, "libref_sintering_rn.so")):
            raise SystemExit("oracle/_ref/libref_sintmix_m*.so missing: run `make -C oracle ref`")
    with mp.get_context("spawn").Pool(min(len(RUNS), os.cpu_count() or 1)) as pool:
        results = dict(pool.map(_sint_job, RUNS))
    pure = run_sint_pure()
    out = {"steps": STEPS, "runs": np.array([[m, t] for m, t in RUNS])}
    for (m, t), (types, *fields) in results.items():
        k = key(m, t)
        d = [np.abs(f - q) for f, q in zip(fields, pure)]
        out[k + "_types"] = types
        if (m, t) in FIELD_RUNS:
            out[k + "_c"], out[k + "_eta1"], out[k + "_eta2"] = fields
        out[k + "_err"] = np.array([x.mean() for x in d] + [x.max() for x in d])
        print(k, "half tiles per period (first, last):", int((types[0] == 1).sum()), int((types[-1] == 1).sum()),
              "err", out[k + "_err"])
    path = os.path.join(HERE, "sintering_mix_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


def main():
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    if which in ("sintering", "all"):
        make_sintering()
    if which in ("graingrowth", "all"):
        make_graingrowth()


def make_graingrowth():
    for m in (1, 2):
        if not os.path.exists(os.path.join(ob.REF_DIR, f"libref_ggmix_m{m}.so")):
            raise SystemExit("oracle/_ref/libref_ggmix_m*.so missing: run `make -C oracle ref`")
    with mp.get_context("spawn").Pool(min(len(RUNS), os.cpu_count() or 1)) as pool:
        results = dict(pool.map(_job, RUNS))
    p1, p2 = run_pure()
    out = {"steps": STEPS, "runs": np.array([[m, t] for m, t in RUNS])}
    for (m, t), (types, e1, e2) in results.items():
        k = key(m, t)
        d1, d2 = np.abs(e1 - p1), np.abs(e2 - p2)
        out[k + "_types"] = types
        if (m, t) in FIELD_RUNS:
            out[k + "_eta1"] = e1
            out[k + "_eta2"] = e2
        out[k + "_err"] = np.array([d1.mean(), d2.mean(), d1.max(), d2.max()])
        print(k, "half tiles per period (first, last):", int((types[0] == 1).sum()), int((types[-1] == 1).sum()),
              "err", out[k + "_err"])
    path = os.path.join(HERE, "graingrowth_mix_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
