"""amps_reduce_noalloc: the FP64 field reduction for callers that cannot
allocate device memory (its partials live in a fixed device array inside the
library).  Checked through the C ABI against amps_reduce, the handle-based
reduction, on two calls in a row with different sizes, so that the second
call cannot pass on the first call's leftovers.  Kept in its own file that
pytest collects last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_CELLS = 4096 * 4096  # AMPS_REDUCE_NOALLOC_MAX_CELLS in include/amps.h


def _entry():
    import w3914777_gb300 as w
    f = w.lib().amps_reduce_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return w, f


def test_noalloc_reduction_matches_handle_reduction_on_two_calls():
    import torch
    w, noalloc = _entry()
    rng = np.random.default_rng(17)
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    # two calls in a row: a larger array, then a smaller one (fewer partials)
    for nx, ny in ((1024, 768), (192, 160)):
        a = rng.standard_normal((ny, nx)) + 0.25
        p = w.Params.preset("sintering", 1, mode="purehigh", nx=nx, ny=ny)
        dev = torch.from_numpy(a).cuda()
        with w.Simulation(p) as s:
            s.set_field(0, a)
            for kind in (w.amps.REDUCE_SUM, w.amps.REDUCE_MIN, w.amps.REDUCE_MAX, w.amps.REDUCE_SUMSQ):
                rc = noalloc(dev.data_ptr(), dev.numel(), kind, out.data_ptr(), None)
                torch.cuda.synchronize()
                assert rc == 0
                got = float(out.item())
                want = s.reduce(0, kind)
                if kind in (w.amps.REDUCE_MIN, w.amps.REDUCE_MAX):
                    assert got == want
                else:
                    assert abs(got - want) <= 1e-12 * max(abs(want), 1.0), (kind, got, want)


def test_noalloc_reduction_rejects_sizes_beyond_its_array():
    import torch
    w, noalloc = _entry()
    dev = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    # rejected before any device work is queued
    assert noalloc(dev.data_ptr(), MAX_CELLS + 1, 0, out.data_ptr(), None) == 6  # AMPS_ERR_UNSUPPORTED
    assert noalloc(dev.data_ptr(), 0, 0, out.data_ptr(), None) == 1              # AMPS_ERR_INVALID
