"""GB300-native adaptive mixed-precision phase-field stencils (Kobayashi
dendrite, grain growth, sintering) behind a C ABI (include/amps.h)."""
from .amps import (  # noqa: F401
    BC_NOFLUX, BC_PERIODIC, END2END_MIX, F32, F64, GRAINGROWTH, GRAM1, GRAM2, HALF_FP32, HALF_HFMA2, HALF_REF, HALF_SR,
    INIT_REFERENCE, INIT_SEEDED,
    KOBAYASHI, MONITOR_RATE, MONITOR_SPA, MONITOR_TEM, PUREHIGH, PURELOW, REDUCE_MAX, REDUCE_MIN, REDUCE_SUM,
    REDUCE_SUMSQ, SINTERING, TIER_FP32, TIER_FP64, TIER_HALF, AmpsError, Ensemble, Params, Simulation, init_host, lib,
)
