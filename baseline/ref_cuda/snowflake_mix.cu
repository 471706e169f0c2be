// snowflake_mix.cu -- the reference's adaptive mixed-precision Kobayashi
// dendrite (AMSTENCIL: half2 low tier, double high tier): kernel1_mix and
// mix_kernel2 (snowflake/function.h:63-604; the half tiles' h2cos/h2sin
// included), dataprepare_high/_half2, get_max_diff1/2, get_type,
// data_sychro_duringcomputation and data_sychro_aftercomputation
// (snowflake/tools.h), built in place into device code for the GB300 with
// the header settings snowflake/end2end_mix.py writes into paras/total.h:
// typedef double highprecision, AMSTENCIL, End2end, Monitor<REF_MONITOR>,
// monitor_conversion_dependent.  The threshold line the script rewrites per
// run becomes a device variable (`threshold`) set before each run.
#include "prelude.cuh"
#define AMSTENCIL
#define threshold threshold_as_written
#define float double
#include REF_PARA_H
#undef float
#undef threshold
#undef PURE
#undef Monitor1
#undef Monitor2
#if REF_MONITOR == 1
#define Monitor1
#else
#define Monitor2
#endif
#ifndef End2end
#define End2end
#endif
#ifndef monitor_conversion_dependent
#define monitor_conversion_dependent
#endif
__device__ double threshold = 0.99;
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

// the build's compile-time sizes, read by the host driver: dimX, dimY, unitx, unity
__device__ int ref_dims[4] = {dimX, dimY, unitx, unity};
// and its double constants the host converts to half2 (end2end_mix.cu:60-76):
// dxdy, dy*2, dx*2, theta0, aniso, delta, epsilonb, alpha, pi, gama, kappa, teq, dtime, tau
__device__ double ref_consts[14] = {dxdy, dy * 2, dx * 2, theta0, aniso, delta, epsilonb,
                                    alpha, pi, gama, kappa, teq, dtime, tau};
