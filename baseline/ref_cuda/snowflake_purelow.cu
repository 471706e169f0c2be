// snowflake_purelow.cu -- the reference's all-half2 Kobayashi dendrite
// (snowflake/function.h:607-700 kernel1_purelow / kernel2_purelow,
// snowflake/tools.h:43-58 dataprepare_half2) built in place into device code
// for the GB300 in the shipped header state (HALF2, typedef float
// highprecision), as snowflake/simulation_result.py compiles
// snowflake/purelow.cu.  The reference's own code, unchanged.
#include "prelude.cuh"
#include REF_PARA_H
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

// the build's compile-time sizes, read by the host driver: dimX, dimY, unitx, unity
__device__ int ref_dims[4] = {dimX, dimY, unitx, unity};
// and its constants the host converts to half2 (snowflake/purelow.cu:23-39):
// dxdy, dy*2, dx*2, theta0, aniso, delta, epsilonb, alpha, pi, gama, kappa, teq, dtime, tau
__device__ double ref_consts[14] = {dxdy, dy * 2, dx * 2, theta0, aniso, delta, epsilonb,
                                    alpha, pi, gama, kappa, teq, dtime, tau};
