// graingrowth_purelow.cu -- the reference's all-half2 grain growth
// (graingrowth/function.h:280-308 kernel1_lowpure, graingrowth/tools.h:54-81
// dataprepare_half2) built in place into device code for the GB300 in the
// shipped header state (HALF2, typedef float highprecision), as
// graingrowth/purelow.cu compiles it.  The reference's own code, unchanged.
#include "prelude.cuh"
#include REF_PARA_H
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

// the build's compile-time sizes, read by the host driver: dimX, dimY, unitx, unity
__device__ int ref_dims[4] = {dimX, dimY, unitx, unity};
// and its constants the host converts to half2 (graingrowth/purelow.cu:26-34): mobil, grcoef, dxdy, dtime
__device__ double ref_consts[4] = {mobil, grcoef, dxdy, dtime};
