// snowflake_pure.cu -- the reference's plain Kobayashi kernels
// (snowflake/function.h:5-60 kernel1_pure and kernel2_pure, snowflake/tools.h:24-33
// dataprepare_high) built in place from the read-only reference tree into
// device code for the GB300, with the header settings of
// snowflake/end2end_pure.py (typedef double highprecision, PURE, End2end)
// and the parameter set REF_PARA_H.  The reference's own code, unchanged; no
// host code is built (baseline/ref_cuda.cpp drives it).
#include "prelude.cuh"
#define float double
#include REF_PARA_H
#undef float
#undef AMSTENCIL
#undef HALF2
#undef monitor_conversion_independent
#ifndef PURE
#define PURE
#endif
#ifndef End2end
#define End2end
#endif
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

// the build's compile-time sizes, read by the host driver: dimX, dimY, unitx, unity
__device__ int ref_dims[4] = {dimX, dimY, unitx, unity};
