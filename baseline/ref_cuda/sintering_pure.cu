// sintering_pure.cu -- the reference's plain sintering kernels
// (sintering/function.h:51-159: con1_pure, con2_pure, phi1_pure, phi2_pure)
// built in place from the read-only reference tree into device code for the
// GB300, in the shipped header state (PURE; function.h includes
// paras/para5.h, whose highprecision is double).  The reference's own code,
// unchanged; no host code is built (baseline/ref_cuda.cpp drives it).
#include "prelude.cuh"
#include REF_FUNCTION_H

// the build's compile-time sizes, read by the host driver: dimX, dimY, unitx, unity
__device__ int ref_dims[4] = {dimX, dimY, unitx, unity};
