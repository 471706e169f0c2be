/*
 * graingrowth_ref.cpp -- the reference's plain grain-growth kernel
 * (graingrowth/function.h:5-30) and initial state (graingrowth/tools.h:24-38),
 * compiled in place from the read-only reference tree for the CPU with the
 * header settings of graingrowth/end2end_pure.py (typedef double
 * highprecision, #define PURE) and the parameter set in REF_PARA_H.
 * TEST INFRASTRUCTURE ONLY.
 */
#include "cuda_cpu_shim.h"
#define float double
#include REF_PARA_H
#undef float
#undef AMSTENCIL
#undef HALF2
#undef monitor_conversion_independent
#ifndef PURE
#define PURE
#endif
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

extern "C" {
int ref_gg_dims(void) { return dimX; }
void ref_gg_init(double *eta1, double *eta2)
{
    shim_launch(dim3(1, 1, unitdimX * unitdimY), dim3(unitx, unity), dataprepare_high, eta1, eta2);
}
/* graingrowth/purehigh.cu:23-36: both fields from the old pair, then swap. */
void ref_gg_steps(double *eta1, double *eta2, int steps)
{
    const size_t n = (size_t)dimX * dimY;
    double *s = (double *)calloc(6 * n, sizeof(double));
    double *e1 = eta1, *e2 = eta2, *o1 = s + 4 * n, *o2 = s + 5 * n;
    dim3 blocks(unitx, unity), grids(1, 1, unitdimX * unitdimY);
    for (int i = 0; i < steps; ++i) {
        shim_launch(grids, blocks, kernel1_pure, e1, e2, s, s + n, o1);
        shim_launch(grids, blocks, kernel1_pure, e2, e1, s + 2 * n, s + 3 * n, o2);
        std::swap(e1, o1);
        std::swap(e2, o2);
    }
    if (e1 != eta1) { for (size_t i = 0; i < n; ++i) { eta1[i] = e1[i]; eta2[i] = e2[i]; } }
    free(s);
}
void ref_gg_params(double *out)
{
    out[0] = dtime; out[1] = mobil; out[2] = dx; out[3] = dy; out[4] = grcoef; out[5] = R; out[6] = Rx; out[7] = Ry;
}
}
