/*
 * snowflake_ref.cpp -- the reference's plain Kobayashi kernels
 * (snowflake/function.h:5-60) and initial state (snowflake/tools.h:24-33),
 * compiled in place from the read-only reference tree for the CPU with the
 * header settings the reference's own sweep scripts write
 * (snowflake/end2end_pure.py): typedef double highprecision, #define PURE,
 * parameter set REF_PARA.  TEST INFRASTRUCTURE ONLY.
 */
#include "cuda_cpu_shim.h"
/* highprecision: the sweep scripts set "typedef double highprecision".
 * REF_PARA_H / REF_FUNCTION_H / REF_TOOLS_H are quoted paths into the
 * reference tree, given on the compile line by oracle/Makefile. */
#define float double
#include REF_PARA_H
#undef float
#undef AMSTENCIL
#undef HALF2
#undef monitor_conversion_independent
#define PURE
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

extern "C" {
int ref_snowflake_dims(void) { return dimX; }
void ref_snowflake_init(double *phi, double *T)
{
    for (int i = 0; i < dimX * dimY; ++i) { phi[i] = 0; T[i] = 0; }
    shim_launch(dim3(1, 1, unitdimX * unitdimY), dim3(unitx, unity), dataprepare_high, phi);
}
void ref_snowflake_steps(double *phi, double *T, int steps)
{
    const size_t n = (size_t)dimX * dimY;
    double *s = (double *)calloc(6 * n, sizeof(double));
    dim3 blocks(unitx, unity), grids(1, 1, unitdimX * unitdimY);
    for (int i = 0; i < steps; ++i) {
        shim_launch(grids, blocks, kernel1_pure, phi, s, T, s + n, s + 2 * n, s + 3 * n, s + 4 * n, s + 5 * n);
        shim_launch(grids, blocks, kernel2_pure, phi, s, s + 4 * n, s + 5 * n, s + 2 * n, s + 3 * n, T, s + n);
    }
    free(s);
}
void ref_snowflake_params(double *out)
{
    out[0] = dx; out[1] = dy; out[2] = tau; out[3] = epsilonb; out[4] = kappa; out[5] = delta;
    out[6] = aniso; out[7] = alpha; out[8] = gama; out[9] = teq; out[10] = theta0; out[11] = dtime;
    out[12] = pi; out[13] = seed;
}
}
