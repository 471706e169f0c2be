/*
 * sintering_ref.cpp -- the reference's plain sintering kernels
 * (sintering/function.h:51-159: con1_pure, con2_pure, phi1_pure, phi2_pure)
 * compiled in place from the read-only reference tree for the CPU, in the
 * shipped header state (#define PURE; function.h includes paras/para5.h, whose
 * highprecision is already double).  The step sequence follows
 * sintering/main.cu:136-147.  Built twice: as shipped (libref_sintering.so)
 * and with SHIM_CUBE_RN (libref_sintering_rn.so, pow(x, 3) the correctly
 * rounded cube), the plain run the mixed golden is measured against.
 * TEST INFRASTRUCTURE ONLY.
 */
#include "cuda_cpu_shim.h"
#include REF_FUNCTION_H

extern "C" {
int ref_sint_dims(void) { return dimX; }
void ref_sint_steps(double *con, double *eta1, double *eta2, int steps)
{
    const size_t n = (size_t)dimX * dimY;
    double *s = (double *)calloc(9 * n, sizeof(double));
    double *e1 = eta1, *e2 = eta2, *o1 = s + 7 * n, *o2 = s + 8 * n;
    double *con_lap = s, *dummy = s + n, *dummy_lap = s + 2 * n, *dfdcon = s + 3 * n;
    double *e1lap = s + 4 * n, *e2lap = s + 5 * n, *dfde = s + 6 * n;
    dim3 blocks(unitx, unity), grids(1, 1, unitdimX * unitdimY);
    for (int i = 0; i < steps; ++i) {
        shim_launch(grids, blocks, con1_pure, con, con_lap, e1, e2, dfdcon, dummy, i);
        shim_launch(grids, blocks, con2_pure, dummy, dummy_lap, con, e1, e2, i);
        shim_launch(grids, blocks, phi1_pure, e1, o1, e2, e1lap, dfde, con, i);
        shim_launch(grids, blocks, phi2_pure, e2, o2, e1, e2lap, dfde, con, i);
        std::swap(e1, o1);
        std::swap(e2, o2);
    }
    if (e1 != eta1) { for (size_t i = 0; i < n; ++i) { eta1[i] = e1[i]; eta2[i] = e2[i]; } }
    free(s);
}
void ref_sint_params(double *out)
{
    out[0] = coefm; out[1] = coefk; out[2] = coefl; out[3] = dvol; out[4] = dvap; out[5] = dsur; out[6] = dgrb;
    out[7] = dx; out[8] = dy; out[9] = dtime; out[10] = R1; out[11] = R2; out[12] = Rx1; out[13] = Ry1; out[14] = Ry2;
}
}
