// sintering_mix.cu -- the reference's adaptive mixed-precision sintering
// (AMSTENCIL: half2 low tier, double high tier): con1_mix, con2_mix, phi1_mix,
// phi2_mix (sintering/function.h:161-774), dataprepare, get_max_diff1/2,
// data_sychro_duringcomputation and data_sychro_aftercomputation
// (sintering/tools.h), built in place into device code for the GB300 with
// AMSTENCIL defined as sintering/end2end_run1.py writes it; the shipped
// Monitor2 line stays (con1_mix then also refreshes the snapshot, which the
// spatial monitor never reads), so one build serves both monitors.
#include "prelude.cuh"
#define AMSTENCIL
// the threshold is a constant of the parameter file, which function.h
// includes itself: renamed here, and the classification below takes it at
// run time
#define threshold threshold_as_written
#include REF_TOOLS_H
#undef threshold

// get_type (sintering/tools.h:38-56) at a run-time threshold: the same rule
// -- type_old = type_con, then the tile's 5-point maximum of max_diff (not
// periodic) below thr -> 1 (half2), at or above -> 2 -- and the same launch
// shape, restated because the parameter file fixes `threshold` at compile time.
extern "C" __global__ void ref_get_type_rt(const double *max_diff_con, int *type_old, int *type_con, double thr)
{
    const int ux = threadIdx.x + blockIdx.x * blockDim.x, uy = threadIdx.y + blockIdx.y * blockDim.y;
    const int t = uy * unitdimX + ux;
    type_old[t] = type_con[t];
    double m = max_diff_con[t];
    if (uy < unitdimY - 1) m = fmax(m, max_diff_con[t + unitdimX]);
    if (uy > 0) m = fmax(m, max_diff_con[t - unitdimX]);
    if (ux < unitdimX - 1) m = fmax(m, max_diff_con[t + 1]);
    if (ux > 0) m = fmax(m, max_diff_con[t - 1]);
    type_con[t] = m < thr ? 1 : 2;
}

// the build's compile-time sizes, read by the host driver: dimX, dimY, unitx, unity
__device__ int ref_dims[4] = {dimX, dimY, unitx, unity};
// and its double constants the host converts to half2 (sintering/main.cu:78-99):
// coefm, coefk, coefl, dvol, dvap, dsur, dgrb, dxdy, dtime
__device__ double ref_consts[9] = {coefm, coefk, coefl, dvol, dvap, dsur, dgrb, dxdy, dtime};
