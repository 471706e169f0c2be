/*
 * graingrowth_mix_ref.cpp -- the reference's adaptive mixed-precision grain
 * growth (AMSTENCIL, half2 low tier, double high tier) compiled in place from
 * the read-only reference tree for the CPU: kernel1_mix
 * (graingrowth/function.h:33-277), dataprepare_high/_half2,
 * get_max_diff1/2, get_type, data_sychro_duringcomputation and
 * data_sychro_aftercomputation (graingrowth/tools.h), driven by the time loop
 * of graingrowth/end2end_mix.cu:35-105.  TEST INFRASTRUCTURE ONLY: it pins
 * the library's reference-faithful mixed mode (tier decisions per period and
 * the mixed-vs-FP64 error) on the CPU.
 *
 * Header settings, as graingrowth/end2end_mix.py writes them into
 * paras/total.h: typedef double highprecision, #define AMSTENCIL, End2end,
 * Monitor<REF_MONITOR>, monitor_conversion_dependent.  The threshold line is
 * the one the script rewrites per run; here it is a runtime value
 * (ref_ggmix_run's argument) so that one build serves every threshold.
 *
 * Half arithmetic: the host versions of cuda_fp16.h's half2 operators round
 * every operation separately (the reference's expressions as written, each
 * +, -, *, / rounded to binary16).
 */
#include "cuda_cpu_shim.h"
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
static double threshold = 0.99;
#define PARA5_H
#include REF_FUNCTION_H
#include REF_TOOLS_H

extern "C" {
int ref_ggmix_dims(void) { return dimX; }
int ref_ggmix_tiles(void) { return unitdimX * unitdimY; }
int ref_ggmix_monitor(void) { return REF_MONITOR; }

/* graingrowth/end2end_mix.cu:35-105 (AMSTENCIL branch) for `steps` steps at
 * `thr`.  types: [steps/10 + 1][tiles] uint8, the type_curr map (1 = half2,
 * 2 = high) after each classification; metric: the same count of
 * [tiles] max_diff maps.  eta1, eta2: the high arrays at the end, low tiles
 * gathered from their half2 arrays (data_sychro_aftercomputation). */
void ref_ggmix_run(int steps, double thr, double *eta1_out_final, double *eta2_out_final, unsigned char *types,
                   double *metric)
{
    threshold = thr;
    const size_t n = (size_t)dimX * dimY, nh = (size_t)dimXd2 * dimY, nt = (size_t)unitdimX * unitdimY;
    double *hi = (double *)calloc(9 * n, sizeof(double));
    double *eta1 = hi, *eta2 = hi + n, *eta1_out = hi + 2 * n, *eta2_out = hi + 3 * n, *eta1_lap = hi + 4 * n,
           *eta2_lap = hi + 5 * n, *dfdeta1 = hi + 6 * n, *dfdeta2 = hi + 7 * n, *eta2_last = hi + 8 * n;
    half2 *lo = (half2 *)calloc(8 * nh, sizeof(half2));
    half2 *heta1 = lo, *heta2 = lo + nh, *heta1_out = lo + 2 * nh, *heta2_out = lo + 3 * nh, *heta1_lap = lo + 4 * nh,
          *heta2_lap = lo + 5 * nh, *hdfdeta1 = lo + 6 * nh, *hdfdeta2 = lo + 7 * nh;
    int *type_curr = (int *)calloc(nt, sizeof(int)), *type_old = (int *)calloc(nt, sizeof(int));
    double *max_diff = (double *)calloc(nt, sizeof(double));
    shim_launch(dim3(1, 1, unitdimX * unitdimY), dim3(unitx, unity), dataprepare_high, eta1, eta2);
    shim_launch(dim3(1, 1, unitdimX * unitdimY), dim3(uxd2, unity), dataprepare_half2, heta1, heta2);
#if REF_MONITOR == 2
    for (size_t i = 0; i < n; i++) eta2_last[i] = eta2[i] == 0 ? 1.0 : 0.0;
#endif
    const dim3 blocks_detect(unitdimX > 32 ? 32 : unitdimX, unitdimY > 32 ? 32 : unitdimY);
    const dim3 grids_detect(unitdimX > 32 ? unitdimX / 32 : 1, unitdimY > 32 ? unitdimY / 32 : 1);
    const dim3 sync_blocks(uxd2, unity), sync_grids(1, 1, unitdimX * unitdimY);
    const half2 hmobil = __float2half2_rn(mobil), hgrcoef = __float2half2_rn(grcoef),
                hdxdy = __float2half2_rn(dxdy), height = __float2half2_rn(8.0), hdtime = __float2half2_rn(dtime),
                hone = __float2half2_rn(1.0), htwo = __float2half2_rn(2.0);
    const dim3 blocks_mix(uxd2, unity), grids_mix(2, 1, unitdimX * unitdimY);
    int period = 0;
    for (int i = 0; i < steps; i++) {
        if (i % 10 == 0) {
#if REF_MONITOR == 1
            shim_launch(grids_detect, blocks_detect, get_max_diff1, eta2, max_diff);
#else
            shim_launch(grids_detect, blocks_detect, get_max_diff2, eta2_last, eta2, max_diff);
#endif
            shim_launch(grids_detect, blocks_detect, get_type, max_diff, type_old, type_curr);
            shim_launch(sync_grids, sync_blocks, data_sychro_duringcomputation, eta1, eta2, heta1, heta2, type_old,
                        type_curr);
            for (size_t t = 0; t < nt; ++t) {
                if (types) types[(size_t)period * nt + t] = (unsigned char)type_curr[t];
                if (metric) metric[(size_t)period * nt + t] = max_diff[t];
            }
            ++period;
        }
        shim_launch(grids_mix, blocks_mix, kernel1_mix, eta1, eta2_last, eta2, eta1_lap, dfdeta1, eta1_out, heta1,
                    heta2, heta1_lap, hdfdeta1, heta1_out, height, hdxdy, hone, htwo, hdtime, hmobil, hgrcoef,
                    type_curr, i, 1);
        shim_launch(grids_mix, blocks_mix, kernel1_mix, eta2, eta2_last, eta1, eta2_lap, dfdeta2, eta2_out, heta2,
                    heta1, heta2_lap, hdfdeta2, heta2_out, height, hdxdy, hone, htwo, hdtime, hmobil, hgrcoef,
                    type_curr, i, 2);
        std::swap(eta1, eta1_out);
        std::swap(eta2, eta2_out);
        std::swap(heta1, heta1_out);
        std::swap(heta2, heta2_out);
    }
    /* graingrowth/end2end_mix.cu:117-121 gathers eta2 only; eta1 likewise */
    shim_launch(grids_mix, blocks_mix, data_sychro_aftercomputation, eta1, heta1, type_curr);
    shim_launch(grids_mix, blocks_mix, data_sychro_aftercomputation, eta2, heta2, type_curr);
    for (size_t k = 0; k < n; ++k) {
        eta1_out_final[k] = eta1[k];
        eta2_out_final[k] = eta2[k];
    }
    free(hi);
    free(lo);
    free(type_curr);
    free(type_old);
    free(max_diff);
}
}
