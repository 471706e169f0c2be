/*
 * amps_compat.h -- the reference's kernel names as host launch wrappers.
 *
 * For a driver written against the reference's kernel interface
 * (snowflake/function.h, graingrowth/function.h, sintering/function.h and
 * the monitor tools in snowflake/tools.h): each function below takes the
 * same device arrays, in the same order and with the same roles, as the
 * reference kernel it is named after, and computes the same values (FP64,
 * the reference's expression order, no fused multiply-add), so a reference
 * time loop can swap `kernel<<<grid, block>>>(args)` for
 * `amps_<app>_kernel(&params, args, stream)` line by line.  What the
 * reference fixes at compile time -- grid size, tile size, physical
 * constants, the threshold -- comes from an amps_params (amps_preset gives
 * the reference's parameter files).  Arrays are row-major [ny][nx] doubles
 * in device memory, allocated by the caller; the neighbour map follows
 * p->bc (the reference's pure kernels are periodic).  Work is queued on
 * `stream` (cudaStream_t as void*, NULL = default stream); the calls return
 * an amps status.
 *
 * This is the compatibility path: one thread per cell (or half2 pair), intermediates in
 * full-size arrays, several launches per step, as in the reference.  The
 * fast path for the same time loop is amps_run (include/amps.h).
 */
#ifndef AMPS_COMPAT_H
#define AMPS_COMPAT_H
#include "amps.h"

#ifdef __cplusplus
extern "C" {
#endif

/* snowflake/function.h:5-35 -- phi_lap, tempr_lap, phidx, phidy, epsilon,
 * epsilon_deri from phi and tempr. */
AMPS_API int amps_snowflake_kernel1_pure(const amps_params *p, const double *phi, double *phi_lap, const double *tempr,
                                         double *tempr_lap, double *phidx, double *phidy, double *epsilon,
                                         double *epsilon_deri, void *stream);
/* snowflake/function.h:36-60 -- advances phi and tempr in place from the
 * intermediates of kernel1_pure. */
AMPS_API int amps_snowflake_kernel2_pure(const amps_params *p, double *phi, const double *phi_lap,
                                         const double *epsilon, const double *epsilon_deri, const double *phidx,
                                         const double *phidy, double *tempr, const double *tempr_lap, void *stream);
/* snowflake/tools.h:24-33 -- sets phi = 1 inside the reference's seed disc
 * (r^2 < p->init_r2 about the centre + p->init_offset); other cells untouched. */
AMPS_API int amps_snowflake_dataprepare_high(const amps_params *p, double *phi, void *stream);

/* graingrowth/function.h:5-31 -- one order parameter: etaa_lap, dfdetaa and
 * etaa_out from etaa and the other one, etab (the reference's two-grain
 * energy, cross coefficient 1). */
AMPS_API int amps_graingrowth_kernel1_pure(const amps_params *p, const double *etaa, const double *etab,
                                           double *etaa_lap, double *dfdetaa, double *etaa_out, void *stream);

/* sintering/function.h:51-79 -- con_lap, dfdcon and dummy (the chemical
 * potential) from con, eta1, eta2.  `step` is the reference's unused step index. */
AMPS_API int amps_sintering_con1_pure(const amps_params *p, const double *con, double *con_lap, const double *eta1,
                                      const double *eta2, double *dfdcon, double *dummy, int step, void *stream);
/* sintering/function.h:80-108 -- dummy_lap, then con in place (clamped to [0,1]). */
AMPS_API int amps_sintering_con2_pure(const amps_params *p, const double *dummy, double *dummy_lap, double *con,
                                      const double *eta1, const double *eta2, int step, void *stream);
/* sintering/function.h:110-134 and :135-159 -- one particle's eta: eta_lap,
 * dfdeta and eta_out (clamped to [0,1]) from eta, the other particle and con. */
AMPS_API int amps_sintering_phi1_pure(const amps_params *p, const double *eta1, double *eta1_out, const double *eta2,
                                      double *eta1_lap, double *dfdeta1, const double *con, int step, void *stream);
AMPS_API int amps_sintering_phi2_pure(const amps_params *p, const double *eta2, double *eta2_out, const double *eta1,
                                      double *eta2_lap, double *dfdeta2, const double *con, int step, void *stream);

/* snowflake/tools.h:177-193 -- Monitor1: per tile, the range of `con` over
 * the 4x4 sample lattice (scaled to p->tile); max_diff_con [nty][ntx]. */
AMPS_API int amps_get_max_diff1(const amps_params *p, const double *con, double *max_diff_con, void *stream);
/* snowflake/tools.h:194-211 -- Monitor2: per tile, max |last - now| over the
 * lattice {2,6,10,14} (scaled). */
AMPS_API int amps_get_max_diff2(const amps_params *p, const double *test_data_last, const double *test_data,
                                double *max_diffs, void *stream);
/* snowflake/tools.h:212-230 -- tile types: type_old = type_con; type_con =
 * 2 where the 5-point (non-periodic) max of max_diff_con >= p->thr_hi,
 * else 1.  int arrays [nty][ntx]. */
AMPS_API int amps_get_type(const amps_params *p, const double *max_diff_con, int *type_old, int *type_con,
                           void *stream);

/* ---- binary16 kernels (HALF2) ---------------------------------------------
 * Arrays of half2 pairs [ny][nx/2] (void *: each 32-bit element a half2 of
 * columns 2x (low) and 2x+1 (high) of a row), as the reference's purelow
 * programs keep them; periodic grids (p->bc = AMPS_BC_PERIODIC), even nx.
 * The half2 constants the reference's drivers pass (__float2half2_rn of its
 * compile-time constants) are formed from p. */

/* graingrowth/function.h:280-308 -- one order parameter of the all-half2
 * step: etaa_lap, dfdetaa, etaa_out from etaa and the other one, etab. */
AMPS_API int amps_graingrowth_kernel1_lowpure(const amps_params *p, const void *etaa, const void *etab,
                                              void *etaa_lap, void *dfdetaa, void *etaa_out, void *stream);
/* graingrowth/tools.h:54-81 -- the initial circle (radius p->init_r about
 * the centre) into two half2 arrays. */
AMPS_API int amps_graingrowth_dataprepare_half2(const amps_params *p, void *eta1, void *eta2, void *stream);
/* snowflake/function.h:607-659 -- phi_lap, tempr_lap, phidx, phidy, epsilon,
 * epsilon_deri of the all-half2 step (atan2 per half in float, h2cos/h2sin). */
AMPS_API int amps_snowflake_kernel1_purelow(const amps_params *p, const void *phi, void *phi_lap, const void *tempr,
                                            void *tempr_lap, void *phidx, void *phidy, void *epsilon,
                                            void *epsilon_deri, void *stream);
/* snowflake/function.h:660-700 -- advances phi and tempr in place. */
AMPS_API int amps_snowflake_kernel2_purelow(const amps_params *p, void *phi, const void *phi_lap, const void *epsilon,
                                            const void *epsilon_deri, const void *phidx, const void *phidy,
                                            void *tempr, const void *tempr_lap, void *stream);
/* snowflake/tools.h:43-58 -- the seed disc into a half2 phi: 1 where r^2 <
 * p->init_r2 about the centre + p->init_offset, 0 elsewhere. */
AMPS_API int amps_snowflake_dataprepare_half2(const amps_params *p, void *phi, void *stream);
/* graingrowth/tools.h:133-155, snowflake/tools.h:108-130 -- half2 pairs to
 * a float array [ny][nx]. */
AMPS_API int amps_purelow2high_aftercomputing(const amps_params *p, const void *hdata, float *fdata, void *stream);

/* ---- the adaptive grain-growth step (AMSTENCIL) ----------------------------
 * Dual storage as the reference's end2end_mix program keeps it: FP64 arrays
 * [ny][nx] and half2 arrays [ny][nx/2] of every field, and the tile types
 * type_curr [ny/tile][nx/tile] (1: half2, 2: FP64).  Square tiles of
 * p->tile (even, at most 32, dividing both sides); periodic grids, even nx.
 * The monitor step cadence is p->cadence (the reference's 10). */

/* graingrowth/function.h:33-277 -- one order parameter of the adaptive step:
 * a type-2 tile computes etaa_lap, dfdetaa, etaa_out in FP64 from the FP64
 * arrays; a type-1 tile computes hetaa_lap, hdfdetaa, hetaa_out in half2,
 * taking cells of type-2 neighbour tiles from etaa, and converts its edge
 * cells (all its cells when (i + 1) % cadence == 0) into etaa_out.  With
 * p->monitor == AMPS_MONITOR_TEM (the reference's Monitor2 build), step i
 * with i % cadence == 0 and etai == 2 first copies etaa into etaa_last: every
 * cell of a type-2 tile, the left half of a type-1 tile, as the reference's
 * kernel does. */
AMPS_API int amps_graingrowth_kernel1_mix(const amps_params *p, const double *etaa, double *etaa_last,
                                          const double *etab, double *etaa_lap, double *dfdetaa, double *etaa_out,
                                          const void *hetaa, const void *hetab, void *hetaa_lap, void *hdfdetaa,
                                          void *hetaa_out, const int *type_curr, int i, int etai, void *stream);
/* graingrowth/tools.h:24-38 -- the initial circle (radius p->init_r about
 * the centre) into two FP64 arrays. */
AMPS_API int amps_graingrowth_dataprepare_high(const amps_params *p, double *eta1, double *eta2, void *stream);
/* graingrowth/tools.h:256-271 -- tiles whose type went 2 -> 1 (old_con ->
 * new_con) take their half2 pairs of both fields from the FP64 arrays. */
AMPS_API int amps_graingrowth_data_sychro_duringcomputation(const amps_params *p, const double *eta1,
                                                            const double *eta2, void *heta1, void *heta2,
                                                            const int *old_con, const int *new_con, void *stream);
/* graingrowth/tools.h:172-200 -- type-1 tiles' half2 pairs into the FP64 array. */
AMPS_API int amps_graingrowth_data_sychro_aftercomputation(const amps_params *p, double *highdata,
                                                           const void *lowdata, const int *typedata, void *stream);
/* graingrowth/tools.h:158-171 -- every half2 pair from the FP64 array. */
AMPS_API int amps_graingrowth_highdata_to_low(const amps_params *p, const double *highdata, void *lowdata,
                                              void *stream);
/* graingrowth/function.h:323-341 -- kernel1_mix's conversion of type-1
 * tiles' cells into etaa_out as its own launch (the reference's
 * monitor_conversion_independent build). */
AMPS_API int amps_graingrowth_kernel1_conversion(const amps_params *p, double *etaa_out, const void *hetaa_out,
                                                 const int *type_curr, int i, void *stream);
/* graingrowth/function.h:311-321 -- every cell of etaa into etaa_last. */
AMPS_API int amps_graingrowth_monitor2_lastdata_store(const amps_params *p, const double *etaa, double *etaa_last,
                                                      void *stream);

/* ---- the adaptive Kobayashi step (AMSTENCIL) -------------------------------
 * The same dual storage for phi, tempr and the step's intermediates; tiles
 * of at least 4 cells a side. */

/* snowflake/function.h:63-375 -- Laplacians, gradients, epsilon and its
 * derivative: a type-2 tile in FP64 from the FP64 arrays; a type-1 tile in
 * half2, taking the cells of type-2 neighbour tiles (two cells deep, left,
 * right, up, down) from phi / tempr, and converting its edge cells of phidx,
 * phidy, epsilon, epsilon_deri into the FP64 arrays.  With p->monitor ==
 * AMPS_MONITOR_TEM, step i with i % cadence == 0 first copies phi into
 * phi_last as the reference's Monitor2 build does (a type-1 tile's left half). */
AMPS_API int amps_snowflake_kernel1_mix(const amps_params *p, const double *phi, double *phi_last, double *phi_lap,
                                        double *epsilon, double *epsilon_deri, double *phidx, double *phidy,
                                        const double *tempr, double *tempr_lap, const void *hphi, void *hphi_lap,
                                        const void *htempr, void *htempr_lap, void *hphidx, void *hphidy,
                                        void *hepsilon, void *hepsilon_deri, const int *type_curr, int i,
                                        void *stream);
/* snowflake/function.h:376-604 -- phi and tempr advanced in place, each
 * tile at its type; a type-1 tile converts its two-cell edge band (all its
 * cells when (i + 1) % cadence == 0) into phi / tempr. */
AMPS_API int amps_snowflake_mix_kernel2(const amps_params *p, double *phi, const double *phi_lap,
                                        const double *epsilon, const double *epsilon_deri, const double *phidx,
                                        const double *phidy, double *tempr, const double *tempr_lap, void *hphi,
                                        const void *hphi_lap, const void *hepsilon, const void *hepsilon_deri,
                                        const void *hphidx, const void *hphidy, void *htempr, const void *htempr_lap,
                                        const int *type_curr, int i, void *stream);
/* snowflake/function.h:715-759 -- kernel1_mix's conversion as its own launch. */
AMPS_API int amps_snowflake_kernel1_conversion(const amps_params *p, double *epsilon, double *epsilon_deri,
                                               double *phidx, double *phidy, const void *hphidx, const void *hphidy,
                                               const void *hepsilon, const void *hepsilon_deri, const int *type_curr,
                                               int i, void *stream);
/* snowflake/function.h:760-790 -- mix_kernel2's conversion as its own launch. */
AMPS_API int amps_snowflake_kernel2_conversion(const amps_params *p, double *phi, double *tempr, const void *hphi,
                                               const void *htempr, const int *type_curr, int i, void *stream);
/* snowflake/function.h:704-714, snowflake/tools.h:133-176 and 231-246 --
 * the same tools as grain growth's, for phi and tempr. */
AMPS_API int amps_snowflake_monitor2_lastdata_store(const amps_params *p, const double *phi, double *phi_last,
                                                    void *stream);
AMPS_API int amps_snowflake_data_sychro_duringcomputation(const amps_params *p, const double *phi,
                                                          const double *tempr, void *hphi, void *htempr,
                                                          const int *old_con, const int *new_con, void *stream);
AMPS_API int amps_snowflake_data_sychro_aftercomputation(const amps_params *p, double *highdata, const void *lowdata,
                                                         const int *typedata, void *stream);
AMPS_API int amps_snowflake_highdata_to_low(const amps_params *p, const double *highdata, void *lowdata,
                                            void *stream);

/* ---- the adaptive sintering step (AMSTENCIL) -------------------------------
 * The same dual storage for con, eta1, eta2 and the intermediates, but a
 * half2 word of sintering holds a tile's two halves: pair xo of tile tx (in
 * row y) holds cells tx*tile + xo (low) and tx*tile + xo + tile/2 (high),
 * as the reference packs them.  A type-2 tile keeps its first and last
 * columns in the half2 output arrays, where type-1 neighbours read them. */

/* sintering/function.h:161-330 -- con_lap, dfdcon and the chemical potential
 * dummy.  With p->monitor == AMPS_MONITOR_TEM, step i with i % cadence == 0
 * first copies every cell of con into con_last (the reference's Monitor2). */
AMPS_API int amps_sintering_con1_mix(const amps_params *p, const int *type_curr, const double *con, double *con_last,
                                     double *con_lap, const double *eta1, const double *eta2, double *dfdcon,
                                     double *dummy, const void *hcon, void *hcon_lap, const void *heta1,
                                     const void *heta2, void *hdfdcon, void *hdummy, int i, void *stream);
/* sintering/function.h:331-482 -- con advanced in place (clamped to [0, 1]). */
AMPS_API int amps_sintering_con2_mix(const amps_params *p, const int *type_curr, const double *dummy,
                                     double *dummy_lap, double *con, const double *eta1, const double *eta2,
                                     const void *hdummy, void *hdummy_lap, void *hcon, const void *heta1,
                                     const void *heta2, int i, void *stream);
/* sintering/function.h:483-628, 629-774 -- one particle's order parameter
 * into eta_out (clamped to [0, 1]). */
AMPS_API int amps_sintering_phi1_mix(const amps_params *p, const int *type_curr, const double *eta1, double *eta1_out,
                                     const double *eta2, double *eta1_lap, double *dfdeta1, const double *con,
                                     const void *heta1, void *heta1_out, const void *heta2, void *heta1_lap,
                                     void *hdfdeta1, const void *hcon, int i, void *stream);
AMPS_API int amps_sintering_phi2_mix(const amps_params *p, const int *type_curr, const double *eta2, double *eta2_out,
                                     const double *eta1, double *eta2_lap, double *dfdeta2, const double *con,
                                     const void *heta2, void *heta2_out, const void *heta1, void *heta2_lap,
                                     void *hdfdeta2, const void *hcon, int i, void *stream);
/* sintering/function.h:792-900 -- the four kernels' conversions as their own
 * launches: type-1 tiles' edge cells (all cells when (i + 1) % cadence == 0,
 * except for dummy) into the FP64 array, type-2 tiles' first and last
 * columns into the half2 array. */
AMPS_API int amps_sintering_con1_conversion(const amps_params *p, const int *type_curr, double *dummy, void *hdummy,
                                            void *stream);
AMPS_API int amps_sintering_con2_conversion(const amps_params *p, const int *type_curr, double *con, void *hcon,
                                            int i, void *stream);
AMPS_API int amps_sintering_phi1_conversion(const amps_params *p, const int *type_curr, double *eta1_out,
                                            void *heta1_out, int i, void *stream);
AMPS_API int amps_sintering_phi2_conversion(const amps_params *p, const int *type_curr, double *eta2_out,
                                            void *heta2_out, int i, void *stream);
/* sintering/function.h:778-790 -- con into con_last when i % cadence == 0. */
AMPS_API int amps_sintering_monitor2_lastdata_store(const amps_params *p, const double *con, double *con_last, int i,
                                                    void *stream);
/* sintering/tools.h:57-79 -- tiles whose type went 2 -> 1 take their pairs
 * of con, eta1, eta2 from the FP64 arrays. */
AMPS_API int amps_sintering_data_sychro_duringcomputation(const amps_params *p, const double *con,
                                                          const double *eta1, const double *eta2, void *hcon,
                                                          void *heta1, void *heta2, const int *old_con,
                                                          const int *new_con, void *stream);
/* sintering/tools.h:80-94 -- every pair from the FP64 array. */
AMPS_API int amps_sintering_dataprepare(const amps_params *p, const double *highdata, void *lowdata, void *stream);
/* sintering/tools.h:95-121 -- type-1 tiles' pairs into the FP64 array. */
AMPS_API int amps_sintering_data_sychro_aftercomputation(const amps_params *p, double *highdata, const void *lowdata,
                                                         const int *typedata, void *stream);

#ifdef __cplusplus
}
#endif
#endif
