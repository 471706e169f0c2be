/*
 * amps_oracle.h -- CPU FP64 oracle for the adaptive mixed-precision phase-field
 * stencil path (Kobayashi dendrite, grain growth, sintering).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: tests/, the smoke entry and
 * the CPU-baseline leg of bench.py call it; the product library never links,
 * loads or calls it.
 *
 * Every function restates one piece of the reference's algorithm in plain C,
 * keeping the reference's expression order (per-term divisions, pow() calls,
 * left-to-right sums) so that, compiled with -ffp-contract=off, it reproduces
 * the reference kernels bit for bit.  That claim is pinned by
 * tests/test_oracle_ref.py against the reference's own kernels compiled for the
 * CPU (oracle/ref_shim/, built into oracle/_ref/).
 *
 * Layout: every field is a row-major double array [ny][nx].
 */
#ifndef AMPS_ORACLE_H
#define AMPS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BC_PERIODIC = 0, ORC_BC_NOFLUX = 1 };

/* ---- counter-based RNG (splitmix64 finaliser; Steele, Lea & Flood 2014) ---- */
uint64_t orc_hash3(uint64_t seed, uint64_t a, uint64_t b);
double orc_uniform01(uint64_t seed, uint64_t a, uint64_t b);

/* ---- Kobayashi dendrite ------------------------------------------------- */
typedef struct {
    int nx, ny, bc;
    double dx, dy, tau, epsb, kappa, delta, aniso, alpha, gama, teq, theta0, dt;
    double pi;          /* the reference's pi macro (3.1415926) */
    double noise;       /* amplitude a of the driving-term noise a*chi, chi in [-1/2,1/2) */
    uint64_t seed;
} orc_kob_params;

/* One explicit step: snowflake/function.h:5-60 (kernel1_pure + kernel2_pure).
 * scratch holds 6*nx*ny doubles (lap phi, lap T, phix, phiy, eps, eps'). */
void orc_kob_step(const orc_kob_params *p, double *phi, double *T, double *scratch, int64_t step);
/* Initial disc: snowflake/tools.h:24-33 (phi=1 where (x-cx)^2+(y-cy)^2 < r2). */
void orc_kob_init_disc(int nx, int ny, int cx, int cy, double r2, double *phi, double *T);

/* ---- grain growth (Allen-Cahn, Q order parameters) --------------------- */
typedef struct {
    int nx, ny, bc, q;
    int stencil;        /* 0 = reference 8-neighbour, 1 = 5-point */
    double dx, dy, dt, mobil, grcoef, gamma;
} orc_gg_params;

/* One step for all q fields (Jacobi: every field reads the old fields).
 * graingrowth/function.h:5-30 generalised to q fields:
 * dfd_i = 1.0*(2.0*gamma*eta_i*sum_{j!=i} pow(eta_j,2) + pow(eta_i,3) - eta_i). */
void orc_gg_step(const orc_gg_params *p, double *const *eta_in, double *const *eta_out);
/* The same update restructured for speed (fields outer, a row at a time,
 * sum_{j!=i} eta_j^2 as S - eta_i^2): the timed CPU baseline, not a checker;
 * equal to orc_gg_step to rounding. */
void orc_gg_step_fast(const orc_gg_params *p, double *const *eta_in, double *const *eta_out);
/* Circle initial state: graingrowth/tools.h:24-38 (eta2=1 inside radius R). */
void orc_gg_init_circle(int nx, int ny, double rx, double ry, double r, double *eta1, double *eta2);

/* Seeded start of the multi-grain workloads (no reference counterpart):
 * eta_i ~ U[-amp, amp) i.i.d. from orc_uniform01(seed, i, cell). */
void orc_gg_init_uniform(int nx, int ny, int q, double amp, uint64_t seed, double *const *eta);

/* ---- sintering (Cahn-Hilliard c + Allen-Cahn eta_i) -------------------- */
typedef struct {
    int nx, ny, bc, n;
    double dx, dy, dt, coefm, coefk, coefl, dvol, dvap, dsur, dgrb;
    double A, B;        /* bulk free-energy coefficients (reference: A=16, B=1) */
} orc_sint_params;

/* One step: sintering/function.h:51-159 (con1, con2, phi1..phiN), operator
 * split as in sintering/main.cu:136-147: c updated in place first, then every
 * eta_i from the new c and the old eta_j.  scratch: 3*nx*ny doubles. */
void orc_sint_step(const orc_sint_params *p, double *c, double *const *eta_in,
                   double *const *eta_out, double *scratch);
/* Two touching discs: sintering/main.cu:45-59. */
void orc_sint_init_two(int nx, int ny, double rx1, double ry1, double r1, double ry2, double r2,
                       double *c, double *eta1, double *eta2);

/* ---- precision monitor and tile classification ------------------------- */
/* Monitor1 (spatial range) on a tile lattice: snowflake/tools.h:177-193.
 * samples==0: the reference's 4x4 lattice scaled to the tile; 1: every cell. */
void orc_monitor_spa(const double *f, int nx, int ny, int tile, int samples, double *metric);
/* Monitor2 (temporal change): snowflake/tools.h:194-211. */
void orc_monitor_tem(const double *f, const double *last, int nx, int ny, int tile, int samples,
                     double *metric);
/* Per-step change times the cadence (no reference counterpart: the
 * snapshot-free estimate of Monitor2), in FP32 arithmetic; lattice of the
 * temporal monitor. */
void orc_monitor_rate(const double *f, const double *prev, int nx, int ny, int tile, int samples, int cadence,
                      double *metric);
/* get_type: snowflake/tools.h:212-230 -- max over the tile and its 4 tile
 * neighbours (not periodic), then thresholds.  Three tiers: metric >= thr_hi
 * -> 2 (FP64), >= thr_lo -> 1 (FP32), else 0 (half).  The reference's two-tier
 * rule is thr_lo == thr_hi. */
void orc_classify(const double *metric, int ntx, int nty, double thr_lo, double thr_hi,
                  uint8_t *tier);
/* Sample offsets of the reference lattices for a tile of side `tile`. */
void orc_sample_points(int tile, int kind, int *pts4);

/* ---- diagnostics -------------------------------------------------------- */
double orc_max_abs_diff(const double *a, const double *b, int64_t n);
double orc_l2_diff(const double *a, const double *b, int64_t n);
double orc_sum(const double *a, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
