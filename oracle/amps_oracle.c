/*
 * amps_oracle.c -- CPU FP64 oracle (TEST INFRASTRUCTURE ONLY; see amps_oracle.h).
 *
 * Restates the reference's per-cell arithmetic in the reference's own expression
 * order.  Build with -O2 -ffp-contract=off so that no multiply-add is fused:
 * the reference kernels, compiled for the CPU by oracle/ref_shim with the same
 * flags, then give identical bits (pinned by tests/test_oracle_ref.py).
 * Loops are OpenMP-parallel over rows; every cell is independent within a
 * pass, so the thread count never changes a result.
 */
#include "amps_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- RNG ---- */
static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
uint64_t orc_hash3(uint64_t seed, uint64_t a, uint64_t b)
{
    return mix64(mix64(seed ^ mix64(a)) + b);
}
double orc_uniform01(uint64_t seed, uint64_t a, uint64_t b)
{
    return (double)(orc_hash3(seed, a, b) >> 11) * 0x1.0p-53;
}

/* ------------------------------------------------------- neighbours ---- */
/* periodic wrap as in snowflake/function.h:13-18; mirror (zero flux) ghost
 * cells reflect about the domain face: -1 -> 0, -2 -> 1, n -> n-1, n+1 -> n-2. */
static inline int nb(int i, int n, int bc)
{
    if (bc == ORC_BC_PERIODIC) {
        if (i < 0) return i + n;
        if (i >= n) return i - n;
        return i;
    }
    if (i < 0) return -i - 1;
    if (i >= n) return 2 * n - i - 1;
    return i;
}

/* --------------------------------------------------------- Kobayashi ---- */
void orc_kob_init_disc(int nx, int ny, int cx, int cy, double r2, double *phi, double *T)
{
    /* snowflake/tools.h:24-33: dis1 is a float; phi is set to 1 inside only,
     * the managed allocation is zero elsewhere. */
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            float dis1 = (float)(pow((double)(x - cx), 2) + pow((double)(y - cy), 2));
            phi[(int64_t)y * nx + x] = dis1 < r2 ? 1.0 : 0.0;
            T[(int64_t)y * nx + x] = 0.0;
        }
}

void orc_kob_step(const orc_kob_params *p, double *phi, double *T, double *scratch, int64_t step)
{
    const int nx = p->nx, ny = p->ny, bc = p->bc;
    const int64_t n = (int64_t)nx * ny;
    double *phi_lap = scratch, *T_lap = scratch + n, *phidx = scratch + 2 * n,
           *phidy = scratch + 3 * n, *eps = scratch + 4 * n, *epsd = scratch + 5 * n;
    const double dxdy = p->dx * p->dy;
    /* kernel1_pure, snowflake/function.h:5-35 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
        const int ys2 = nb(y - 2, ny, bc), ya2 = nb(y + 2, ny, bc);
        for (int x = 0; x < nx; ++x) {
            const int xs1 = nb(x - 1, nx, bc), xa1 = nb(x + 1, nx, bc);
            const int xs2 = nb(x - 2, nx, bc), xa2 = nb(x + 2, nx, bc);
            const double *r = phi + (int64_t)y * nx;
            const double *t = T + (int64_t)y * nx;
            const int64_t i = (int64_t)y * nx + x;
            phi_lap[i] = r[xs1] / dxdy + r[xs2] / dxdy + r[xa1] / dxdy + r[xa2] / dxdy
                       + phi[(int64_t)ys1 * nx + x] / dxdy + phi[(int64_t)ys2 * nx + x] / dxdy
                       + phi[(int64_t)ya1 * nx + x] / dxdy + phi[(int64_t)ya2 * nx + x] / dxdy
                       - 8.0 * r[x] / dxdy;
            T_lap[i] = t[xs1] / dxdy + t[xs2] / dxdy + t[xa1] / dxdy + t[xa2] / dxdy
                     + T[(int64_t)ys1 * nx + x] / dxdy + T[(int64_t)ys2 * nx + x] / dxdy
                     + T[(int64_t)ya1 * nx + x] / dxdy + T[(int64_t)ya2 * nx + x] / dxdy
                     - 8.0 * t[x] / dxdy;
            phidx[i] = (r[xa1] - r[xs1]) / (2.0 * p->dx);
            phidy[i] = (phi[(int64_t)ya1 * nx + x] - phi[(int64_t)ys1 * nx + x]) / (2.0 * p->dy);
            const double theta = atan2(phidy[i], phidx[i]);
            eps[i] = p->epsb * (1.0 + p->delta * cos(p->aniso * (theta - p->theta0)));
            epsd[i] = -p->epsb * p->aniso * p->delta * sin(p->aniso * (theta - p->theta0));
        }
    }
    /* kernel2_pure, snowflake/function.h:36-60 (phi and T updated in place;
     * neighbour reads only touch the intermediates). */
    const double dtt = p->dt / p->tau, apc = p->alpha / p->pi;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
        for (int x = 0; x < nx; ++x) {
            const int xs1 = nb(x - 1, nx, bc), xa1 = nb(x + 1, nx, bc);
            const int64_t i = (int64_t)y * nx + x;
            const int64_t iu = (int64_t)ya1 * nx + x, id = (int64_t)ys1 * nx + x;
            const int64_t ir = (int64_t)y * nx + xa1, il = (int64_t)y * nx + xs1;
            const double phi_old = phi[i];
            const double term1 = (eps[iu] * epsd[iu] * phidx[iu] - eps[id] * epsd[id] * phidx[id]) / (2.0 * p->dy);
            const double term2 = -(eps[ir] * epsd[ir] * phidy[ir] - eps[il] * epsd[il] * phidy[il]) / (2.0 * p->dx);
            const double m = apc * atan(p->gama * (p->teq - T[i]));
            double drive = phi_old - 0.5 + m;
            if (p->noise != 0.0)
                drive = drive + p->noise * (orc_uniform01(p->seed, (uint64_t)step, (uint64_t)i) - 0.5);
            phi[i] = phi[i] + dtt * (term1 + term2 + pow(eps[i], 2) * phi_lap[i] + phi_old * (1.0 - phi_old) * drive);
            T[i] = T[i] + p->dt * T_lap[i] + p->kappa * (phi[i] - phi_old);
        }
    }
}

/* ------------------------------------------------------- grain growth ---- */
void orc_gg_init_circle(int nx, int ny, double rx, double ry, double r, double *eta1, double *eta2)
{
    /* graingrowth/tools.h:24-38 (dis1 is a float) */
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            float dis1 = (float)sqrt(pow(x - (float)rx, 2) + pow(y - (float)ry, 2));
            const int64_t i = (int64_t)y * nx + x;
            if (dis1 <= (float)r) { eta1[i] = 0; eta2[i] = 1; }
            else { eta1[i] = 1; eta2[i] = 0; }
        }
}

void orc_gg_init_uniform(int nx, int ny, int q, double amp, uint64_t seed, double *const *eta)
{
    /* no reference counterpart: eta_i ~ U[-amp, amp) i.i.d., keyed by
     * (seed, field, cell) through the counter-based generator above */
    const int64_t n = (int64_t)nx * ny;
    for (int f = 0; f < q; ++f)
        for (int64_t i = 0; i < n; ++i) eta[f][i] = amp * (2.0 * orc_uniform01(seed, (uint64_t)f, (uint64_t)i) - 1.0);
}

void orc_gg_step(const orc_gg_params *p, double *const *eta_in, double *const *eta_out)
{
    const int nx = p->nx, ny = p->ny, bc = p->bc, q = p->q;
    const double dxdy = p->dx * p->dy, dtm = p->dt * p->mobil, g2 = 2.0 * p->gamma;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
        for (int x = 0; x < nx; ++x) {
            const int xs1 = nb(x - 1, nx, bc), xa1 = nb(x + 1, nx, bc);
            const int64_t i = (int64_t)y * nx + x;
            for (int a = 0; a < q; ++a) {
                const double *e = eta_in[a];
                const double *rd = e + (int64_t)ys1 * nx, *rc = e + (int64_t)y * nx, *ru = e + (int64_t)ya1 * nx;
                double lap;
                if (p->stencil == 0) /* graingrowth/function.h:20 */
                    lap = (rd[xs1] + rd[x] + rd[xa1] + rc[xs1] + rc[xa1] + ru[xs1] + ru[x] + ru[xa1] - 8.0 * rc[x]) / dxdy;
                else
                    lap = (rc[xs1] + rc[xa1] + rd[x] + ru[x] - 4.0 * rc[x]) / dxdy;
                double sum = 0.0;
                int first = 1;
                for (int b = 0; b < q; ++b) {
                    if (b == a) continue;
                    const double s = pow(eta_in[b][i], 2);
                    sum = first ? s : sum + s;
                    first = 0;
                }
                const double ea = rc[x];
                /* graingrowth/function.h:21-23 with 2.0*1.0 -> 2.0*gamma */
                const double dfd = 1.0 * (g2 * ea * sum + pow(ea, 3) - ea);
                eta_out[a][i] = ea - dtm * (dfd - p->grcoef * lap);
            }
        }
    }
}

/* The timed CPU baseline of the same update (not a checker): fields outer,
 * one row at a time, the per-cell sum of squares S = sum_b eta_b^2 formed
 * once per row and sum_{b!=a} taken as S - eta_a^2, so the interior loop
 * over x is branch-free and vectorises.  Agrees with orc_gg_step to rounding
 * (tests/test_oracle_golden.py). */
static inline double gg_cell_fast(int stencil, const double *rd, const double *rc, const double *ru, int xs1,
                                  int x, int xa1, double S, double inv, double dtm, double g2, double kap)
{
    const double lap = stencil == 0
                           ? rd[xs1] + rd[x] + rd[xa1] + rc[xs1] + rc[xa1] + ru[xs1] + ru[x] + ru[xa1] - 8.0 * rc[x]
                           : rc[xs1] + rc[xa1] + rd[x] + ru[x] - 4.0 * rc[x];
    const double ea = rc[x];
    const double dfd = g2 * ea * (S - ea * ea) + ea * ea * ea - ea;
    return ea - dtm * (dfd - kap * lap * inv);
}

static void gg_row_fast(const orc_gg_params *p, double *const *eta_in, double *const *eta_out, int y,
                        double *S)
{
    const int nx = p->nx, ny = p->ny, bc = p->bc, q = p->q, st = p->stencil;
    const double inv = 1.0 / (p->dx * p->dy), dtm = p->dt * p->mobil, g2 = 2.0 * p->gamma, kap = p->grcoef;
    const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
    for (int x = 0; x < nx; ++x) S[x] = 0.0;
    for (int b = 0; b < q; ++b) {
        const double *restrict e = eta_in[b] + (int64_t)y * nx;
        for (int x = 0; x < nx; ++x) S[x] += e[x] * e[x];
    }
    for (int a = 0; a < q; ++a) {
        const double *restrict rd = eta_in[a] + (int64_t)ys1 * nx;
        const double *restrict rc = eta_in[a] + (int64_t)y * nx;
        const double *restrict ru = eta_in[a] + (int64_t)ya1 * nx;
        double *restrict o = eta_out[a] + (int64_t)y * nx;
        /* edge columns through the boundary map, the interior branch-free */
        o[0] = gg_cell_fast(st, rd, rc, ru, nb(-1, nx, bc), 0, nb(1, nx, bc), S[0], inv, dtm, g2, kap);
        for (int x = 1; x < nx - 1; ++x)
            o[x] = gg_cell_fast(st, rd, rc, ru, x - 1, x, x + 1, S[x], inv, dtm, g2, kap);
        if (nx > 1)
            o[nx - 1] = gg_cell_fast(st, rd, rc, ru, nx - 2, nx - 1, nb(nx, nx, bc), S[nx - 1], inv, dtm, g2, kap);
    }
}

void orc_gg_step_fast(const orc_gg_params *p, double *const *eta_in, double *const *eta_out)
{
#pragma omp parallel
    {
        double *S = (double *)malloc((size_t)p->nx * sizeof(double));
#pragma omp for schedule(static)
        for (int y = 0; y < p->ny; ++y) gg_row_fast(p, eta_in, eta_out, y, S);
        free(S);
    }
}

/* ---------------------------------------------------------- sintering ---- */
void orc_sint_init_two(int nx, int ny, double rx1, double ry1, double r1, double ry2, double r2,
                       double *c, double *eta1, double *eta2)
{
    /* sintering/main.cu:45-59 (1-based loop indices, float distances) */
    const int64_t n = (int64_t)nx * ny;
    memset(c, 0, n * sizeof(double));
    memset(eta1, 0, n * sizeof(double));
    memset(eta2, 0, n * sizeof(double));
    for (int y = 1; y <= ny; ++y)
        for (int x = 1; x <= nx; ++x) {
            float dis1 = (float)sqrt(pow(x - (float)rx1, 2) + pow(y - (float)ry1, 2));
            float dis2 = (float)sqrt(pow(x - (float)rx1, 2) + pow(y - (float)ry2, 2));
            const int64_t i = (int64_t)(y - 1) * nx + x - 1;
            if (dis1 <= (float)r1) { c[i] = 1; eta1[i] = 1; }
            if (dis2 <= (float)r2) { c[i] = 1; eta2[i] = 1; eta1[i] = 0.0; }
        }
}

void orc_sint_step(const orc_sint_params *p, double *c, double *const *eta_in,
                   double *const *eta_out, double *scratch)
{
    const int nx = p->nx, ny = p->ny, bc = p->bc, np = p->n;
    const int64_t n = (int64_t)nx * ny;
    double *mu = scratch;
    const double dxdy = p->dx * p->dy;
    const double A2 = 2.0 * p->A;
    /* con1_pure, sintering/function.h:51-79 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
        for (int x = 0; x < nx; ++x) {
            const int xs1 = nb(x - 1, nx, bc), xa1 = nb(x + 1, nx, bc);
            const int64_t i = (int64_t)y * nx + x;
            const double cc = c[i];
            const double lap = (c[(int64_t)y * nx + xs1] + c[(int64_t)y * nx + xa1] + c[(int64_t)ys1 * nx + x]
                                + c[(int64_t)ya1 * nx + x] - 4.0 * cc) / dxdy;
            double sum2 = pow(eta_in[0][i], 2), sum3 = pow(eta_in[0][i], 3);
            for (int k = 1; k < np; ++k) {
                sum2 = sum2 + pow(eta_in[k][i], 2);
                sum3 = sum3 + pow(eta_in[k][i], 3);
            }
            const double dfdc = p->B * (2.0 * cc + 4.0 * sum3 - 6.0 * sum2) - A2 * pow(cc, 2) * (1.0 - cc)
                              + A2 * cc * pow(1.0 - cc, 2);
            mu[i] = dfdc - 0.5 * p->coefm * lap;
        }
    }
    /* con2_pure, sintering/function.h:80-108 (c updated in place, clamped) */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
        for (int x = 0; x < nx; ++x) {
            const int xs1 = nb(x - 1, nx, bc), xa1 = nb(x + 1, nx, bc);
            const int64_t i = (int64_t)y * nx + x;
            const double lapm = (mu[(int64_t)y * nx + xs1] + mu[(int64_t)y * nx + xa1] + mu[(int64_t)ys1 * nx + x]
                                 + mu[(int64_t)ya1 * nx + x] - 4.0 * mu[i]) / dxdy;
            const double cc = c[i];
            const double phi = pow(cc, 3) * (10.0 - 15.0 * cc + 6.0 * pow(cc, 2));
            double sum = 0.0;
            for (int a = 0; a < np; ++a)
                for (int b = a + 1; b < np; ++b)
                    sum = sum + eta_in[a][i] * eta_in[b][i] * 2;
            const double mobil = p->dvol * phi + p->dvap * (1.0 - phi) + p->dsur * cc * (1.0 - cc) + p->dgrb * sum;
            double cn = cc + p->dt * mobil * lapm;
            if (cn >= 1) cn = 1;
            else if (cn < 0) cn = 0;
            scratch[n + i] = cn;
        }
    }
    memcpy(c, scratch + n, n * sizeof(double));
    /* phi1_pure / phi2_pure, sintering/function.h:110-159 */
    const double dtl = p->dt * p->coefl, hk = 0.5 * p->coefk;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        const int ys1 = nb(y - 1, ny, bc), ya1 = nb(y + 1, ny, bc);
        for (int x = 0; x < nx; ++x) {
            const int xs1 = nb(x - 1, nx, bc), xa1 = nb(x + 1, nx, bc);
            const int64_t i = (int64_t)y * nx + x;
            const double cc = c[i];
            double sum2 = pow(eta_in[0][i], 2);
            for (int k = 1; k < np; ++k) sum2 = sum2 + pow(eta_in[k][i], 2);
            for (int a = 0; a < np; ++a) {
                const double *e = eta_in[a];
                const double ea = e[i];
                const double lap = (e[(int64_t)y * nx + xs1] + e[(int64_t)y * nx + xa1] + e[(int64_t)ys1 * nx + x]
                                    + e[(int64_t)ya1 * nx + x] - 4.0 * ea) / dxdy;
                const double dfd = p->B * (-12.0 * pow(ea, 2) * (2.0 - cc) + 12.0 * ea * (1.0 - cc) + 12.0 * ea * sum2);
                double out = ea - dtl * (dfd - hk * lap);
                if (out >= 1) out = 1;
                else if (out < 0) out = 0;
                eta_out[a][i] = out;
            }
        }
    }
}

/* ------------------------------------------------------------ monitor ---- */
void orc_sample_points(int tile, int kind, int *pts4)
{
    /* kind 1 (spatial): {0,5,10,15} for 16-wide tiles (snowflake/tools.h:185);
     * kind 2 (temporal): {2,6,10,14} (snowflake/tools.h:203); scaled to the tile. */
    for (int k = 0; k < 4; ++k)
        pts4[k] = kind == 1 ? (int)floor(k * (tile - 1) / 3.0 + 0.5) : tile / 8 + k * (tile / 4);
}

void orc_monitor_spa(const double *f, int nx, int ny, int tile, int samples, double *metric)
{
    /* a side that is not a multiple of the tile: partial edge tiles, whose
     * samples past the domain are skipped */
    const int ntx = (nx + tile - 1) / tile, nty = (ny + tile - 1) / tile;
    int pts[4];
    orc_sample_points(tile, 1, pts);
    for (int ty = 0; ty < nty; ++ty)
        for (int tx = 0; tx < ntx; ++tx) {
            /* the reference starts from min=1, max=0 (snowflake/tools.h:184);
             * the every-cell mode uses the true range. */
            double mn = samples ? INFINITY : 1.0, mx = samples ? -INFINITY : 0.0;
            const int cnt = samples ? tile : 4;
            for (int j = 0; j < cnt; ++j)
                for (int k = 0; k < cnt; ++k) {
                    const int y = ty * tile + (samples ? j : pts[j]);
                    const int x = tx * tile + (samples ? k : pts[k]);
                    if (x >= nx || y >= ny) continue;
                    const double v = f[(int64_t)y * nx + x];
                    if (v < mn) mn = v;
                    if (v > mx) mx = v;
                }
            metric[ty * ntx + tx] = mx - mn;
        }
}

void orc_monitor_tem(const double *f, const double *last, int nx, int ny, int tile, int samples,
                     double *metric)
{
    /* a side that is not a multiple of the tile: partial edge tiles, whose
     * samples past the domain are skipped */
    const int ntx = (nx + tile - 1) / tile, nty = (ny + tile - 1) / tile;
    int pts[4];
    orc_sample_points(tile, 2, pts);
    for (int ty = 0; ty < nty; ++ty)
        for (int tx = 0; tx < ntx; ++tx) {
            double mx = 0.0;
            const int cnt = samples ? tile : 4;
            for (int j = 0; j < cnt; ++j)
                for (int k = 0; k < cnt; ++k) {
                    const int y = ty * tile + (samples ? j : pts[j]);
                    const int x = tx * tile + (samples ? k : pts[k]);
                    if (x >= nx || y >= ny) continue;
                    const double d = fabs(last[(int64_t)y * nx + x] - f[(int64_t)y * nx + x]);
                    if (d > mx) mx = d;
                }
            metric[ty * ntx + tx] = mx;
        }
}

void orc_monitor_rate(const double *f, const double *prev, int nx, int ny, int tile, int samples, int cadence,
                      double *metric)
{
    /* defined in FP32 arithmetic: max |float(f) - float(prev)|, times the cadence in double */
    /* a side that is not a multiple of the tile: partial edge tiles, whose
     * samples past the domain are skipped */
    const int ntx = (nx + tile - 1) / tile, nty = (ny + tile - 1) / tile;
    int pts[4];
    orc_sample_points(tile, 2, pts);
    for (int ty = 0; ty < nty; ++ty)
        for (int tx = 0; tx < ntx; ++tx) {
            float mx = 0.f;
            const int cnt = samples ? tile : 4;
            for (int j = 0; j < cnt; ++j)
                for (int k = 0; k < cnt; ++k) {
                    const int y = ty * tile + (samples ? j : pts[j]);
                    const int x = tx * tile + (samples ? k : pts[k]);
                    if (x >= nx || y >= ny) continue;
                    const int64_t i = (int64_t)y * nx + x;
                    const float d = fabsf((float)f[i] - (float)prev[i]);
                    if (d > mx) mx = d;
                }
            metric[ty * ntx + tx] = (double)mx * cadence;
        }
}

void orc_classify(const double *metric, int ntx, int nty, double thr_lo, double thr_hi, uint8_t *tier)
{
    for (int ty = 0; ty < nty; ++ty)
        for (int tx = 0; tx < ntx; ++tx) {
            double m = metric[ty * ntx + tx];
            if (ty < nty - 1 && metric[(ty + 1) * ntx + tx] > m) m = metric[(ty + 1) * ntx + tx];
            if (ty > 0 && metric[(ty - 1) * ntx + tx] > m) m = metric[(ty - 1) * ntx + tx];
            if (tx < ntx - 1 && metric[ty * ntx + tx + 1] > m) m = metric[ty * ntx + tx + 1];
            if (tx > 0 && metric[ty * ntx + tx - 1] > m) m = metric[ty * ntx + tx - 1];
            tier[ty * ntx + tx] = m >= thr_hi ? 2 : (m >= thr_lo ? 1 : 0);
        }
}

/* -------------------------------------------------------- diagnostics ---- */
double orc_max_abs_diff(const double *a, const double *b, int64_t n)
{
    double m = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double d = fabs(a[i] - b[i]);
        if (d > m || d != d) m = d;
    }
    return m;
}
double orc_l2_diff(const double *a, const double *b, int64_t n)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += (a[i] - b[i]) * (a[i] - b[i]);
    return sqrt(s / (double)n);
}
double orc_sum(const double *a, int64_t n)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += a[i];
    return s;
}
