// compat.cu -- the reference's plain-FP64 kernels and monitor tools under
// their own names, as host launch wrappers over caller-owned device arrays
// (include/amps_compat.h).  One thread per cell on a 2-D grid; each cell's
// arithmetic follows the reference kernel's expression order term by term
// (this file is compiled with -fmad=false, so no multiply-add is fused and
// the FP64 results are the reference kernels' own, up to the device libm).
// The compile-time constants of the reference come from an amps_params.
#include "../../include/amps_compat.h"
#include "amps_internal.cuh"

#include <math.h>

namespace {

using amps::bc_map;

constexpr int kBX = 32, kBY = 8;

struct Geo {
    int nx, ny, bc;
};

__device__ __forceinline__ bool cell(const Geo &g, int &x, int &y)
{
    x = blockIdx.x * kBX + threadIdx.x;
    y = blockIdx.y * kBY + threadIdx.y;
    return x < g.nx && y < g.ny;
}

// The reference's pow(x, 2): glibc returns the correctly rounded square,
// which is the product x * x rounded once (the device pow may differ by an
// ulp).  Cubes keep pow.
__device__ __forceinline__ double sq(double x) { return x * x; }

__device__ __forceinline__ int64_t at(const Geo &g, int x, int y)
{
    return (int64_t)bc_map(y, g.ny, g.bc) * g.nx + bc_map(x, g.nx, g.bc);
}

struct KobC {
    double dx, dy, dxdy, epsb, delta, aniso, theta0, alpha, pi, gama, teq, dt, tau, kappa;
};

// snowflake/function.h:27-34
__global__ void snowflake_k1(Geo g, KobC c, const double *phi, double *phi_lap, const double *tempr,
                             double *tempr_lap, double *phidx, double *phidy, double *eps, double *epsd)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const int64_t i = (int64_t)y * g.nx + x;
    const double d = c.dxdy;
    phi_lap[i] = phi[at(g, x - 1, y)] / d + phi[at(g, x - 2, y)] / d + phi[at(g, x + 1, y)] / d +
                 phi[at(g, x + 2, y)] / d + phi[at(g, x, y - 1)] / d + phi[at(g, x, y - 2)] / d +
                 phi[at(g, x, y + 1)] / d + phi[at(g, x, y + 2)] / d - 8.0 * phi[i] / d;
    tempr_lap[i] = tempr[at(g, x - 1, y)] / d + tempr[at(g, x - 2, y)] / d + tempr[at(g, x + 1, y)] / d +
                   tempr[at(g, x + 2, y)] / d + tempr[at(g, x, y - 1)] / d + tempr[at(g, x, y - 2)] / d +
                   tempr[at(g, x, y + 1)] / d + tempr[at(g, x, y + 2)] / d - 8.0 * tempr[i] / d;
    const double px = (phi[at(g, x + 1, y)] - phi[at(g, x - 1, y)]) / (2.0 * c.dx);
    const double py = (phi[at(g, x, y + 1)] - phi[at(g, x, y - 1)]) / (2.0 * c.dy);
    phidx[i] = px;
    phidy[i] = py;
    const double theta = atan2(py, px);
    eps[i] = c.epsb * (1.0 + c.delta * cos(c.aniso * (theta - c.theta0)));
    epsd[i] = -c.epsb * c.aniso * c.delta * sin(c.aniso * (theta - c.theta0));
}

// snowflake/function.h:54-59
__global__ void snowflake_k2(Geo g, KobC c, double *phi, const double *phi_lap, const double *eps,
                             const double *epsd, const double *phidx, const double *phidy, double *tempr,
                             const double *tempr_lap)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const int64_t i = (int64_t)y * g.nx + x;
    const int64_t n = at(g, x, y + 1), s = at(g, x, y - 1), e = at(g, x + 1, y), w = at(g, x - 1, y);
    const double p0 = phi[i];
    const double term1 = (eps[n] * epsd[n] * phidx[n] - eps[s] * epsd[s] * phidx[s]) / (2.0 * c.dy);
    const double term2 = -(eps[e] * epsd[e] * phidy[e] - eps[w] * epsd[w] * phidy[w]) / (2.0 * c.dx);
    const double m = c.alpha / c.pi * atan(c.gama * (c.teq - tempr[i]));
    const double pn = p0 + (c.dt / c.tau) * (term1 + term2 + sq(eps[i]) * phi_lap[i] + p0 * (1.0 - p0) * (p0 - 0.5 + m));
    phi[i] = pn;
    tempr[i] = tempr[i] + c.dt * tempr_lap[i] + c.kappa * (pn - p0);
}

// snowflake/tools.h:24-33 (the seed disc; distance in float as there)
__global__ void snowflake_prep(Geo g, double r2, int off, double *phi)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const float dis = pow(x - (g.nx / 2 + off), 2) + pow(y - (g.ny / 2 + off), 2);
    if (dis < r2) phi[(int64_t)y * g.nx + x] = 1;
}

// graingrowth/function.h:20-23
__global__ void gg_k1(Geo g, double dxdy, double dt, double mobil, double grcoef, const double *a, const double *b,
                      double *lap, double *dfd, double *out)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const int64_t i = (int64_t)y * g.nx + x;
    const double l = (a[at(g, x - 1, y - 1)] + a[at(g, x, y - 1)] + a[at(g, x + 1, y - 1)] + a[at(g, x - 1, y)] +
                      a[at(g, x + 1, y)] + a[at(g, x - 1, y + 1)] + a[at(g, x, y + 1)] + a[at(g, x + 1, y + 1)] -
                      8.0 * a[i]) / dxdy;
    lap[i] = l;
    const double sum = sq(b[i]);
    const double f = 1.0 * (2.0 * 1.0 * a[i] * sum + pow(a[i], 3) - a[i]);
    dfd[i] = f;
    out[i] = a[i] - dt * mobil * (f - grcoef * l);
}

struct SintC {
    double dxdy, dt, coefm, coefk, coefl, dvol, dvap, dsur, dgrb, A2, B;
};

__device__ __forceinline__ double lap5(const Geo &g, const double *f, int x, int y, int64_t i, double dxdy)
{
    return (f[at(g, x - 1, y)] + f[at(g, x + 1, y)] + f[at(g, x, y - 1)] + f[at(g, x, y + 1)] - 4.0 * f[i]) / dxdy;
}

// sintering/function.h:66-70
__global__ void sint_con1(Geo g, SintC c, const double *con, double *con_lap, const double *e1, const double *e2,
                          double *dfdcon, double *dummy)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const int64_t i = (int64_t)y * g.nx + x;
    const double l = lap5(g, con, x, y, i, c.dxdy);
    con_lap[i] = l;
    const double cc = con[i];
    const double sum2 = sq(e1[i]) + sq(e2[i]);
    const double sum3 = pow(e1[i], 3) + pow(e2[i], 3);
    const double f = c.B * (2.0 * cc + 4.0 * sum3 - 6.0 * sum2) - c.A2 * sq(cc) * (1.0 - cc) +
                     c.A2 * cc * sq(1.0 - cc);
    dfdcon[i] = f;
    dummy[i] = f - 0.5 * c.coefm * l;
}

// sintering/function.h:95-101
__global__ void sint_con2(Geo g, SintC c, const double *dummy, double *dummy_lap, double *con, const double *e1,
                          const double *e2)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const int64_t i = (int64_t)y * g.nx + x;
    const double l = lap5(g, dummy, x, y, i, c.dxdy);
    dummy_lap[i] = l;
    const double cc = con[i];
    const double phi = pow(cc, 3) * (10.0 - 15.0 * cc + 6.0 * sq(cc));
    const double sum = e1[i] * e2[i] * 2;
    const double mobil = c.dvol * phi + c.dvap * (1.0 - phi) + c.dsur * cc * (1.0 - cc) + c.dgrb * sum;
    double v = cc + c.dt * mobil * l;
    if (v >= 1) v = 1;
    else if (v < 0) v = 0;
    con[i] = v;
}

// sintering/function.h:126-133 (phi1) and :151-158 (phi2): one particle
__global__ void sint_phi(Geo g, SintC c, const double *ea, double *ea_out, const double *eb, double *ea_lap,
                         double *dfd, const double *con)
{
    int x, y;
    if (!cell(g, x, y)) return;
    const int64_t i = (int64_t)y * g.nx + x;
    const double l = lap5(g, ea, x, y, i, c.dxdy);
    ea_lap[i] = l;
    const double sum2 = sq(ea[i]) + sq(eb[i]);
    const double f = c.B * (-12.0 * sq(ea[i]) * (2.0 - con[i]) + 12.0 * ea[i] * (1.0 - con[i]) + 12.0 * ea[i] * sum2);
    dfd[i] = f;
    double v = ea[i] - c.dt * c.coefl * (f - 0.5 * c.coefk * l);
    if (v >= 1) v = 1;
    else if (v < 0) v = 0;
    ea_out[i] = v;
}

// snowflake/tools.h:177-211: one thread per tile
__global__ void max_diff(int nx, int ntx, int nty, int tile, int kind, const double *last, const double *now,
                         double *out)
{
    const int tx = blockIdx.x * blockDim.x + threadIdx.x, ty = blockIdx.y * blockDim.y + threadIdx.y;
    if (tx >= ntx || ty >= nty) return;
    // the reference's lattices {0,5,10,15} / {2,6,10,14} for 16-cell tiles,
    // scaled to the tile as the library's monitor does
    int pp[4];
    for (int k = 0; k < 4; ++k) pp[k] = kind == 1 ? (int)floor(k * (tile - 1) / 3.0 + 0.5) : tile / 8 + k * (tile / 4);
    double mn = 1.0, mx = 0.0, md = 0.0;
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i) {
            const int64_t k = (int64_t)(ty * tile + pp[j]) * nx + tx * tile + pp[i];
            if (kind == 1) {
                if (now[k] < mn) mn = now[k];
                if (now[k] > mx) mx = now[k];
            } else {
                const double d = fabs(last[k] - now[k]);
                if (d > md) md = d;
            }
        }
    out[ty * ntx + tx] = kind == 1 ? mx - mn : md;
}

// snowflake/tools.h:212-230
__global__ void get_type_k(int ntx, int nty, double thr, const double *md, int *old, int *cur)
{
    const int tx = blockIdx.x * blockDim.x + threadIdx.x, ty = blockIdx.y * blockDim.y + threadIdx.y;
    if (tx >= ntx || ty >= nty) return;
    const int t = ty * ntx + tx;
    old[t] = cur[t];
    double m = md[t];
    m = ty < nty - 1 ? fmax(m, md[t + ntx]) : m;
    m = ty > 0 ? fmax(m, md[t - ntx]) : m;
    m = tx < ntx - 1 ? fmax(m, md[t + 1]) : m;
    m = tx > 0 ? fmax(m, md[t - 1]) : m;
    if (m < thr) cur[t] = 1;
    else if (m >= thr) cur[t] = 2;
}

int check_grid(const amps_params *p)
{
    if (!p || p->nx < 3 || p->ny < 3 || (p->bc != AMPS_BC_PERIODIC && p->bc != AMPS_BC_NOFLUX)) return AMPS_ERR_INVALID;
    return AMPS_OK;
}

int check_tiles(const amps_params *p)
{
    if (check_grid(p) || (p->tile != 16 && p->tile != 32) || p->nx % p->tile || p->ny % p->tile)
        return AMPS_ERR_INVALID;
    return AMPS_OK;
}

Geo geo(const amps_params *p) { return Geo{p->nx, p->ny, p->bc}; }
dim3 grid2(const amps_params *p) { return dim3((p->nx + kBX - 1) / kBX, (p->ny + kBY - 1) / kBY); }
dim3 tgrid(const amps_params *p) { return dim3((p->nx / p->tile + 15) / 16, (p->ny / p->tile + 15) / 16); }

KobC kobc(const amps_params *p)
{
    return KobC{p->dx, p->dy, p->dx * p->dy, p->epsb, p->delta, p->aniso, p->theta0, p->alpha, p->pi, p->gama, p->teq,
                p->dt, p->tau, p->kappa};
}

SintC sintc(const amps_params *p)
{
    return SintC{p->dx * p->dy, p->dt, p->coefm, p->coefk, p->coefl, p->dvol, p->dvap, p->dsur, p->dgrb,
                 2.0 * p->A, p->B};
}

int launched() { return cudaGetLastError() == cudaSuccess ? AMPS_OK : AMPS_ERR_CUDA; }

}  // namespace

#define S_ (cudaStream_t) stream

extern "C" int amps_snowflake_kernel1_pure(const amps_params *p, const double *phi, double *phi_lap,
                                           const double *tempr, double *tempr_lap, double *phidx, double *phidy,
                                           double *epsilon, double *epsilon_deri, void *stream)
{
    if (check_grid(p) || !phi || !phi_lap || !tempr || !tempr_lap || !phidx || !phidy || !epsilon || !epsilon_deri)
        return AMPS_ERR_INVALID;
    snowflake_k1<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), kobc(p), phi, phi_lap, tempr, tempr_lap, phidx, phidy,
                                                      epsilon, epsilon_deri);
    return launched();
}

extern "C" int amps_snowflake_kernel2_pure(const amps_params *p, double *phi, const double *phi_lap,
                                           const double *epsilon, const double *epsilon_deri, const double *phidx,
                                           const double *phidy, double *tempr, const double *tempr_lap, void *stream)
{
    if (check_grid(p) || !phi || !phi_lap || !tempr || !tempr_lap || !phidx || !phidy || !epsilon || !epsilon_deri)
        return AMPS_ERR_INVALID;
    snowflake_k2<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), kobc(p), phi, phi_lap, epsilon, epsilon_deri, phidx,
                                                      phidy, tempr, tempr_lap);
    return launched();
}

extern "C" int amps_snowflake_dataprepare_high(const amps_params *p, double *phi, void *stream)
{
    if (check_grid(p) || !phi) return AMPS_ERR_INVALID;
    snowflake_prep<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), p->init_r2, p->init_offset, phi);
    return launched();
}

extern "C" int amps_graingrowth_kernel1_pure(const amps_params *p, const double *etaa, const double *etab,
                                             double *etaa_lap, double *dfdetaa, double *etaa_out, void *stream)
{
    if (check_grid(p) || !etaa || !etab || !etaa_lap || !dfdetaa || !etaa_out || etaa == etaa_out)
        return AMPS_ERR_INVALID;
    gg_k1<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), p->dx * p->dy, p->dt, p->mobil, p->grcoef, etaa, etab,
                                               etaa_lap, dfdetaa, etaa_out);
    return launched();
}

extern "C" int amps_sintering_con1_pure(const amps_params *p, const double *con, double *con_lap, const double *eta1,
                                        const double *eta2, double *dfdcon, double *dummy, int step, void *stream)
{
    (void)step;
    if (check_grid(p) || !con || !con_lap || !eta1 || !eta2 || !dfdcon || !dummy) return AMPS_ERR_INVALID;
    sint_con1<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), sintc(p), con, con_lap, eta1, eta2, dfdcon, dummy);
    return launched();
}

extern "C" int amps_sintering_con2_pure(const amps_params *p, const double *dummy, double *dummy_lap, double *con,
                                        const double *eta1, const double *eta2, int step, void *stream)
{
    (void)step;
    if (check_grid(p) || !dummy || !dummy_lap || !con || !eta1 || !eta2) return AMPS_ERR_INVALID;
    sint_con2<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), sintc(p), dummy, dummy_lap, con, eta1, eta2);
    return launched();
}

extern "C" int amps_sintering_phi1_pure(const amps_params *p, const double *eta1, double *eta1_out,
                                        const double *eta2, double *eta1_lap, double *dfdeta1, const double *con,
                                        int step, void *stream)
{
    (void)step;
    if (check_grid(p) || !eta1 || !eta1_out || !eta2 || !eta1_lap || !dfdeta1 || !con || eta1 == eta1_out)
        return AMPS_ERR_INVALID;
    sint_phi<<<grid2(p), dim3(kBX, kBY), 0, S_>>>(geo(p), sintc(p), eta1, eta1_out, eta2, eta1_lap, dfdeta1, con);
    return launched();
}

extern "C" int amps_sintering_phi2_pure(const amps_params *p, const double *eta2, double *eta2_out,
                                        const double *eta1, double *eta2_lap, double *dfdeta2, const double *con,
                                        int step, void *stream)
{
    return amps_sintering_phi1_pure(p, eta2, eta2_out, eta1, eta2_lap, dfdeta2, con, step, stream);
}

extern "C" int amps_get_max_diff1(const amps_params *p, const double *con, double *max_diff_con, void *stream)
{
    if (check_tiles(p) || !con || !max_diff_con) return AMPS_ERR_INVALID;
    max_diff<<<tgrid(p), dim3(16, 16), 0, S_>>>(p->nx, p->nx / p->tile, p->ny / p->tile, p->tile, 1, nullptr, con,
                                                 max_diff_con);
    return launched();
}

extern "C" int amps_get_max_diff2(const amps_params *p, const double *test_data_last, const double *test_data,
                                  double *max_diffs, void *stream)
{
    if (check_tiles(p) || !test_data_last || !test_data || !max_diffs) return AMPS_ERR_INVALID;
    max_diff<<<tgrid(p), dim3(16, 16), 0, S_>>>(p->nx, p->nx / p->tile, p->ny / p->tile, p->tile, 2, test_data_last,
                                                 test_data, max_diffs);
    return launched();
}

extern "C" int amps_get_type(const amps_params *p, const double *max_diff_con, int *type_old, int *type_con,
                             void *stream)
{
    if (check_tiles(p) || !max_diff_con || !type_old || !type_con) return AMPS_ERR_INVALID;
    get_type_k<<<tgrid(p), dim3(16, 16), 0, S_>>>(p->nx / p->tile, p->ny / p->tile, p->thr_hi, max_diff_con,
                                                  type_old, type_con);
    return launched();
}
