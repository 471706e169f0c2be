// compat_half.cu -- the reference's binary16 kernels and their data tools
// under their own names (include/amps_compat.h): the all-half2 ("purelow",
// HALF2) steps of grain growth and the Kobayashi dendrite and the half2
// preparation / gathering tools, as host launch wrappers over caller-owned
// device arrays in the reference's layout -- half2 arrays [ny][nx/2], each
// half2 holding columns 2x (low) and 2x+1 (high) of a row.  One thread per
// half2 pair; each pair's arithmetic is the reference kernel's half2
// expression, term by term and in its order, so the same compiler makes the
// same choices (compiled like the reference, multiply-adds allowed).  The
// half2 constants the reference's drivers pass (TOLOW = __float2half2_rn of
// its compile-time constants) are formed here from an amps_params.  Periodic
// grids only, as the reference's kernels are.
#include "../../include/amps_compat.h"
#include "amps_internal.cuh"

#include <math.h>

namespace {

constexpr int kBX = 32, kBY = 8;

struct GeoH {
    int np, ny;  // pairs per row (nx / 2), rows
};

__device__ __forceinline__ bool pair(const GeoH &g, int &x, int &y)
{
    x = blockIdx.x * kBX + threadIdx.x;
    y = blockIdx.y * kBY + threadIdx.y;
    return x < g.np && y < g.ny;
}

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// the pair (high half of pair l, low half of pair r): the cells one column
// to the left of pair r (l = r - 1) or to the right of pair l (r = l + 1)
__device__ __forceinline__ __half2 shift(__half2 l, __half2 r) { return __halves2half2(__high2half(l), __low2half(r)); }

__half2 h2(double v) { return __float2half2_rn((float)v); }

struct GgH {
    __half2 one, two, eight, dt, mobil, grcoef, dxdy;
};

// graingrowth/function.h:280-308 (HALF2)
__global__ void gg_lowpure(GeoH g, GgH c, const __half2 *a, const __half2 *b, __half2 *lap, __half2 *dfd, __half2 *out)
{
    int x, y;
    if (!pair(g, x, y)) return;
    const int xs1 = wrap(x - 1, g.np), xa1 = wrap(x + 1, g.np), ys1 = wrap(y - 1, g.ny), ya1 = wrap(y + 1, g.ny);
    auto A = [&](int yy, int xx) { return a[(int64_t)yy * g.np + xx]; };
    const int64_t i = (int64_t)y * g.np + x;
    const __half2 l = (shift(A(ys1, xs1), A(ys1, x)) + A(ys1, x) + shift(A(ys1, x), A(ys1, xa1)) +
                       shift(A(y, xs1), A(y, x)) + shift(A(y, x), A(y, xa1)) + shift(A(ya1, xs1), A(ya1, x)) +
                       A(ya1, x) + shift(A(ya1, x), A(ya1, xa1)) - c.eight * A(y, x)) / c.dxdy;
    lap[i] = l;
    const __half2 sum = b[i] * b[i];
    const __half2 e = a[i];
    const __half2 f = c.one * (c.two * c.one * e * sum + (e * e * e) - e);
    dfd[i] = f;
    out[i] = e - c.dt * c.mobil * (f - c.grcoef * l);
}

// graingrowth/tools.h:54-81 -- the initial circle, one half2 pair a thread
// (centre and radius in float, distances in float, as there)
__global__ void gg_prep_half2(GeoH g, float rx, float ry, float r, __half2 *e1, __half2 *e2)
{
    int x, y;
    if (!pair(g, x, y)) return;
    const float d1 = sqrt(pow(2 * x - rx, 2) + pow(y - ry, 2)), d2 = sqrt(pow(2 * x + 1 - rx, 2) + pow(y - ry, 2));
    const float a1 = d1 <= r ? 0.f : 1.f, a2 = d2 <= r ? 0.f : 1.f;
    const int64_t i = (int64_t)y * g.np + x;
    e1[i] = __floats2half2_rn(a1, a2);
    e2[i] = __floats2half2_rn(1.f - a1, 1.f - a2);
}

// graingrowth/tools.h:133-155 and snowflake/tools.h:108-130 (HALF2): half2 pairs to floats
__global__ void purelow_to_float(GeoH g, const __half2 *h, float *f)
{
    int x, y;
    if (!pair(g, x, y)) return;
    const __half2 v = h[(int64_t)y * g.np + x];
    f[(int64_t)y * 2 * g.np + 2 * x] = __low2float(v);
    f[(int64_t)y * 2 * g.np + 2 * x + 1] = __high2float(v);
}

struct KobH {
    __half2 dxdy, theta0, aniso, one, dxm2, dym2, delta, epsb, eight, gama, teq, alpha, pi, zpf, dt, tau, kappa;
};

// snowflake/function.h:607-659 (HALF2): the Laplacians, gradients and the
// anisotropy of one half2 pair
__global__ void kob_low_k1(GeoH g, KobH c, const __half2 *phi, __half2 *phi_lap, const __half2 *tempr,
                           __half2 *tempr_lap, __half2 *phidx, __half2 *phidy, __half2 *eps, __half2 *epsd)
{
    int x, y;
    if (!pair(g, x, y)) return;
    const int xs1 = wrap(x - 1, g.np), xa1 = wrap(x + 1, g.np);
    const int ys1 = wrap(y - 1, g.ny), ya1 = wrap(y + 1, g.ny), ys2 = wrap(y - 2, g.ny), ya2 = wrap(y + 2, g.ny);
    auto P = [&](int yy, int xx) { return phi[(int64_t)yy * g.np + xx]; };
    auto T = [&](int yy, int xx) { return tempr[(int64_t)yy * g.np + xx]; };
    const int64_t i = (int64_t)y * g.np + x;
    const __half2 d = c.dxdy;
    phi_lap[i] = (shift(P(y, xs1), P(y, x)) / d + P(y, xs1) / d + shift(P(y, x), P(y, xa1)) / d + P(y, xa1) / d +
                  P(ys1, x) / d + P(ys2, x) / d + P(ya1, x) / d + P(ya2, x) / d - c.eight * P(y, x) / d);
    tempr_lap[i] = (shift(T(y, xs1), T(y, x)) / d + T(y, xs1) / d + shift(T(y, x), T(y, xa1)) / d + T(y, xa1) / d +
                    T(ys1, x) / d + T(ys2, x) / d + T(ya1, x) / d + T(ya2, x) / d - c.eight * T(y, x) / d);
    const __half2 px = (shift(P(y, x), P(y, xa1)) - shift(P(y, xs1), P(y, x))) / c.dxm2;
    phidx[i] = px;
    const __half2 py = (P(ya1, x) - P(ys1, x)) / c.dym2;
    phidy[i] = py;
    const __half2 theta = __floats2half2_rn(atan2(__low2float(py), __low2float(px)), atan2(__high2float(py), __high2float(px)));
    const __half2 tmp = c.aniso * (theta - c.theta0);
    const __half2 t1 = h2cos(tmp), t2 = h2sin(tmp);
    eps[i] = c.epsb * (c.one + c.delta * t1);
    epsd[i] = -c.epsb * c.aniso * c.delta * t2;
}

// snowflake/function.h:660-700 (HALF2): phi and T of one half2 pair, in place
__global__ void kob_low_k2(GeoH g, KobH c, __half2 *phi, const __half2 *phi_lap, const __half2 *eps,
                           const __half2 *epsd, const __half2 *phidx, const __half2 *phidy, __half2 *tempr,
                           const __half2 *tempr_lap)
{
    int x, y;
    if (!pair(g, x, y)) return;
    const int xs1 = wrap(x - 1, g.np), xa1 = wrap(x + 1, g.np), ys1 = wrap(y - 1, g.ny), ya1 = wrap(y + 1, g.ny);
    auto at = [&](int yy, int xx) { return (int64_t)yy * g.np + xx; };
    const int64_t i = at(y, x);
    const __half2 phi_old = phi[i];
    const __half2 term1 = (eps[at(ya1, x)] * epsd[at(ya1, x)] * phidx[at(ya1, x)] -
                           eps[at(ys1, x)] * epsd[at(ys1, x)] * phidx[at(ys1, x)]) / c.dym2;
    const __half2 term2 = -(shift(eps[i], eps[at(y, xa1)]) * shift(epsd[i], epsd[at(y, xa1)]) *
                                shift(phidy[i], phidy[at(y, xa1)]) -
                            shift(eps[at(y, xs1)], eps[i]) * shift(epsd[at(y, xs1)], epsd[i]) *
                                shift(phidy[at(y, xs1)], phidy[i])) / c.dxm2;
    __half2 tmp = c.gama * (c.teq - tempr[i]);
    tmp = __floats2half2_rn(atan(__low2float(tmp)), atan(__high2float(tmp)));
    const __half2 m = c.alpha / c.pi * tmp;
    const __half2 pn = phi[i] + (c.dt / c.tau) * (term1 + term2 + (eps[i] * eps[i]) * phi_lap[i] +
                                                  phi_old * (c.one - phi_old) * (phi_old - c.zpf + m));
    phi[i] = pn;
    tempr[i] = tempr[i] + c.dt * tempr_lap[i] + c.kappa * (pn - phi_old);
}

// snowflake/tools.h:43-58 (HALF2): the seed disc into phi (every pair
// written: 1 inside, 0 outside), one half2 pair a thread
__global__ void kob_prep_half2(GeoH g, double r2, int off, __half2 *phi)
{
    int x, y;
    if (!pair(g, x, y)) return;
    const int nx = 2 * g.np;
    const float d1 = pow(2 * x - (nx / 2 + off), 2) + pow(y - (g.ny / 2 + off), 2);
    const float d2 = pow(2 * x + 1 - (nx / 2 + off), 2) + pow(y - (g.ny / 2 + off), 2);
    const float p1 = d1 < r2 ? 1.f : 0.f, p2 = d2 < r2 ? 1.f : 0.f;
    phi[(int64_t)y * g.np + x] = __floats2half2_rn(p1, p2);
}

int check_half2(const amps_params *p)
{
    if (!p || p->nx < 4 || p->ny < 5 || p->nx % 2 || p->bc != AMPS_BC_PERIODIC) return AMPS_ERR_INVALID;
    return AMPS_OK;
}

GeoH geoh(const amps_params *p) { return GeoH{p->nx / 2, p->ny}; }
dim3 gridh(const amps_params *p) { return dim3((p->nx / 2 + kBX - 1) / kBX, (p->ny + kBY - 1) / kBY); }

KobH kobh(const amps_params *p)
{
    return KobH{h2(p->dx * p->dy), h2(p->theta0), h2(p->aniso), h2(1.0), h2(p->dx * 2), h2(p->dy * 2), h2(p->delta),
                h2(p->epsb), h2(8.0), h2(p->gama), h2(p->teq), h2(p->alpha), h2(p->pi), h2(0.5), h2(p->dt),
                h2(p->tau), h2(p->kappa)};
}

int launched() { return cudaGetLastError() == cudaSuccess ? AMPS_OK : AMPS_ERR_CUDA; }

}  // namespace

#define S_ (cudaStream_t) stream

extern "C" int amps_graingrowth_kernel1_lowpure(const amps_params *p, const void *etaa, const void *etab,
                                                void *etaa_lap, void *dfdetaa, void *etaa_out, void *stream)
{
    if (check_half2(p) || !etaa || !etab || !etaa_lap || !dfdetaa || !etaa_out || etaa == etaa_out)
        return AMPS_ERR_INVALID;
    const GgH c{h2(1.0), h2(2.0), h2(8.0), h2(p->dt), h2(p->mobil), h2(p->grcoef), h2(p->dx * p->dy)};
    gg_lowpure<<<gridh(p), dim3(kBX, kBY), 0, S_>>>(geoh(p), c, (const __half2 *)etaa, (const __half2 *)etab,
                                                    (__half2 *)etaa_lap, (__half2 *)dfdetaa, (__half2 *)etaa_out);
    return launched();
}

extern "C" int amps_graingrowth_dataprepare_half2(const amps_params *p, void *eta1, void *eta2, void *stream)
{
    if (check_half2(p) || !eta1 || !eta2) return AMPS_ERR_INVALID;
    gg_prep_half2<<<gridh(p), dim3(kBX, kBY), 0, S_>>>(geoh(p), (float)(p->nx / 2), (float)(p->ny / 2),
                                                       (float)p->init_r, (__half2 *)eta1, (__half2 *)eta2);
    return launched();
}

extern "C" int amps_purelow2high_aftercomputing(const amps_params *p, const void *hdata, float *fdata, void *stream)
{
    if (check_half2(p) || !hdata || !fdata) return AMPS_ERR_INVALID;
    purelow_to_float<<<gridh(p), dim3(kBX, kBY), 0, S_>>>(geoh(p), (const __half2 *)hdata, fdata);
    return launched();
}

extern "C" int amps_snowflake_kernel1_purelow(const amps_params *p, const void *phi, void *phi_lap, const void *tempr,
                                              void *tempr_lap, void *phidx, void *phidy, void *epsilon,
                                              void *epsilon_deri, void *stream)
{
    if (check_half2(p) || !phi || !phi_lap || !tempr || !tempr_lap || !phidx || !phidy || !epsilon || !epsilon_deri)
        return AMPS_ERR_INVALID;
    kob_low_k1<<<gridh(p), dim3(kBX, kBY), 0, S_>>>(geoh(p), kobh(p), (const __half2 *)phi, (__half2 *)phi_lap,
                                                    (const __half2 *)tempr, (__half2 *)tempr_lap, (__half2 *)phidx,
                                                    (__half2 *)phidy, (__half2 *)epsilon, (__half2 *)epsilon_deri);
    return launched();
}

extern "C" int amps_snowflake_kernel2_purelow(const amps_params *p, void *phi, const void *phi_lap,
                                              const void *epsilon, const void *epsilon_deri, const void *phidx,
                                              const void *phidy, void *tempr, const void *tempr_lap, void *stream)
{
    if (check_half2(p) || !phi || !phi_lap || !tempr || !tempr_lap || !phidx || !phidy || !epsilon || !epsilon_deri)
        return AMPS_ERR_INVALID;
    kob_low_k2<<<gridh(p), dim3(kBX, kBY), 0, S_>>>(geoh(p), kobh(p), (__half2 *)phi, (const __half2 *)phi_lap,
                                                    (const __half2 *)epsilon, (const __half2 *)epsilon_deri,
                                                    (const __half2 *)phidx, (const __half2 *)phidy, (__half2 *)tempr,
                                                    (const __half2 *)tempr_lap);
    return launched();
}

extern "C" int amps_snowflake_dataprepare_half2(const amps_params *p, void *phi, void *stream)
{
    if (check_half2(p) || !phi) return AMPS_ERR_INVALID;
    kob_prep_half2<<<gridh(p), dim3(kBX, kBY), 0, S_>>>(geoh(p), p->init_r2, p->init_offset, (__half2 *)phi);
    return launched();
}
