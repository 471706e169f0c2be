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

// ---- the adaptive (AMSTENCIL) grain-growth step, graingrowth/function.h:33-277 ----
// Dual storage as the reference keeps it: FP64 arrays [ny][nx] (every tile's
// cells where the tile is high, type 2; a low tile's edge cells, converted
// each step, and all its cells after a period's last step) and half2 arrays
// [ny][nx/2] (low tiles, type 1).  One CTA per tile, one thread per half2
// pair: (T/2) x T threads.  A low tile's thread computes its pair in half2
// from the half2 array, taking the cells of a high neighbour tile from the
// FP64 array (graingrowth/function.h:81-170); a high tile's thread computes
// its two cells in FP64 from the FP64 array (:232-271).
struct GeoM {
    int nx, ny, T, ntx, nty;
};

__device__ __forceinline__ void tile_of(const GeoM &g, int &tx, int &ty)
{
    tx = (int)blockIdx.x % g.ntx;
    ty = (int)blockIdx.x / g.ntx;
}

struct MixPtrs {
    const double *a;   // etaa
    double *last;      // etaa_last (Monitor2 snapshot) or null
    const double *b;   // etab
    double *lap, *dfd, *out;
    const __half2 *ha, *hb;
    __half2 *hlap, *hdfd, *hout;
    const int *type;   // type_curr [nty][ntx]
};

// low half := v (float of an FP64 cell), high half kept
__device__ __forceinline__ __half2 set_lo(__half2 p, double v) { return __halves2half2(__float2half(v), __high2half(p)); }
// high half := v, low half kept
__device__ __forceinline__ __half2 set_hi(__half2 p, double v) { return __halves2half2(__low2half(p), __float2half(v)); }

__global__ void gg_mix_k(GeoM g, GgH c, double dxdy, double dtm, double grcoef, MixPtrs m, int step, int etai,
                         int cadence, bool snap)
{
    int tx, ty;
    tile_of(g, tx, ty);
    const int th = g.T / 2, np = g.nx / 2;
    const int xo = threadIdx.x, yo = threadIdx.y;
    const int y = ty * g.T + yo;
    const int ys1 = y > 0 ? y - 1 : g.ny - 1, ya1 = y < g.ny - 1 ? y + 1 : 0;
    const int tys1 = ty == 0 ? g.nty - 1 : ty - 1, tya1 = ty == g.nty - 1 ? 0 : ty + 1;
    const int txs1 = tx == 0 ? g.ntx - 1 : tx - 1, txa1 = tx == g.ntx - 1 ? 0 : tx + 1;
    auto type = [&](int yy, int xx) { return m.type[yy * g.ntx + xx]; };
    const int own = type(ty, tx);
    const int64_t row = (int64_t)y * g.nx;
    const int c0 = tx * g.T + xo;  // this thread's cell; a high tile's thread also has c0 + th
    // Monitor2 (End2end): the snapshot at the period's first step, of every
    // cell of a high tile and of the left half of a low tile (whose second
    // block returned before the snapshot there)
    if (snap && step % cadence == 0 && etai == 2) {
        m.last[row + c0] = m.a[row + c0];
        if (own != 1) m.last[row + c0 + th] = m.a[row + c0 + th];
    }
    if (own == 1) {
        const int x = tx * th + xo;  // pair index
        const int xs1 = x > 0 ? x - 1 : np - 1, xa1 = x < np - 1 ? x + 1 : 0;
        auto H = [&](int yy, int xx) { return m.ha[(int64_t)yy * np + xx]; };
        auto F = [&](int yy, int cx) { return m.a[(int64_t)yy * g.nx + cx]; };
        // the eight neighbour pairs: W (cells 2x-1, 2x), C (2x, 2x+1), E (2x+1, 2x+2) of rows ys1 / ya1, W / E of y
        __half2 w_u = shift(H(ys1, xs1), H(ys1, x)), c_u = H(ys1, x), e_u = shift(H(ys1, x), H(ys1, xa1));
        __half2 w_m = shift(H(y, xs1), H(y, x)), e_m = shift(H(y, x), H(y, xa1));
        __half2 w_d = shift(H(ya1, xs1), H(ya1, x)), c_d = H(ya1, x), e_d = shift(H(ya1, x), H(ya1, xa1));
        // cells of high neighbour tiles come from the FP64 array (function.h:91-170)
        const bool lef = xo == 0, rig = xo == th - 1, top = yo == 0, bot = yo == g.T - 1;
        const int xl = 2 * xs1 + 1, xc = 2 * x, xr = 2 * xa1;  // columns 2x-1, 2x, 2x+2
        if (lef && top) {
            if (type(ty, txs1) == 2) {
                w_m = set_lo(w_m, F(y, xl));
                w_d = set_lo(w_d, F(ya1, xl));
            }
            if (type(tys1, tx) == 2) {
                w_u = set_hi(w_u, F(ys1, xc));
                c_u = __floats2half2_rn(F(ys1, xc), F(ys1, xc + 1));
                e_u = __floats2half2_rn(F(ys1, xc + 1), F(ys1, xr));
            }
            if (type(tys1, txs1) == 2) w_u = set_lo(w_u, F(ys1, xl));
        } else if (lef && bot) {
            if (type(ty, txs1) == 2) {
                w_m = set_lo(w_m, F(y, xl));
                w_u = set_lo(w_u, F(ys1, xl));
            }
            if (type(tya1, tx) == 2) {
                w_d = set_hi(w_d, F(ya1, xc));
                c_d = __floats2half2_rn(F(ya1, xc), F(ya1, xc + 1));
                e_d = __floats2half2_rn(F(ya1, xc + 1), F(ya1, xr));
            }
            if (type(tya1, txs1) == 2) w_d = set_lo(w_d, F(ya1, xl));
        } else if (rig && top) {
            if (type(ty, txa1) == 2) {
                e_m = set_hi(e_m, F(y, xr));
                e_d = set_hi(e_d, F(ya1, xr));
            }
            if (type(tys1, tx) == 2) {
                w_u = __floats2half2_rn(F(ys1, xl), F(ys1, xc));
                c_u = __floats2half2_rn(F(ys1, xc), F(ys1, xc + 1));
                e_u = set_lo(e_u, F(ys1, xc + 1));
            }
            if (type(tys1, txa1) == 2) e_u = set_hi(e_u, F(ys1, xr));
        } else if (rig && bot) {
            if (type(ty, txa1) == 2) {
                e_u = set_hi(e_u, F(ys1, xr));
                e_m = set_hi(e_m, F(y, xr));
            }
            if (type(tya1, tx) == 2) {
                w_d = __floats2half2_rn(F(ya1, xl), F(ya1, xc));
                c_d = __floats2half2_rn(F(ya1, xc), F(ya1, xc + 1));
                e_d = set_lo(e_d, F(ya1, xc + 1));
            }
            if (type(tya1, txa1) == 2) e_d = set_hi(e_d, F(ya1, xr));
        } else if (lef && type(ty, txs1) == 2) {
            w_u = set_lo(w_u, F(ys1, xl));
            w_m = set_lo(w_m, F(y, xl));
            w_d = set_lo(w_d, F(ya1, xl));
        } else if (rig && type(ty, txa1) == 2) {
            e_u = set_hi(e_u, F(ys1, xr));
            e_m = set_hi(e_m, F(y, xr));
            e_d = set_hi(e_d, F(ya1, xr));
        } else if (top && type(tys1, tx) == 2) {
            w_u = __floats2half2_rn(F(ys1, xl), F(ys1, xc));
            c_u = __floats2half2_rn(F(ys1, xc), F(ys1, xc + 1));
            e_u = __floats2half2_rn(F(ys1, xc + 1), F(ys1, xr));
        } else if (bot && type(tya1, tx) == 2) {
            w_d = __floats2half2_rn(F(ya1, xl), F(ya1, xc));
            c_d = __floats2half2_rn(F(ya1, xc), F(ya1, xc + 1));
            e_d = __floats2half2_rn(F(ya1, xc + 1), F(ya1, xr));
        }
        // function.h:163-166, term by term
        const int64_t i = (int64_t)y * np + x;
        const __half2 e = m.ha[i];
        const __half2 l = (w_u + c_u + e_u + w_m + e_m + w_d + c_d + e_d - c.eight * e) / c.dxdy;
        m.hlap[i] = l;
        const __half2 sum = m.hb[i] * m.hb[i];
        const __half2 f = c.one * (c.two * c.one * e * sum + (e * e * e) - e);
        m.hdfd[i] = f;
        const __half2 o = e - c.dt * c.mobil * (f - c.grcoef * l);
        m.hout[i] = o;
        // function.h:168-176: the tile's edge cells into the FP64 output
        // (all its cells at a period's last step)
        if (yo == 0 || yo == g.T - 1 || (step + 1) % cadence == 0) {
            m.out[row + xc] = __low2float(o);
            m.out[row + xc + 1] = __high2float(o);
        } else if (lef) {
            m.out[row + xc] = __low2float(o);
        } else if (rig) {
            m.out[row + xc + 1] = __high2float(o);
        }
        return;
    }
    // a high tile: two cells, FP64, function.h:232-271
    for (int k = 0; k < 2; ++k) {
        const int x = c0 + k * th;
        const int xs1 = x > 0 ? x - 1 : g.nx - 1, xa1 = x < g.nx - 1 ? x + 1 : 0;
        auto A = [&](int yy, int xx) { return m.a[(int64_t)yy * g.nx + xx]; };
        const int64_t i = row + x;
        const double lap = (A(ys1, xs1) + A(ys1, x) + A(ys1, xa1) + A(y, xs1) + A(y, xa1) + A(ya1, xs1) + A(ya1, x) +
                            A(ya1, xa1) - 8.0 * A(y, x)) /
                           dxdy;
        m.lap[i] = lap;
        const double sum = pow(m.b[i], 2);
        const double e = m.a[i];
        const double f = 1.0 * (2.0 * 1.0 * e * sum + pow(e, 3) - e);
        m.dfd[i] = f;
        m.out[i] = e - dtm * (f - grcoef * lap);
    }
}

// ---- the adaptive (AMSTENCIL) Kobayashi step, snowflake/function.h:63-604 ----
// The same dual storage and launch shape as gg_mix_k: phi, tempr and the
// step's intermediates (phi_lap, tempr_lap, phidx, phidy, epsilon,
// epsilon_deri) each as an FP64 array and a half2 array.  The stencils reach
// two cells (the reference's cross Laplacian): a low tile takes the cells of a
// high neighbour tile (left, right, up, down) from the FP64 arrays, and its
// edge band is converted into them after each kernel.
struct KobMixPtrs {
    double *phi, *last, *phi_lap, *eps, *epsd, *phidx, *phidy, *tempr, *tempr_lap;
    __half2 *hphi, *hphi_lap, *htempr, *htempr_lap, *hphidx, *hphidy, *heps, *hepsd;
    const int *type;
};

// the FP64 constants of a high tile as the reference's compile-time
// expressions fold them: dx*dy, 2*dx, 2*dy, -epsilonb*aniso*delta,
// alpha/pi, dtime/tau
struct KobD {
    double dxdy, dx2, dy2, epsb, delta, aniso, theta0, nead, apk, gama, teq, dtt, dt, kappa;
};

struct TileAt {
    int tx, ty, txs1, txa1, tys1, tya1, xo, yo, th, y, c0;
};
__device__ __forceinline__ TileAt tile_at(const GeoM &g)
{
    TileAt t;
    tile_of(g, t.tx, t.ty);
    t.txs1 = t.tx == 0 ? g.ntx - 1 : t.tx - 1;
    t.txa1 = t.tx == g.ntx - 1 ? 0 : t.tx + 1;
    t.tys1 = t.ty == 0 ? g.nty - 1 : t.ty - 1;
    t.tya1 = t.ty == g.nty - 1 ? 0 : t.ty + 1;
    t.xo = threadIdx.x;
    t.yo = threadIdx.y;
    t.th = g.T / 2;
    t.y = t.ty * g.T + t.yo;
    t.c0 = t.tx * g.T + t.xo;
    return t;
}

__device__ __forceinline__ int wrapn(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// snowflake/function.h:63-375: Laplacians, gradients and the anisotropy
__global__ void kob_mix_k1(GeoM g, KobH c, KobD d, KobMixPtrs m, int step, int cadence, bool snap)
{
    const TileAt t = tile_at(g);
    auto type = [&](int yy, int xx) { return m.type[yy * g.ntx + xx]; };
    const int own = type(t.ty, t.tx);
    const int y = t.y, nx = g.nx, np = g.nx / 2;
    const int ys1 = wrapn(y - 1, g.ny), ya1 = wrapn(y + 1, g.ny), ys2 = wrapn(y - 2, g.ny), ya2 = wrapn(y + 2, g.ny);
    const int64_t row = (int64_t)y * nx;
    // Monitor2: the snapshot at the period's first step (a low tile's left half only)
    if (snap && step % cadence == 0) {
        m.last[row + t.c0] = m.phi[row + t.c0];
        if (own != 1) m.last[row + t.c0 + t.th] = m.phi[row + t.c0 + t.th];
    }
    if (own == 1) {
        const int x = t.tx * t.th + t.xo;
        const int xs1 = x > 0 ? x - 1 : np - 1, xa1 = x < np - 1 ? x + 1 : 0;
        auto HP = [&](int yy, int xx) { return m.hphi[(int64_t)yy * np + xx]; };
        auto HT = [&](int yy, int xx) { return m.htempr[(int64_t)yy * np + xx]; };
        auto FP = [&](int yy, int cx) { return m.phi[(int64_t)yy * nx + cx]; };
        auto FT = [&](int yy, int cx) { return m.tempr[(int64_t)yy * nx + cx]; };
        __half2 p_xs1 = shift(HP(y, xs1), HP(y, x)), p_xs2 = HP(y, xs1), p_xa1 = shift(HP(y, x), HP(y, xa1)),
                p_xa2 = HP(y, xa1), p_ys1 = HP(ys1, x), p_ys2 = HP(ys2, x), p_ya1 = HP(ya1, x), p_ya2 = HP(ya2, x);
        __half2 t_xs1 = shift(HT(y, xs1), HT(y, x)), t_xs2 = HT(y, xs1), t_xa1 = shift(HT(y, x), HT(y, xa1)),
                t_xa2 = HT(y, xa1), t_ys1 = HT(ys1, x), t_ys2 = HT(ys2, x), t_ya1 = HT(ya1, x), t_ya2 = HT(ya2, x);
        const int xl = 2 * xs1, xr = 2 * xa1;
        // function.h:137-158, the x chain
        if (t.xo == 0 && type(t.ty, t.txs1) == 2) {
            p_xs1 = set_lo(p_xs1, FP(y, xl + 1));
            t_xs1 = set_lo(t_xs1, FT(y, xl + 1));
            p_xs2 = __halves2half2(__float2half(FP(y, xl)), __float2half(FP(y, xl + 1)));
            t_xs2 = __halves2half2(__float2half(FT(y, xl)), __float2half(FT(y, xl + 1)));
        } else if (t.xo == 1 && type(t.ty, t.txs1) == 2) {
            p_xs2 = __halves2half2(__float2half(FP(y, xl)), __float2half(FP(y, xl + 1)));
            t_xs2 = __halves2half2(__float2half(FT(y, xl)), __float2half(FT(y, xl + 1)));
        } else if (t.xo == t.th - 1 && type(t.ty, t.txa1) == 2) {
            p_xa1 = set_hi(p_xa1, FP(y, xr));
            t_xa1 = set_hi(t_xa1, FT(y, xr));
            p_xa2 = __halves2half2(__float2half(FP(y, xr)), __float2half(FP(y, xr + 1)));
            t_xa2 = __halves2half2(__float2half(FT(y, xr)), __float2half(FT(y, xr + 1)));
        } else if (t.xo == t.th - 2 && type(t.ty, t.txa1) == 2) {
            p_xa2 = __halves2half2(__float2half(FP(y, xr)), __float2half(FP(y, xr + 1)));
            t_xa2 = __halves2half2(__float2half(FT(y, xr)), __float2half(FT(y, xr + 1)));
        }
        // function.h:160-180, the y chain
        const int xc = 2 * x;
        if (t.yo == 0 && type(t.tys1, t.tx) == 2) {
            p_ys1 = __floats2half2_rn(FP(ys1, xc), FP(ys1, xc + 1));
            t_ys1 = __floats2half2_rn(FT(ys1, xc), FT(ys1, xc + 1));
            p_ys2 = __floats2half2_rn(FP(ys2, xc), FP(ys2, xc + 1));
            t_ys2 = __floats2half2_rn(FT(ys2, xc), FT(ys2, xc + 1));
        } else if (t.yo == 1 && type(t.tys1, t.tx) == 2) {
            p_ys2 = __floats2half2_rn(FP(ys2, xc), FP(ys2, xc + 1));
            t_ys2 = __floats2half2_rn(FT(ys2, xc), FT(ys2, xc + 1));
        } else if (t.yo == g.T - 1 && type(t.tya1, t.tx) == 2) {
            p_ya1 = __floats2half2_rn(FP(ya1, xc), FP(ya1, xc + 1));
            t_ya1 = __floats2half2_rn(FT(ya1, xc), FT(ya1, xc + 1));
            p_ya2 = __floats2half2_rn(FP(ya2, xc), FP(ya2, xc + 1));
            t_ya2 = __floats2half2_rn(FT(ya2, xc), FT(ya2, xc + 1));
        } else if (t.yo == g.T - 2 && type(t.tya1, t.tx) == 2) {
            p_ya2 = __floats2half2_rn(FP(ya2, xc), FP(ya2, xc + 1));
            t_ya2 = __floats2half2_rn(FT(ya2, xc), FT(ya2, xc + 1));
        }
        // function.h:204-220, term by term
        const int64_t i = (int64_t)y * np + x;
        const __half2 dd = c.dxdy;
        m.hphi_lap[i] = p_xs1 / dd + p_xs2 / dd + p_xa1 / dd + p_xa2 / dd + p_ys1 / dd + p_ys2 / dd + p_ya1 / dd +
                        p_ya2 / dd - c.eight * HP(y, x) / dd;
        m.htempr_lap[i] = t_xs1 / dd + t_xs2 / dd + t_xa1 / dd + t_xa2 / dd + t_ys1 / dd + t_ys2 / dd + t_ya1 / dd +
                          t_ya2 / dd - c.eight * HT(y, x) / dd;
        const __half2 px = (p_xa1 - p_xs1) / c.dxm2;
        m.hphidx[i] = px;
        const __half2 py = (p_ya1 - p_ys1) / c.dym2;
        m.hphidy[i] = py;
        const __half2 theta =
            __floats2half2_rn(atan2(__low2float(py), __low2float(px)), atan2(__high2float(py), __high2float(px)));
        const __half2 tmp = c.aniso * (theta - c.theta0);
        const __half2 t1 = h2cos(tmp), t2 = h2sin(tmp);
        const __half2 e = c.epsb * (c.one + c.delta * t1);
        m.heps[i] = e;
        const __half2 ed = -c.epsb * c.aniso * c.delta * t2;
        m.hepsd[i] = ed;
        // function.h:221-245: the tile's edge cells into the FP64 arrays
        if (t.yo == 0 || t.yo == g.T - 1) {
            m.phidx[row + xc] = __low2float(px);
            m.phidx[row + xc + 1] = __high2float(px);
            m.phidy[row + xc] = __low2float(py);
            m.phidy[row + xc + 1] = __high2float(py);
            m.eps[row + xc] = __low2float(e);
            m.eps[row + xc + 1] = __high2float(e);
            m.epsd[row + xc] = __low2float(ed);
            m.epsd[row + xc + 1] = __high2float(ed);
        } else if (t.xo == 0) {
            m.phidx[row + xc] = __low2float(px);
            m.phidy[row + xc] = __low2float(py);
            m.eps[row + xc] = __low2float(e);
            m.epsd[row + xc] = __low2float(ed);
        } else if (t.xo == t.th - 1) {
            m.phidx[row + xc + 1] = __high2float(px);
            m.phidy[row + xc + 1] = __high2float(py);
            m.eps[row + xc + 1] = __high2float(e);
            m.epsd[row + xc + 1] = __high2float(ed);
        }
        return;
    }
    // a high tile: two cells in FP64, function.h:266-352
    for (int k = 0; k < 2; ++k) {
        const int x = t.c0 + k * t.th;
        const int xs1 = x > 0 ? x - 1 : nx - 1, xa1 = x < nx - 1 ? x + 1 : 0;
        const int xs2 = x - 2 < 0 ? x - 2 + nx : x - 2, xa2 = x + 2 > nx - 1 ? x + 2 - nx : x + 2;
        auto P = [&](int yy, int xx) { return m.phi[(int64_t)yy * nx + xx]; };
        auto T = [&](int yy, int xx) { return m.tempr[(int64_t)yy * nx + xx]; };
        const int64_t i = row + x;
        m.phi_lap[i] = P(y, xs1) / d.dxdy + P(y, xs2) / d.dxdy + P(y, xa1) / d.dxdy + P(y, xa2) / d.dxdy +
                       P(ys1, x) / d.dxdy + P(ys2, x) / d.dxdy + P(ya1, x) / d.dxdy + P(ya2, x) / d.dxdy -
                       8.0 * P(y, x) / d.dxdy;
        m.tempr_lap[i] = T(y, xs1) / d.dxdy + T(y, xs2) / d.dxdy + T(y, xa1) / d.dxdy + T(y, xa2) / d.dxdy +
                         T(ys1, x) / d.dxdy + T(ys2, x) / d.dxdy + T(ya1, x) / d.dxdy + T(ya2, x) / d.dxdy -
                         8.0 * T(y, x) / d.dxdy;
        const double px = (P(y, xa1) - P(y, xs1)) / d.dx2;
        m.phidx[i] = px;
        const double py = (P(ya1, x) - P(ys1, x)) / d.dy2;
        m.phidy[i] = py;
        const double theta = atan2(py, px);
        m.eps[i] = d.epsb * (1.0 + d.delta * cos(d.aniso * (theta - d.theta0)));
        m.epsd[i] = d.nead * sin(d.aniso * (theta - d.theta0));
    }
}

// snowflake/function.h:376-604: phi and tempr advanced in place
__global__ void kob_mix_k2(GeoM g, KobH c, KobD d, KobMixPtrs m, int step, int cadence)
{
    const TileAt t = tile_at(g);
    auto type = [&](int yy, int xx) { return m.type[yy * g.ntx + xx]; };
    const int own = type(t.ty, t.tx);
    const int y = t.y, nx = g.nx, np = g.nx / 2;
    const int ys1 = wrapn(y - 1, g.ny), ya1 = wrapn(y + 1, g.ny);
    const int64_t row = (int64_t)y * nx;
    if (own == 1) {
        const int x = t.tx * t.th + t.xo;
        const int xs1 = x > 0 ? x - 1 : np - 1, xa1 = x < np - 1 ? x + 1 : 0;
        auto at = [&](int yy, int xx) { return (int64_t)yy * np + xx; };
        auto F = [&](const double *a, int yy, int cx) { return a[(int64_t)yy * nx + cx]; };
        const int64_t i = at(y, x);
        const int xc = 2 * x;
        const __half2 phi_old = m.hphi[i];
        __half2 pdx_ya1, e_ya1, ed_ya1, pdx_ys1, e_ys1, ed_ys1, e_xs1, ed_xs1, pdy_xs1, e_xa1, ed_xa1, pdy_xa1;
        // function.h:429-471: neighbours of a high tile from the FP64 arrays
        if (t.yo < g.T - 1 || type(t.tya1, t.tx) == 1) {
            pdx_ya1 = m.hphidx[at(ya1, x)];
            e_ya1 = m.heps[at(ya1, x)];
            ed_ya1 = m.hepsd[at(ya1, x)];
        } else {
            pdx_ya1 = __floats2half2_rn(F(m.phidx, ya1, xc), F(m.phidx, ya1, xc + 1));
            e_ya1 = __floats2half2_rn(F(m.eps, ya1, xc), F(m.eps, ya1, xc + 1));
            ed_ya1 = __floats2half2_rn(F(m.epsd, ya1, xc), F(m.epsd, ya1, xc + 1));
        }
        if (t.yo > 0 || type(t.tys1, t.tx) == 1) {
            pdx_ys1 = m.hphidx[at(ys1, x)];
            ed_ys1 = m.hepsd[at(ys1, x)];
            e_ys1 = m.heps[at(ys1, x)];
        } else {
            pdx_ys1 = __floats2half2_rn(F(m.phidx, ys1, xc), F(m.phidx, ys1, xc + 1));
            ed_ys1 = __floats2half2_rn(F(m.epsd, ys1, xc), F(m.epsd, ys1, xc + 1));
            e_ys1 = __floats2half2_rn(F(m.eps, ys1, xc), F(m.eps, ys1, xc + 1));
        }
        if (t.xo > 0 || type(t.ty, t.txs1) == 1) {
            e_xs1 = shift(m.heps[at(y, xs1)], m.heps[i]);
            ed_xs1 = shift(m.hepsd[at(y, xs1)], m.hepsd[i]);
            pdy_xs1 = shift(m.hphidy[at(y, xs1)], m.hphidy[i]);
        } else {
            e_xs1 = __halves2half2(__float2half(F(m.eps, y, 2 * xs1 + 1)), __low2half(m.heps[i]));
            ed_xs1 = __halves2half2(__float2half(F(m.epsd, y, 2 * xs1 + 1)), __low2half(m.hepsd[i]));
            pdy_xs1 = __halves2half2(__float2half(F(m.phidy, y, 2 * xs1 + 1)), __low2half(m.hphidy[i]));
        }
        if (t.xo < t.th - 1 || type(t.ty, t.txa1) == 1) {
            e_xa1 = shift(m.heps[i], m.heps[at(y, xa1)]);
            ed_xa1 = shift(m.hepsd[i], m.hepsd[at(y, xa1)]);
            pdy_xa1 = shift(m.hphidy[i], m.hphidy[at(y, xa1)]);
        } else {
            e_xa1 = __halves2half2(__high2half(m.heps[i]), __float2half(F(m.eps, y, 2 * xa1)));
            ed_xa1 = __halves2half2(__high2half(m.hepsd[i]), __float2half(F(m.epsd, y, 2 * xa1)));
            pdy_xa1 = __halves2half2(__high2half(m.hphidy[i]), __float2half(F(m.phidy, y, 2 * xa1)));
        }
        // function.h:478-489, term by term
        const __half2 term1 = (e_ya1 * ed_ya1 * pdx_ya1 - e_ys1 * ed_ys1 * pdx_ys1) / c.dym2;
        const __half2 term2 = -(e_xa1 * ed_xa1 * pdy_xa1 - e_xs1 * ed_xs1 * pdy_xs1) / c.dxm2;
        __half2 tmp = c.gama * (c.teq - m.htempr[i]);
        tmp = __floats2half2_rn(atan(__low2float(tmp)), atan(__high2float(tmp)));
        const __half2 mm = c.alpha / c.pi * tmp;
        const __half2 pn = m.hphi[i] + (c.dt / c.tau) * (term1 + term2 + (m.heps[i] * m.heps[i]) * m.hphi_lap[i] +
                                                          phi_old * (c.one - phi_old) * (phi_old - c.zpf + mm));
        m.hphi[i] = pn;
        const __half2 tn = m.htempr[i] + c.dt * m.htempr_lap[i] + c.kappa * (pn - phi_old);
        m.htempr[i] = tn;
        // function.h:490-499: the two-cell edge band (every cell at a period's last step)
        if (t.yo < 2 || t.yo + 2 > g.T - 1 || t.xo == 0 || t.xo == t.th - 1 || (step + 1) % cadence == 0) {
            m.phi[row + xc] = __low2float(pn);
            m.phi[row + xc + 1] = __high2float(pn);
            m.tempr[row + xc] = __low2float(tn);
            m.tempr[row + xc + 1] = __high2float(tn);
        }
        return;
    }
    // a high tile: two cells in FP64, function.h:511-600
    for (int k = 0; k < 2; ++k) {
        const int x = t.c0 + k * t.th;
        const int xs1 = x > 0 ? x - 1 : nx - 1, xa1 = x < nx - 1 ? x + 1 : 0;
        auto A = [&](const double *a, int yy, int xx) { return a[(int64_t)yy * nx + xx]; };
        const int64_t i = row + x;
        const double phi_old = m.phi[i];
        const double term1 = (A(m.eps, ya1, x) * A(m.epsd, ya1, x) * A(m.phidx, ya1, x) -
                              A(m.eps, ys1, x) * A(m.epsd, ys1, x) * A(m.phidx, ys1, x)) /
                             d.dy2;
        const double term2 = -(A(m.eps, y, xa1) * A(m.epsd, y, xa1) * A(m.phidy, y, xa1) -
                               A(m.eps, y, xs1) * A(m.epsd, y, xs1) * A(m.phidy, y, xs1)) /
                             d.dx2;
        const double mm = d.apk * atan(d.gama * (d.teq - m.tempr[i]));
        m.phi[i] = m.phi[i] + d.dtt * (term1 + term2 + pow(m.eps[i], 2) * m.phi_lap[i] +
                                       phi_old * (1.0 - phi_old) * (phi_old - 0.5 + mm));
        m.tempr[i] = m.tempr[i] + d.dt * m.tempr_lap[i] + d.kappa * (m.phi[i] - phi_old);
    }
}

// snowflake/function.h:715-759: kernel1_mix's conversion as its own launch
__global__ void kob_conv1(GeoM g, KobMixPtrs m)
{
    const TileAt t = tile_at(g);
    if (m.type[t.ty * g.ntx + t.tx] != 1) return;
    const int64_t i = (int64_t)t.y * (g.nx / 2) + t.tx * t.th + t.xo;
    const int64_t c = (int64_t)t.y * g.nx + 2 * (t.tx * t.th + t.xo);
    const __half2 px = m.hphidx[i], py = m.hphidy[i], e = m.heps[i], ed = m.hepsd[i];
    if (t.yo == 0 || t.yo == g.T - 1) {
        m.phidx[c] = __low2float(px);
        m.phidx[c + 1] = __high2float(px);
        m.phidy[c] = __low2float(py);
        m.phidy[c + 1] = __high2float(py);
        m.eps[c] = __low2float(e);
        m.eps[c + 1] = __high2float(e);
        m.epsd[c] = __low2float(ed);
        m.epsd[c + 1] = __high2float(ed);
    } else if (t.xo == 0) {
        m.phidx[c] = __low2float(px);
        m.phidy[c] = __low2float(py);
        m.eps[c] = __low2float(e);
        m.epsd[c] = __low2float(ed);
    } else if (t.xo == t.th - 1) {
        m.phidx[c + 1] = __high2float(px);
        m.phidy[c + 1] = __high2float(py);
        m.eps[c + 1] = __high2float(e);
        m.epsd[c + 1] = __high2float(ed);
    }
}

// snowflake/function.h:760-790: mix_kernel2's conversion as its own launch
__global__ void kob_conv2(GeoM g, KobMixPtrs m, int step, int cadence)
{
    const TileAt t = tile_at(g);
    if (m.type[t.ty * g.ntx + t.tx] != 1) return;
    if (!(t.yo < 2 || t.yo + 2 > g.T - 1 || t.xo == 0 || t.xo == t.th - 1 || (step + 1) % cadence == 0)) return;
    const int64_t i = (int64_t)t.y * (g.nx / 2) + t.tx * t.th + t.xo;
    const int64_t c = (int64_t)t.y * g.nx + 2 * (t.tx * t.th + t.xo);
    m.phi[c] = __low2float(m.hphi[i]);
    m.phi[c + 1] = __high2float(m.hphi[i]);
    m.tempr[c] = __low2float(m.htempr[i]);
    m.tempr[c + 1] = __high2float(m.htempr[i]);
}

// ---- the adaptive (AMSTENCIL) sintering step, sintering/function.h:161-774 ----
// Sintering packs a tile's two halves into its half2 words: pair xo of tile
// tx holds cells x0 + xo (low) and x0 + xo + T/2 (high), x0 = tx * T.  A low
// tile reads its x neighbours from the half2 arrays only (high tiles keep
// their first and last columns there, written after each update) and its y
// neighbours from the FP64 arrays where the tile above / below is high.
struct SintH {
    __half2 cf, dxdy, zpfive, one, two, four, six, ten, twelve, fifteen, thirtytwo, coefm, coefk, coefl, dvol, dvap,
        dsur, dgrb, dt, hi, lo;
};
// the FP64 constants the reference's compile-time expressions fold:
// 0.5 * coefm, 0.5 * coefk, dtime * coefl
struct SintD {
    double dxdy, hcoefm, hcoefk, dtcoefl, dt, dvol, dvap, dsur, dgrb;
};

// the x and y neighbour pairs of a low tile's pair (sintering/function.h:213-216)
struct NbH {
    __half2 xs1, xa1, ys1, ya1;
};
__device__ __forceinline__ NbH nb_low(const GeoM &g, const TileAt &t, const int *type, const __half2 *h,
                                      const double *f)
{
    const int np = g.nx / 2, th = t.th;
    const int x = t.tx * th + t.xo, y = t.y;
    const int xs1 = x > 0 ? x - 1 : np - 1, xa1 = x < np - 1 ? x + 1 : 0;
    const int ys1 = y > 0 ? y - 1 : g.ny - 1, ya1 = y < g.ny - 1 ? y + 1 : 0;
    auto H = [&](int yy, int xx) { return h[(int64_t)yy * np + xx]; };
    const int cl = t.tx * g.T + t.xo;  // the pair's low cell
    NbH n;
    n.xs1 = t.xo > 0 ? H(y, xs1) : __halves2half2(__high2half(H(y, xs1)), __low2half(H(y, x + th - 1)));
    n.xa1 = t.xo < th - 1 ? H(y, xa1) : __halves2half2(__high2half(H(y, x - th + 1)), __low2half(H(y, xa1)));
    n.ys1 = (t.yo == 0 && type[t.tys1 * g.ntx + t.tx] == 2)
                ? __floats2half2_rn(f[(int64_t)ys1 * g.nx + cl], f[(int64_t)ys1 * g.nx + cl + th])
                : H(ys1, x);
    n.ya1 = (t.yo == g.T - 1 && type[t.tya1 * g.ntx + t.tx] == 2)
                ? __floats2half2_rn(f[(int64_t)ya1 * g.nx + cl], f[(int64_t)ya1 * g.nx + cl + th])
                : H(ya1, x);
    return n;
}

// a low tile's pair into the FP64 array: both cells on the tile's first and
// last rows (and, with `all`, everywhere), else the first / last column's cell
__device__ __forceinline__ void low_to_f64(const GeoM &g, const TileAt &t, __half2 v, double *f, bool all)
{
    const int64_t c = (int64_t)t.y * g.nx + t.tx * g.T + t.xo;
    if (t.yo == 0 || t.yo == g.T - 1 || all) {
        f[c] = __low2float(v);
        f[c + t.th] = __high2float(v);
    } else if (t.xo == 0) {
        f[c] = __low2float(v);
    } else if (t.xo == t.th - 1) {
        f[c + t.th] = __high2float(v);
    }
}

// a high tile's first / last column cell into the half2 array (the low half
// of the tile's first pair, the high half of its last pair)
__device__ __forceinline__ void high_edge_to_h2(const GeoM &g, const TileAt &t, int cx, double v, __half2 *h)
{
    const int64_t row = (int64_t)t.y * (g.nx / 2);
    if (cx == 0) {
        __half2 &w = h[row + t.tx * t.th];
        w = __halves2half2(__float2half(v), __high2half(w));
    }
    if (cx == g.T - 1) {
        __half2 &w = h[row + t.tx * t.th + t.th - 1];
        w = __halves2half2(__low2half(w), __float2half(v));
    }
}

struct SintPtrs {
    double *con, *last, *con_lap, *eta1, *eta2, *dfd, *dummy, *dummy_lap;
    __half2 *hcon, *hcon_lap, *heta1, *heta2, *hdfd, *hdummy, *hdummy_lap;
    const int *type;
};

// sintering/function.h:161-330: con_lap, dfdcon and the chemical potential (dummy)
__global__ void sint_con1_k(GeoM g, SintH c, SintD d, SintPtrs m, int step, int cadence, bool snap)
{
    const TileAt t = tile_at(g);
    const int own = m.type[t.ty * g.ntx + t.tx];
    const int y = t.y, nx = g.nx, np = g.nx / 2;
    const int64_t row = (int64_t)y * nx;
    // Monitor2: every cell of con at the period's first step
    if (snap && step % cadence == 0) {
        m.last[row + t.c0] = m.con[row + t.c0];
        m.last[row + t.c0 + t.th] = m.con[row + t.c0 + t.th];
    }
    if (own == 1) {
        const int64_t i = (int64_t)y * np + t.tx * t.th + t.xo;
        const NbH n = nb_low(g, t, m.type, m.hcon, m.con);
        const __half2 cc = m.hcon[i], e1 = m.heta1[i], e2 = m.heta2[i];
        const __half2 lap = (n.xs1 + n.xa1 + n.ys1 + n.ya1 - c.cf * cc) / c.dxdy;
        m.hcon_lap[i] = lap;
        const __half2 sum2 = e1 * e1 + e2 * e2;
        const __half2 sum3 = e1 * e1 * e1 + e2 * e2 * e2;
        const __half2 f = (c.two * cc + c.four * sum3 - c.six * sum2) - c.thirtytwo * (cc * cc) * (c.one - cc) +
                          c.thirtytwo * cc * ((c.one - cc) * (c.one - cc));
        m.hdfd[i] = f;
        const __half2 mu = f - c.zpfive * c.coefm * lap;
        m.hdummy[i] = mu;
        low_to_f64(g, t, mu, m.dummy, false);
        return;
    }
    for (int k = 0; k < 2; ++k) {
        const int cx = t.xo + k * t.th, x = t.tx * g.T + cx;
        const int xs1 = x > 0 ? x - 1 : nx - 1, xa1 = x < nx - 1 ? x + 1 : 0;
        const int ys1 = y > 0 ? y - 1 : g.ny - 1, ya1 = y < g.ny - 1 ? y + 1 : 0;
        auto C = [&](int yy, int xx) { return m.con[(int64_t)yy * nx + xx]; };
        const int64_t i = row + x;
        const double lap = (C(y, xs1) + C(y, xa1) + C(ys1, x) + C(ya1, x) - 4.0 * C(y, x)) / d.dxdy;
        m.con_lap[i] = lap;
        const double e1 = m.eta1[i], e2 = m.eta2[i], cc = m.con[i];
        const double sum2 = pow(e1, 2) + pow(e2, 2);
        const double sum3 = pow(e1, 3) + pow(e2, 3);
        const double f = 1.0 * (2.0 * cc + 4.0 * sum3 - 6.0 * sum2) - 2.0 * 16.0 * pow(cc, 2) * (1.0 - cc) +
                         2.0 * 16.0 * cc * pow(1.0 - cc, 2);
        m.dfd[i] = f;
        const double mu = f - d.hcoefm * lap;
        m.dummy[i] = mu;
        high_edge_to_h2(g, t, cx, mu, m.hdummy);
    }
}

// sintering/function.h:331-482: con advanced by the mobility times the potential's Laplacian, clamped to [0, 1]
__global__ void sint_con2_k(GeoM g, SintH c, SintD d, SintPtrs m, int step, int cadence)
{
    const TileAt t = tile_at(g);
    const int own = m.type[t.ty * g.ntx + t.tx];
    const int y = t.y, nx = g.nx, np = g.nx / 2;
    const int64_t row = (int64_t)y * nx;
    if (own == 1) {
        const int64_t i = (int64_t)y * np + t.tx * t.th + t.xo;
        const NbH n = nb_low(g, t, m.type, m.hdummy, m.dummy);
        const __half2 lap = (n.xs1 + n.xa1 + n.ys1 + n.ya1 - c.cf * m.hdummy[i]) / c.dxdy;
        m.hdummy_lap[i] = lap;
        const __half2 cc = m.hcon[i];
        const __half2 phi = cc * cc * cc * (c.ten - c.fifteen * cc + c.six * (cc * cc));
        const __half2 sum = m.heta1[i] * m.heta2[i] * c.two;
        const __half2 mob = c.dvol * phi + c.dvap * (c.one - phi) + c.dsur * cc * (c.one - cc) + c.dgrb * sum;
        __half2 v = cc + c.dt * mob * lap;
        v = __hmin2(c.hi, v);
        v = __hmax2(c.lo, v);
        m.hcon[i] = v;
        low_to_f64(g, t, v, m.con, (step + 1) % cadence == 0);
        return;
    }
    for (int k = 0; k < 2; ++k) {
        const int cx = t.xo + k * t.th, x = t.tx * g.T + cx;
        const int xs1 = x > 0 ? x - 1 : nx - 1, xa1 = x < nx - 1 ? x + 1 : 0;
        const int ys1 = y > 0 ? y - 1 : g.ny - 1, ya1 = y < g.ny - 1 ? y + 1 : 0;
        auto D = [&](int yy, int xx) { return m.dummy[(int64_t)yy * nx + xx]; };
        const int64_t i = row + x;
        const double lap = (D(y, xs1) + D(y, xa1) + D(ys1, x) + D(ya1, x) - 4.0 * D(y, x)) / d.dxdy;
        m.dummy_lap[i] = lap;
        const double cc = m.con[i];
        const double phi = pow(cc, 3) * (10.0 - 15.0 * cc + 6.0 * pow(cc, 2));
        const double sum = m.eta1[i] * m.eta2[i] * 2;
        const double mob = d.dvol * phi + d.dvap * (1.0 - phi) + d.dsur * cc * (1.0 - cc) + d.dgrb * sum;
        double v = cc + d.dt * mob * lap;
        if (v >= 1) v = 1;
        else if (v < 0) v = 0;
        m.con[i] = v;
        high_edge_to_h2(g, t, cx, v, m.hcon);
    }
}

struct SintPhiPtrs {
    const double *a, *b, *con;  // this order parameter, the other one, con
    double *out, *lap, *dfd;
    const __half2 *ha, *hb, *hcon;
    __half2 *hout, *hlap, *hdfd;
    const int *type;
};

// sintering/function.h:483-774 (phi1_mix, and phi2_mix with the fields
// swapped): one order parameter's update, clamped to [0, 1].  The sum of
// squares keeps the reference's operand order, eta1's term first (SECOND:
// this is eta2), in two kernels as the reference has them: the compiler
// canonicalises a run-time choice between the two orders into one, and the
// two orders can round differently once a product is fused.
template <bool SECOND>
__global__ void sint_phi_k(GeoM g, SintH c, SintD d, SintPhiPtrs m, int step, int cadence)
{
    const TileAt t = tile_at(g);
    const int own = m.type[t.ty * g.ntx + t.tx];
    const int y = t.y, nx = g.nx, np = g.nx / 2;
    const int64_t row = (int64_t)y * nx;
    if (own == 1) {
        const int64_t i = (int64_t)y * np + t.tx * t.th + t.xo;
        const NbH n = nb_low(g, t, m.type, m.ha, m.a);
        const __half2 e = m.ha[i], o = m.hb[i], cc = m.hcon[i];
        const __half2 lap = (n.xs1 + n.xa1 + n.ys1 + n.ya1 - c.cf * e) / c.dxdy;
        m.hlap[i] = lap;
        __half2 sum2;
        if constexpr (SECOND) sum2 = (o * o) + (e * e);
        else sum2 = (e * e) + (o * o);
        const __half2 f = c.one * (-c.twelve * (e * e) * (c.two - cc) + c.twelve * e * (c.one - cc) + c.twelve * e * sum2);
        m.hdfd[i] = f;
        __half2 v = e - c.dt * c.coefl * (f - c.zpfive * c.coefk * lap);
        v = __hmin2(c.hi, v);
        v = __hmax2(c.lo, v);
        m.hout[i] = v;
        low_to_f64(g, t, v, m.out, (step + 1) % cadence == 0);
        return;
    }
    for (int k = 0; k < 2; ++k) {
        const int cx = t.xo + k * t.th, x = t.tx * g.T + cx;
        const int xs1 = x > 0 ? x - 1 : nx - 1, xa1 = x < nx - 1 ? x + 1 : 0;
        const int ys1 = y > 0 ? y - 1 : g.ny - 1, ya1 = y < g.ny - 1 ? y + 1 : 0;
        auto A = [&](int yy, int xx) { return m.a[(int64_t)yy * nx + xx]; };
        const int64_t i = row + x;
        const double lap = (A(y, xs1) + A(y, xa1) + A(ys1, x) + A(ya1, x) - 4.0 * A(y, x)) / d.dxdy;
        m.lap[i] = lap;
        const double e = m.a[i], cc = m.con[i];
        double sum2;
        if constexpr (SECOND) sum2 = pow(m.b[i], 2) + pow(e, 2);
        else sum2 = pow(e, 2) + pow(m.b[i], 2);
        // the reference's expression with its multiply-adds fused as its
        // build fuses them (each sum takes the product on its left; the
        // update, e - dtime*coefl*(...), one fused step), stated with
        // explicit roundings: inlined in this kernel the compiler left the
        // last one unfused
        const double m12 = __dmul_rn(12.0, e);
        const double s12 = __fma_rn(__dmul_rn(-12.0, pow(e, 2)), 2.0 - cc, __dmul_rn(m12, 1.0 - cc));
        const double f = __fma_rn(m12, sum2, s12);
        m.dfd[i] = f;
        double v = __fma_rn(-d.dtcoefl, __fma_rn(-d.hcoefk, lap, f), e);
        if (v >= 1) v = 1;
        else if (v < 0) v = 0;
        m.out[i] = v;
        high_edge_to_h2(g, t, cx, v, (__half2 *)m.hout);
    }
}

// sintering/function.h:792-900: the conversions of con1/con2/phi1/phi2_mix as
// their own launches (`all`: every low-tile cell at a period's last step,
// when the field's conversion has that clause)
__global__ void sint_conv_k(GeoM g, const int *type, double *f, __half2 *h, int step, int cadence, bool period_clause)
{
    const TileAt t = tile_at(g);
    if (type[t.ty * g.ntx + t.tx] == 1) {
        const __half2 v = h[(int64_t)t.y * (g.nx / 2) + t.tx * t.th + t.xo];
        low_to_f64(g, t, v, f, period_clause && (step + 1) % cadence == 0);
        return;
    }
    for (int k = 0; k < 2; ++k) {
        const int cx = t.xo + k * t.th;
        high_edge_to_h2(g, t, cx, f[(int64_t)t.y * g.nx + t.tx * g.T + cx], h);
    }
}

// sintering/tools.h:57-79: tiles turning high -> low take their pairs of con, eta1, eta2 from the FP64 arrays
__global__ void sint_sync_during(GeoM g, const double *c, const double *e1, const double *e2, __half2 *hc,
                                 __half2 *h1, __half2 *h2p, const int *old_t, const int *new_t)
{
    const TileAt t = tile_at(g);
    const int tile = t.ty * g.ntx + t.tx;
    if (!(old_t[tile] == 2 && new_t[tile] == 1)) return;
    const int64_t i = (int64_t)t.y * (g.nx / 2) + t.tx * t.th + t.xo, f = (int64_t)t.y * g.nx + t.c0;
    hc[i] = __floats2half2_rn(c[f], c[f + t.th]);
    h1[i] = __floats2half2_rn(e1[f], e1[f + t.th]);
    h2p[i] = __floats2half2_rn(e2[f], e2[f + t.th]);
}

// sintering/tools.h:80-94 and 95-121: every pair from the FP64 array / low tiles' pairs into it
__global__ void sint_to_low(GeoM g, const double *f, __half2 *h)
{
    const TileAt t = tile_at(g);
    const int64_t c = (int64_t)t.y * g.nx + t.c0;
    h[(int64_t)t.y * (g.nx / 2) + t.tx * t.th + t.xo] = __floats2half2_rn(f[c], f[c + t.th]);
}
__global__ void sint_sync_after(GeoM g, double *f, const __half2 *h, const int *type)
{
    const TileAt t = tile_at(g);
    if (type[t.ty * g.ntx + t.tx] != 1) return;
    const __half2 v = h[(int64_t)t.y * (g.nx / 2) + t.tx * t.th + t.xo];
    const int64_t c = (int64_t)t.y * g.nx + t.c0;
    f[c] = __low2float(v);
    f[c + t.th] = __high2float(v);
}

// sintering/function.h:778-790: con into con_last at a period's first step
__global__ void sint_last_k(GeoM g, const double *con, double *last, int step, int cadence)
{
    if (step % cadence) return;
    const TileAt t = tile_at(g);
    const int64_t c = (int64_t)t.y * g.nx + t.c0;
    last[c] = con[c];
    last[c + t.th] = con[c + t.th];
}

// graingrowth/tools.h:24-38 -- the initial circle in FP64 arrays, one cell a thread
__global__ void gg_prep_high(int nx, int ny, float rx, float ry, float r, double *e1, double *e2)
{
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const float d = sqrt(pow(x - rx, 2) + pow(y - ry, 2));
    const int64_t i = (int64_t)y * nx + x;
    e1[i] = d <= r ? 0 : 1;
    e2[i] = d <= r ? 1 : 0;
}

// per-pair tools over tiles (one CTA per tile, (T/2) x T threads): the pair
// index and row of this thread, and its tile's type
struct PairAt {
    int x, y, tile;
};
__device__ __forceinline__ PairAt pair_at(const GeoM &g)
{
    int tx, ty;
    tile_of(g, tx, ty);
    return PairAt{tx * (g.T / 2) + (int)threadIdx.x, ty * g.T + (int)threadIdx.y, ty * g.ntx + tx};
}

// graingrowth/tools.h:256-271: tiles turning high -> low take their half2 pairs from the FP64 arrays
__global__ void gg_sync_during(GeoM g, const double *e1, const double *e2, __half2 *h1, __half2 *h2p,
                               const int *old_t, const int *new_t)
{
    const PairAt q = pair_at(g);
    if (!(old_t[q.tile] == 2 && new_t[q.tile] == 1)) return;
    const int64_t i = (int64_t)q.y * (g.nx / 2) + q.x, c = (int64_t)q.y * g.nx + 2 * q.x;
    h1[i] = __floats2half2_rn(e1[c], e1[c + 1]);
    h2p[i] = __floats2half2_rn(e2[c], e2[c + 1]);
}

// graingrowth/tools.h:172-200 (AMSTENCIL): low tiles' pairs into the FP64 array
__global__ void gg_sync_after(GeoM g, double *hi, const __half2 *lo, const int *type)
{
    const PairAt q = pair_at(g);
    if (type[q.tile] != 1) return;
    const __half2 v = lo[(int64_t)q.y * (g.nx / 2) + q.x];
    const int64_t c = (int64_t)q.y * g.nx + 2 * q.x;
    hi[c] = __low2float(v);
    hi[c + 1] = __high2float(v);
}

// graingrowth/tools.h:158-171 (AMSTENCIL): every pair from the FP64 array
__global__ void gg_high_to_low(GeoM g, const double *hi, __half2 *lo)
{
    const PairAt q = pair_at(g);
    const int64_t c = (int64_t)q.y * g.nx + 2 * q.x;
    lo[(int64_t)q.y * (g.nx / 2) + q.x] = __floats2half2_rn(hi[c], hi[c + 1]);
}

// graingrowth/function.h:323-341: kernel1_mix's conversion as its own launch
__global__ void gg_conversion(GeoM g, double *out, const __half2 *hout, const int *type, int step, int cadence)
{
    const PairAt q = pair_at(g);
    if (type[q.tile] != 1) return;
    const int xo = threadIdx.x, yo = threadIdx.y, th = g.T / 2;
    const __half2 o = hout[(int64_t)q.y * (g.nx / 2) + q.x];
    const int64_t c = (int64_t)q.y * g.nx + 2 * q.x;
    if (yo == 0 || yo == g.T - 1 || (step + 1) % cadence == 0) {
        out[c] = __low2float(o);
        out[c + 1] = __high2float(o);
    } else if (xo == 0) {
        out[c] = __low2float(o);
    } else if (xo == th - 1) {
        out[c + 1] = __high2float(o);
    }
}

// graingrowth/function.h:311-321: every cell into the snapshot
__global__ void gg_last_store(GeoM g, const double *a, double *last)
{
    int tx, ty;
    tile_of(g, tx, ty);
    const int64_t c = (int64_t)(ty * g.T + (int)threadIdx.y) * g.nx + tx * g.T + (int)threadIdx.x;
    last[c] = a[c];
    last[c + g.T / 2] = a[c + g.T / 2];
}

int check_half2(const amps_params *p)
{
    if (!p || p->nx < 4 || p->ny < 5 || p->nx % 2 || p->bc != AMPS_BC_PERIODIC) return AMPS_ERR_INVALID;
    return AMPS_OK;
}

GeoH geoh(const amps_params *p) { return GeoH{p->nx / 2, p->ny}; }

// the tiled half2 kernels: square tiles of an even side dividing both sides, at most 32
int check_mix(const amps_params *p)
{
    if (check_half2(p)) return AMPS_ERR_INVALID;
    const int T = p->tile;
    if (T < 2 || T > 32 || T % 2 || p->nx % T || p->ny % T) return AMPS_ERR_INVALID;
    return AMPS_OK;
}
GeoM geom(const amps_params *p) { return GeoM{p->nx, p->ny, p->tile, p->nx / p->tile, p->ny / p->tile}; }
dim3 tiles_grid(const amps_params *p) { return dim3((unsigned)((p->nx / p->tile) * (p->ny / p->tile))); }
dim3 pair_block(const amps_params *p) { return dim3((unsigned)(p->tile / 2), (unsigned)p->tile); }
// sintering/tools.h:122-127: each constant as __floats2half2_rn(v, v)
SintH sinth(const amps_params *p)
{
    return SintH{h2(4.0),      h2(p->dx * p->dy), h2(0.5),      h2(1.0),      h2(2.0),      h2(4.0),
                 h2(6.0),      h2(10.0),          h2(12.0),     h2(15.0),     h2(32.0),     h2(p->coefm),
                 h2(p->coefk), h2(p->coefl),      h2(p->dvol),  h2(p->dvap),  h2(p->dsur),  h2(p->dgrb),
                 h2(p->dt),    h2(1.0),           h2(0.0)};
}
SintD sintd(const amps_params *p)
{
    return SintD{p->dx * p->dy, 0.5 * p->coefm, 0.5 * p->coefk, p->dt * p->coefl, p->dt,
                 p->dvol,       p->dvap,        p->dsur,        p->dgrb};
}
KobD kobd(const amps_params *p)
{
    return KobD{p->dx * p->dy, 2.0 * p->dx, 2.0 * p->dy, p->epsb, p->delta, p->aniso, p->theta0,
                -p->epsb * p->aniso * p->delta, p->alpha / p->pi, p->gama, p->teq, p->dt / p->tau, p->dt, p->kappa};
}
GgH ggh(const amps_params *p)
{
    return GgH{h2(1.0), h2(2.0), h2(8.0), h2(p->dt), h2(p->mobil), h2(p->grcoef), h2(p->dx * p->dy)};
}
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
    const GgH c = ggh(p);
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

extern "C" int amps_graingrowth_kernel1_mix(const amps_params *p, const double *etaa, double *etaa_last,
                                            const double *etab, double *etaa_lap, double *dfdetaa, double *etaa_out,
                                            const void *hetaa, const void *hetab, void *hetaa_lap, void *hdfdetaa,
                                            void *hetaa_out, const int *type_curr, int i, int etai, void *stream)
{
    if (check_mix(p) || !etaa || !etab || !etaa_lap || !dfdetaa || !etaa_out || !hetaa || !hetab || !hetaa_lap ||
        !hdfdetaa || !hetaa_out || !type_curr || etaa == etaa_out || hetaa == hetaa_out || p->cadence < 1)
        return AMPS_ERR_INVALID;
    const bool snap = p->monitor == AMPS_MONITOR_TEM;
    if (snap && !etaa_last) return AMPS_ERR_INVALID;
    const MixPtrs m{etaa, etaa_last, etab, etaa_lap, dfdetaa, etaa_out, (const __half2 *)hetaa, (const __half2 *)hetab,
                    (__half2 *)hetaa_lap, (__half2 *)hdfdetaa, (__half2 *)hetaa_out, type_curr};
    gg_mix_k<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), ggh(p), p->dx * p->dy, p->dt * p->mobil, p->grcoef,
                                                      m, i, etai, p->cadence, snap);
    return launched();
}

extern "C" int amps_graingrowth_dataprepare_high(const amps_params *p, double *eta1, double *eta2, void *stream)
{
    if (!p || p->nx < 1 || p->ny < 1 || !eta1 || !eta2) return AMPS_ERR_INVALID;
    const dim3 grid((p->nx + kBX - 1) / kBX, (p->ny + kBY - 1) / kBY);
    gg_prep_high<<<grid, dim3(kBX, kBY), 0, S_>>>(p->nx, p->ny, (float)(p->nx / 2), (float)(p->ny / 2),
                                                  (float)p->init_r, eta1, eta2);
    return launched();
}

extern "C" int amps_graingrowth_data_sychro_duringcomputation(const amps_params *p, const double *eta1,
                                                              const double *eta2, void *heta1, void *heta2,
                                                              const int *old_con, const int *new_con, void *stream)
{
    if (check_mix(p) || !eta1 || !eta2 || !heta1 || !heta2 || !old_con || !new_con) return AMPS_ERR_INVALID;
    gg_sync_during<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), eta1, eta2, (__half2 *)heta1,
                                                            (__half2 *)heta2, old_con, new_con);
    return launched();
}

extern "C" int amps_graingrowth_data_sychro_aftercomputation(const amps_params *p, double *highdata,
                                                             const void *lowdata, const int *typedata, void *stream)
{
    if (check_mix(p) || !highdata || !lowdata || !typedata) return AMPS_ERR_INVALID;
    gg_sync_after<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), highdata, (const __half2 *)lowdata, typedata);
    return launched();
}

extern "C" int amps_graingrowth_highdata_to_low(const amps_params *p, const double *highdata, void *lowdata,
                                                void *stream)
{
    if (check_mix(p) || !highdata || !lowdata) return AMPS_ERR_INVALID;
    gg_high_to_low<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), highdata, (__half2 *)lowdata);
    return launched();
}

extern "C" int amps_graingrowth_kernel1_conversion(const amps_params *p, double *etaa_out, const void *hetaa_out,
                                                   const int *type_curr, int i, void *stream)
{
    if (check_mix(p) || !etaa_out || !hetaa_out || !type_curr || p->cadence < 1) return AMPS_ERR_INVALID;
    gg_conversion<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), etaa_out, (const __half2 *)hetaa_out,
                                                           type_curr, i, p->cadence);
    return launched();
}

extern "C" int amps_graingrowth_monitor2_lastdata_store(const amps_params *p, const double *etaa, double *etaa_last,
                                                        void *stream)
{
    if (check_mix(p) || !etaa || !etaa_last) return AMPS_ERR_INVALID;
    gg_last_store<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), etaa, etaa_last);
    return launched();
}

// the Kobayashi step's arrays, reference order (snowflake/function.h:63, 376)
static KobMixPtrs kob_ptrs(double *phi, double *phi_last, double *phi_lap, double *epsilon, double *epsilon_deri,
                           double *phidx, double *phidy, double *tempr, double *tempr_lap, void *hphi, void *hphi_lap,
                           void *htempr, void *htempr_lap, void *hphidx, void *hphidy, void *hepsilon,
                           void *hepsilon_deri, const int *type_curr)
{
    return KobMixPtrs{phi,  phi_last, phi_lap, epsilon, epsilon_deri, phidx, phidy, tempr, tempr_lap,
                      (__half2 *)hphi, (__half2 *)hphi_lap, (__half2 *)htempr, (__half2 *)htempr_lap,
                      (__half2 *)hphidx, (__half2 *)hphidy, (__half2 *)hepsilon, (__half2 *)hepsilon_deri, type_curr};
}

extern "C" int amps_snowflake_kernel1_mix(const amps_params *p, const double *phi, double *phi_last, double *phi_lap,
                                          double *epsilon, double *epsilon_deri, double *phidx, double *phidy,
                                          const double *tempr, double *tempr_lap, const void *hphi, void *hphi_lap,
                                          const void *htempr, void *htempr_lap, void *hphidx, void *hphidy,
                                          void *hepsilon, void *hepsilon_deri, const int *type_curr, int i,
                                          void *stream)
{
    if (check_mix(p) || p->tile < 4 || !phi || !phi_lap || !epsilon || !epsilon_deri || !phidx || !phidy || !tempr ||
        !tempr_lap || !hphi || !hphi_lap || !htempr || !htempr_lap || !hphidx || !hphidy || !hepsilon ||
        !hepsilon_deri || !type_curr || p->cadence < 1)
        return AMPS_ERR_INVALID;
    const bool snap = p->monitor == AMPS_MONITOR_TEM;
    if (snap && !phi_last) return AMPS_ERR_INVALID;
    const KobMixPtrs m = kob_ptrs((double *)phi, phi_last, phi_lap, epsilon, epsilon_deri, phidx, phidy,
                                  (double *)tempr, tempr_lap, (void *)hphi, hphi_lap, (void *)htempr, htempr_lap,
                                  hphidx, hphidy, hepsilon, hepsilon_deri, type_curr);
    kob_mix_k1<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), kobh(p), kobd(p), m, i, p->cadence, snap);
    return launched();
}

extern "C" int amps_snowflake_mix_kernel2(const amps_params *p, double *phi, const double *phi_lap,
                                          const double *epsilon, const double *epsilon_deri, const double *phidx,
                                          const double *phidy, double *tempr, const double *tempr_lap, void *hphi,
                                          const void *hphi_lap, const void *hepsilon, const void *hepsilon_deri,
                                          const void *hphidx, const void *hphidy, void *htempr,
                                          const void *htempr_lap, const int *type_curr, int i, void *stream)
{
    if (check_mix(p) || p->tile < 4 || !phi || !phi_lap || !epsilon || !epsilon_deri || !phidx || !phidy || !tempr ||
        !tempr_lap || !hphi || !hphi_lap || !hepsilon || !hepsilon_deri || !hphidx || !hphidy || !htempr ||
        !htempr_lap || !type_curr || p->cadence < 1)
        return AMPS_ERR_INVALID;
    const KobMixPtrs m = kob_ptrs(phi, nullptr, (double *)phi_lap, (double *)epsilon, (double *)epsilon_deri,
                                  (double *)phidx, (double *)phidy, tempr, (double *)tempr_lap, hphi, (void *)hphi_lap,
                                  htempr, (void *)htempr_lap, (void *)hphidx, (void *)hphidy, (void *)hepsilon,
                                  (void *)hepsilon_deri, type_curr);
    kob_mix_k2<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), kobh(p), kobd(p), m, i, p->cadence);
    return launched();
}

extern "C" int amps_snowflake_kernel1_conversion(const amps_params *p, double *epsilon, double *epsilon_deri,
                                                 double *phidx, double *phidy, const void *hphidx, const void *hphidy,
                                                 const void *hepsilon, const void *hepsilon_deri,
                                                 const int *type_curr, int i, void *stream)
{
    (void)i;  // the reference's conversion takes the step and does not use it
    if (check_mix(p) || !epsilon || !epsilon_deri || !phidx || !phidy || !hphidx || !hphidy || !hepsilon ||
        !hepsilon_deri || !type_curr)
        return AMPS_ERR_INVALID;
    const KobMixPtrs m = kob_ptrs(nullptr, nullptr, nullptr, epsilon, epsilon_deri, phidx, phidy, nullptr, nullptr,
                                  nullptr, nullptr, nullptr, nullptr, (void *)hphidx, (void *)hphidy,
                                  (void *)hepsilon, (void *)hepsilon_deri, type_curr);
    kob_conv1<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), m);
    return launched();
}

extern "C" int amps_snowflake_kernel2_conversion(const amps_params *p, double *phi, double *tempr, const void *hphi,
                                                 const void *htempr, const int *type_curr, int i, void *stream)
{
    if (check_mix(p) || p->tile < 4 || !phi || !tempr || !hphi || !htempr || !type_curr || p->cadence < 1)
        return AMPS_ERR_INVALID;
    const KobMixPtrs m = kob_ptrs(phi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, tempr, nullptr,
                                  (void *)hphi, nullptr, (void *)htempr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  type_curr);
    kob_conv2<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), m, i, p->cadence);
    return launched();
}

extern "C" int amps_snowflake_monitor2_lastdata_store(const amps_params *p, const double *phi, double *phi_last,
                                                      void *stream)
{
    return amps_graingrowth_monitor2_lastdata_store(p, phi, phi_last, stream);
}

extern "C" int amps_snowflake_data_sychro_duringcomputation(const amps_params *p, const double *phi,
                                                            const double *tempr, void *hphi, void *htempr,
                                                            const int *old_con, const int *new_con, void *stream)
{
    return amps_graingrowth_data_sychro_duringcomputation(p, phi, tempr, hphi, htempr, old_con, new_con, stream);
}

extern "C" int amps_snowflake_data_sychro_aftercomputation(const amps_params *p, double *highdata, const void *lowdata,
                                                           const int *typedata, void *stream)
{
    return amps_graingrowth_data_sychro_aftercomputation(p, highdata, lowdata, typedata, stream);
}

extern "C" int amps_snowflake_highdata_to_low(const amps_params *p, const double *highdata, void *lowdata,
                                              void *stream)
{
    return amps_graingrowth_highdata_to_low(p, highdata, lowdata, stream);
}

extern "C" int amps_sintering_con1_mix(const amps_params *p, const int *type_curr, const double *con, double *con_last,
                                       double *con_lap, const double *eta1, const double *eta2, double *dfdcon,
                                       double *dummy, const void *hcon, void *hcon_lap, const void *heta1,
                                       const void *heta2, void *hdfdcon, void *hdummy, int i, void *stream)
{
    if (check_mix(p) || !type_curr || !con || !con_lap || !eta1 || !eta2 || !dfdcon || !dummy || !hcon ||
        !hcon_lap || !heta1 || !heta2 || !hdfdcon || !hdummy || p->cadence < 1)
        return AMPS_ERR_INVALID;
    const bool snap = p->monitor == AMPS_MONITOR_TEM;
    if (snap && !con_last) return AMPS_ERR_INVALID;
    const SintPtrs m{(double *)con, con_last, con_lap, (double *)eta1, (double *)eta2, dfdcon, dummy, nullptr,
                     (__half2 *)hcon, (__half2 *)hcon_lap, (__half2 *)heta1, (__half2 *)heta2, (__half2 *)hdfdcon,
                     (__half2 *)hdummy, nullptr, type_curr};
    sint_con1_k<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), sinth(p), sintd(p), m, i, p->cadence, snap);
    return launched();
}

extern "C" int amps_sintering_con2_mix(const amps_params *p, const int *type_curr, const double *dummy,
                                       double *dummy_lap, double *con, const double *eta1, const double *eta2,
                                       const void *hdummy, void *hdummy_lap, void *hcon, const void *heta1,
                                       const void *heta2, int i, void *stream)
{
    if (check_mix(p) || !type_curr || !dummy || !dummy_lap || !con || !eta1 || !eta2 || !hdummy || !hdummy_lap ||
        !hcon || !heta1 || !heta2 || p->cadence < 1)
        return AMPS_ERR_INVALID;
    const SintPtrs m{con, nullptr, nullptr, (double *)eta1, (double *)eta2, nullptr, (double *)dummy, dummy_lap,
                     (__half2 *)hcon, nullptr, (__half2 *)heta1, (__half2 *)heta2, nullptr, (__half2 *)hdummy,
                     (__half2 *)hdummy_lap, type_curr};
    sint_con2_k<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), sinth(p), sintd(p), m, i, p->cadence);
    return launched();
}

static int sint_phi(const amps_params *p, const int *type_curr, const double *eta, double *eta_out,
                    const double *other, double *eta_lap, double *dfdeta, const double *con, const void *heta,
                    void *heta_out, const void *hother, void *heta_lap, void *hdfdeta, const void *hcon, int i,
                    bool second, void *stream)
{
    if (check_mix(p) || !type_curr || !eta || !eta_out || !other || !eta_lap || !dfdeta || !con || !heta ||
        !heta_out || !hother || !heta_lap || !hdfdeta || !hcon || eta == eta_out || heta == heta_out ||
        p->cadence < 1)
        return AMPS_ERR_INVALID;
    const SintPhiPtrs m{eta, other, con, eta_out, eta_lap, dfdeta, (const __half2 *)heta, (const __half2 *)hother,
                        (const __half2 *)hcon, (__half2 *)heta_out, (__half2 *)heta_lap, (__half2 *)hdfdeta,
                        type_curr};
    if (second) sint_phi_k<true><<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), sinth(p), sintd(p), m, i, p->cadence);
    else sint_phi_k<false><<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), sinth(p), sintd(p), m, i, p->cadence);
    return launched();
}

extern "C" int amps_sintering_phi1_mix(const amps_params *p, const int *type_curr, const double *eta1,
                                       double *eta1_out, const double *eta2, double *eta1_lap, double *dfdeta1,
                                       const double *con, const void *heta1, void *heta1_out, const void *heta2,
                                       void *heta1_lap, void *hdfdeta1, const void *hcon, int i, void *stream)
{
    return sint_phi(p, type_curr, eta1, eta1_out, eta2, eta1_lap, dfdeta1, con, heta1, heta1_out, heta2, heta1_lap,
                    hdfdeta1, hcon, i, false, stream);
}

extern "C" int amps_sintering_phi2_mix(const amps_params *p, const int *type_curr, const double *eta2,
                                       double *eta2_out, const double *eta1, double *eta2_lap, double *dfdeta2,
                                       const double *con, const void *heta2, void *heta2_out, const void *heta1,
                                       void *heta2_lap, void *hdfdeta2, const void *hcon, int i, void *stream)
{
    return sint_phi(p, type_curr, eta2, eta2_out, eta1, eta2_lap, dfdeta2, con, heta2, heta2_out, heta1, heta2_lap,
                    hdfdeta2, hcon, i, true, stream);
}

static int sint_conv(const amps_params *p, const int *type_curr, double *f, void *h, int i, bool clause,
                     void *stream)
{
    if (check_mix(p) || !type_curr || !f || !h || p->cadence < 1) return AMPS_ERR_INVALID;
    sint_conv_k<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), type_curr, f, (__half2 *)h, i, p->cadence, clause);
    return launched();
}

extern "C" int amps_sintering_con1_conversion(const amps_params *p, const int *type_curr, double *dummy,
                                              void *hdummy, void *stream)
{
    return sint_conv(p, type_curr, dummy, hdummy, 0, false, stream);
}

extern "C" int amps_sintering_con2_conversion(const amps_params *p, const int *type_curr, double *con, void *hcon,
                                              int i, void *stream)
{
    return sint_conv(p, type_curr, con, hcon, i, true, stream);
}

extern "C" int amps_sintering_phi1_conversion(const amps_params *p, const int *type_curr, double *eta1_out,
                                              void *heta1_out, int i, void *stream)
{
    return sint_conv(p, type_curr, eta1_out, heta1_out, i, true, stream);
}

extern "C" int amps_sintering_phi2_conversion(const amps_params *p, const int *type_curr, double *eta2_out,
                                              void *heta2_out, int i, void *stream)
{
    return sint_conv(p, type_curr, eta2_out, heta2_out, i, true, stream);
}

extern "C" int amps_sintering_monitor2_lastdata_store(const amps_params *p, const double *con, double *con_last,
                                                      int i, void *stream)
{
    if (check_mix(p) || !con || !con_last || p->cadence < 1) return AMPS_ERR_INVALID;
    sint_last_k<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), con, con_last, i, p->cadence);
    return launched();
}

extern "C" int amps_sintering_data_sychro_duringcomputation(const amps_params *p, const double *con,
                                                            const double *eta1, const double *eta2, void *hcon,
                                                            void *heta1, void *heta2, const int *old_con,
                                                            const int *new_con, void *stream)
{
    if (check_mix(p) || !con || !eta1 || !eta2 || !hcon || !heta1 || !heta2 || !old_con || !new_con)
        return AMPS_ERR_INVALID;
    sint_sync_during<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), con, eta1, eta2, (__half2 *)hcon,
                                                              (__half2 *)heta1, (__half2 *)heta2, old_con, new_con);
    return launched();
}

extern "C" int amps_sintering_dataprepare(const amps_params *p, const double *highdata, void *lowdata, void *stream)
{
    if (check_mix(p) || !highdata || !lowdata) return AMPS_ERR_INVALID;
    sint_to_low<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), highdata, (__half2 *)lowdata);
    return launched();
}

extern "C" int amps_sintering_data_sychro_aftercomputation(const amps_params *p, double *highdata, const void *lowdata,
                                                           const int *typedata, void *stream)
{
    if (check_mix(p) || !highdata || !lowdata || !typedata) return AMPS_ERR_INVALID;
    sint_sync_after<<<tiles_grid(p), pair_block(p), 0, S_>>>(geom(p), highdata, (const __half2 *)lowdata, typedata);
    return launched();
}
