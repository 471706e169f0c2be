// k_adjoint.cu -- explicit time step and its hand-written adjoint for the
// Kobayashi dendrite and grain growth, on caller-owned row-major arrays
// (float or double), one thread per cell.  No reference counterpart (the
// reference is forward-only); the step restated is snowflake/function.h:5-60
// and graingrowth/function.h:5-30 in the FMA-friendly form.
//
// Kobayashi step, per cell (periodic or zero-flux neighbour map M):
//   px = (phi[M(x+1)] - phi[M(x-1)]) / 2dx,  py likewise,  a = aniso*(atan2(py,px) - theta0)
//   eps = epsb*(1 + delta*cos a),  epd = -epsb*aniso*delta*sin a
//   lap = (sum of phi at the 8 radius-2 cross neighbours - 8 phi) / dxdy
//   term1 = (eps*epd*px)[N] - (eps*epd*px)[S], /2dy;  term2 = -((eps*epd*py)[E] - (eps*epd*py)[W]), /2dx
//   m = alpha/pi*atan(gama*(teq - T)),  g = phi*(1-phi)*(phi - 1/2 + m + noise*chi)
//   phi' = phi + dt/tau*(term1 + term2 + eps^2*lap + g),  T' = T + dt*lapT + K*(phi' - phi)
// The adjoint maps output cotangents (gphi', gT') to input cotangents and adds
// dL/d(delta, K, epsb) into a device double[3].  Stencil transposes gather
// over every preimage of the neighbour map, so zero-flux (mirror) boundaries
// are differentiated exactly, not only periodic ones.
#include "../../include/amps.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace {

constexpr int kAdjThreads = 256;

struct KobAdj {
    int nx, ny, bc;
    double dx, dy, dxdy, dt, tau, epsb, delta, aniso, theta0, alpha, gama, teq, pi, kappa, noise;
    uint64_t seed;
    int64_t step;
};

__device__ __forceinline__ int nbmap(int i, int n, int bc)
{
    if (bc == 0) return i < 0 ? i + n : (i >= n ? i - n : i);
    return i < 0 ? -i - 1 : (i >= n ? 2 * n - i - 1 : i);
}

// Sum of arr over the cells j whose neighbour at offset k maps to c along one
// axis, i.e. {j : M(j+k) = c}; at most two such j with zero-flux boundaries.
__device__ __forceinline__ int preimages(int c, int k, int n, int bc, int *j)
{
    if (bc == 0) {
        j[0] = nbmap(c - k, n, 0);
        return 1;
    }
    int m = 0;
    if (c - k >= 0 && c - k < n) j[m++] = c - k;
    if (-1 - c - k >= 0) j[m++] = -1 - c - k;
    if (2 * n - 1 - c - k < n) j[m++] = 2 * n - 1 - c - k;
    return m;
}

template <typename R>
__device__ __forceinline__ R fold(const R *arr, int cx, int cy, int kx, int ky, int nx, int ny, int bc)
{
    int jx[3], jy[3];
    const int mx = preimages(cx, kx, nx, bc, jx), my = preimages(cy, ky, ny, bc, jy);
    R s = R(0);
    for (int a = 0; a < my; ++a)
        for (int b = 0; b < mx; ++b) s += arr[(int64_t)jy[a] * nx + jx[b]];
    return s;
}

__device__ __forceinline__ double u01(uint64_t seed, uint64_t a, uint64_t b)
{
    auto mix = [](uint64_t z) {
        z += 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    return (double)(mix(mix(seed ^ mix(a)) + b) >> 11) * 0x1.0p-53;
}

template <typename R> __device__ __forceinline__ R at(const R *f, int x, int y, const KobAdj &p)
{
    return f[(int64_t)nbmap(y, p.ny, p.bc) * p.nx + nbmap(x, p.nx, p.bc)];
}

// Per-cell intermediates: w = [eps, epd, px, py, lap phi] (each an n-array).
template <typename R> __global__ void kob_inter_kernel(KobAdj p, const R *phi, R *w)
{
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % p.nx), y = (int)(i / p.nx);
    const R px = (at(phi, x + 1, y, p) - at(phi, x - 1, y, p)) * R(0.5 / p.dx);
    const R py = (at(phi, x, y + 1, p) - at(phi, x, y - 1, p)) * R(0.5 / p.dy);
    const R a = R(p.aniso) * (atan2(py, px) - R(p.theta0));
    w[i] = R(p.epsb) * (R(1) + R(p.delta) * cos(a));
    w[n + i] = R(-p.epsb * p.aniso * p.delta) * sin(a);
    w[2 * n + i] = px;
    w[3 * n + i] = py;
    const R s = (at(phi, x - 1, y, p) + at(phi, x + 1, y, p)) + (at(phi, x - 2, y, p) + at(phi, x + 2, y, p)) +
                (at(phi, x, y - 1, p) + at(phi, x, y + 1, p)) + (at(phi, x, y - 2, p) + at(phi, x, y + 2, p));
    w[4 * n + i] = (s - R(8) * phi[i]) * R(1.0 / p.dxdy);
}

// phi' - phi at cell i from the intermediates (the dt/tau bracket).
template <typename R>
__device__ __forceinline__ R kob_dphi(const KobAdj &p, const R *phi, const R *T, const R *w, int x, int y, int64_t i,
                                      int64_t n, R *m_out, R *drive_out)
{
    auto prod = [&](int xx, int yy, int which) {
        const int64_t j = (int64_t)nbmap(yy, p.ny, p.bc) * p.nx + nbmap(xx, p.nx, p.bc);
        return w[j] * w[n + j] * w[(2 + which) * n + j];
    };
    const R term1 = (prod(x, y + 1, 0) - prod(x, y - 1, 0)) * R(0.5 / p.dy);
    const R term2 = -(prod(x + 1, y, 1) - prod(x - 1, y, 1)) * R(0.5 / p.dx);
    const R ph = phi[i];
    const R m = R(p.alpha / p.pi) * atan(R(p.gama) * (R(p.teq) - T[i]));
    R drive = ph - R(0.5) + m;
    if (p.noise != 0.0) drive += R(p.noise) * (R(u01(p.seed, (uint64_t)p.step, (uint64_t)i)) - R(0.5));
    *m_out = m;
    *drive_out = drive;
    return R(p.dt / p.tau) * (term1 + term2 + w[i] * w[i] * w[4 * n + i] + ph * (R(1) - ph) * drive);
}

template <typename R>
__global__ void kob_update_kernel(KobAdj p, const R *phi, const R *T, const R *w, R *phi_out, R *T_out)
{
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % p.nx), y = (int)(i / p.nx);
    R m, drive;
    const R d = kob_dphi(p, phi, T, w, x, y, i, n, &m, &drive);
    const R s = (at(T, x - 1, y, p) + at(T, x + 1, y, p)) + (at(T, x - 2, y, p) + at(T, x + 2, y, p)) +
                (at(T, x, y - 1, p) + at(T, x, y + 1, p)) + (at(T, x, y - 2, p) + at(T, x, y + 2, p));
    const R lapT = (s - R(8) * T[i]) * R(1.0 / p.dxdy);
    phi_out[i] = phi[i] + d;
    T_out[i] = T[i] + R(p.dt) * lapT + R(p.kappa) * d;
}

// Adjoint, pass 1: mu = gphi' + K gT' (the total cotangent of phi').
template <typename R> __global__ void kob_mu_kernel(KobAdj p, const R *gphi_out, const R *gT_out, R *mu)
{
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) mu[i] = gphi_out[i] + R(p.kappa) * gT_out[i];
}

template <typename R> __device__ __forceinline__ double block_sum(R v, double *red)
{
    double d = (double)v;
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < kAdjThreads / 32; ++k) s += red[k];
    return s;
}

// Adjoint, pass 2: cotangents of (eps, epd, px, py) at every cell, pushed
// through theta = atan2(py, px); writes lpx, lpy and Q = dt/tau*mu*eps^2/dxdy
// (into v = [lpx, lpy, Q]); adds dL/d delta and dL/d epsb.
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) kob_adj_inter_kernel(KobAdj p, const R *w, const R *mu, R *v,
                                                                    double *gparams)
{
    __shared__ double red[kAdjThreads / 32];
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    R gd = R(0), ge = R(0);
    if (i < n) {
        const int x = (int)(i % p.nx), y = (int)(i / p.nx);
        const R dtt = R(p.dt / p.tau);
        // term1 at e uses (eps*epd*px) at N = M(e+y) (+) and S = M(e-y) (-), over 2dy
        const R A = dtt * R(0.5 / p.dy) *
                    (fold(mu, x, y, 0, 1, p.nx, p.ny, p.bc) - fold(mu, x, y, 0, -1, p.nx, p.ny, p.bc));
        // term2 at e uses (eps*epd*py) at E = M(e+x) (-) and W = M(e-x) (+), over 2dx
        const R B = dtt * R(0.5 / p.dx) *
                    (fold(mu, x, y, -1, 0, p.nx, p.ny, p.bc) - fold(mu, x, y, 1, 0, p.nx, p.ny, p.bc));
        const R C = dtt * mu[i] * w[4 * n + i];
        const R e = w[i], ed = w[n + i], px = w[2 * n + i], py = w[3 * n + i];
        const R le = A * ed * px + B * ed * py + R(2) * C * e;
        const R led = A * e * px + B * e * py;
        R lpx = A * e * ed, lpy = B * e * ed;
        const R a = R(p.aniso) * (atan2(py, px) - R(p.theta0));
        const R sa = sin(a), ca = cos(a);
        const R la = le * R(-p.epsb * p.delta) * sa + led * R(-p.epsb * p.aniso * p.delta) * ca;
        const R lth = R(p.aniso) * la;
        const R r2 = px * px + py * py;
        if (r2 > R(0)) {  // atan2 has no derivative where the gradient vanishes
            lpx += lth * (-py / r2);
            lpy += lth * (px / r2);
        }
        v[i] = lpx;
        v[n + i] = lpy;
        v[2 * n + i] = dtt * mu[i] * e * e * R(1.0 / p.dxdy);
        gd = le * R(p.epsb) * ca + led * R(-p.epsb * p.aniso) * sa;
        ge = le * (R(1) + R(p.delta) * ca) + led * R(-p.aniso * p.delta) * sa;
    }
    const double sd = block_sum(gd, red);
    const double se = block_sum(ge, red);
    if (threadIdx.x == 0) {
        atomicAdd(&gparams[0], sd);
        atomicAdd(&gparams[2], se);
    }
}

// Adjoint, pass 3: input cotangents (gphi, gT) and dL/dK.
template <typename R>
__global__ void __launch_bounds__(kAdjThreads)
    kob_adj_out_kernel(KobAdj p, const R *phi, const R *T, const R *w, const R *mu, const R *v, const R *gphi_out,
                       const R *gT_out, R *gphi, R *gT, double *gparams)
{
    __shared__ double red[kAdjThreads / 32];
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    R gk = R(0);
    if (i < n) {
        const int x = (int)(i % p.nx), y = (int)(i / p.nx);
        const int nx = p.nx, ny = p.ny, bc = p.bc;
        R m, drive;
        const R d = kob_dphi(p, phi, T, w, x, y, i, n, &m, &drive);
        const R ph = phi[i], dtt = R(p.dt / p.tau);
        const R *Q = v + 2 * n;
        // radius-2 cross transpose of Q (lap of phi) and of gT' (lap of T)
        R lq = -R(8) * Q[i], lt = -R(8) * gT_out[i];
        const int off[4] = {-2, -1, 1, 2};
        for (int k = 0; k < 4; ++k) {
            lq += fold(Q, x, y, off[k], 0, nx, ny, bc) + fold(Q, x, y, 0, off[k], nx, ny, bc);
            lt += fold(gT_out, x, y, off[k], 0, nx, ny, bc) + fold(gT_out, x, y, 0, off[k], nx, ny, bc);
        }
        const R dpx = (fold(v, x, y, 1, 0, nx, ny, bc) - fold(v, x, y, -1, 0, nx, ny, bc)) * R(0.5 / p.dx);
        const R dpy = (fold(v + n, x, y, 0, 1, nx, ny, bc) - fold(v + n, x, y, 0, -1, nx, ny, bc)) * R(0.5 / p.dy);
        const R dg = (R(1) - R(2) * ph) * drive + ph * (R(1) - ph);
        gphi[i] = gphi_out[i] + dtt * mu[i] * dg + lq + dpx + dpy;
        const R z = R(p.gama) * (R(p.teq) - T[i]);
        const R dm = R(p.alpha / p.pi) * (-R(p.gama)) / (R(1) + z * z);
        gT[i] = gT_out[i] + R(p.dt / p.dxdy) * lt + dtt * mu[i] * ph * (R(1) - ph) * dm;
        gk = gT_out[i] * d;
        (void)m;
    }
    const double sk = block_sum(gk, red);
    if (threadIdx.x == 0) atomicAdd(&gparams[1], sk);
}

}  // namespace

// ---------------------------------------------------------------- grain growth
namespace {

struct GgAdj {
    int nx, ny, bc, q, stencil;
    double dxdy, dt, mobil, grcoef, gamma;
};

template <typename R> __device__ __forceinline__ R gg_at(const R *f, int x, int y, const GgAdj &p)
{
    return f[(int64_t)nbmap(y, p.ny, p.bc) * p.nx + nbmap(x, p.nx, p.bc)];
}

// 8-neighbour (graingrowth/function.h:20) or 5-point Laplacian, / dxdy
template <typename R> __device__ __forceinline__ R gg_lap(const R *f, int x, int y, const GgAdj &p)
{
    R s;
    if (p.stencil == 0)
        s = gg_at(f, x - 1, y - 1, p) + gg_at(f, x, y - 1, p) + gg_at(f, x + 1, y - 1, p) + gg_at(f, x - 1, y, p) +
            gg_at(f, x + 1, y, p) + gg_at(f, x - 1, y + 1, p) + gg_at(f, x, y + 1, p) + gg_at(f, x + 1, y + 1, p) -
            R(8) * gg_at(f, x, y, p);
    else
        s = gg_at(f, x - 1, y, p) + gg_at(f, x + 1, y, p) + gg_at(f, x, y - 1, p) + gg_at(f, x, y + 1, p) -
            R(4) * gg_at(f, x, y, p);
    return s * R(1.0 / p.dxdy);
}

// transpose of gg_lap (exact for both boundary maps)
template <typename R> __device__ __forceinline__ R gg_lap_t(const R *f, int x, int y, const GgAdj &p)
{
    R s;
    const int64_t i = (int64_t)y * p.nx + x;
    if (p.stencil == 0) {
        s = -R(8) * f[i];
        for (int ky = -1; ky <= 1; ++ky)
            for (int kx = -1; kx <= 1; ++kx)
                if (kx || ky) s += fold(f, x, y, kx, ky, p.nx, p.ny, p.bc);
    } else {
        s = fold(f, x, y, -1, 0, p.nx, p.ny, p.bc) + fold(f, x, y, 1, 0, p.nx, p.ny, p.bc) +
            fold(f, x, y, 0, -1, p.nx, p.ny, p.bc) + fold(f, x, y, 0, 1, p.nx, p.ny, p.bc) - R(4) * f[i];
    }
    return s * R(1.0 / p.dxdy);
}

template <typename R> __global__ void gg_fwd_kernel(GgAdj p, const R *eta, R *out)
{
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % p.nx), y = (int)(i / p.nx);
    R S = R(0);
    for (int k = 0; k < p.q; ++k) S += eta[k * n + i] * eta[k * n + i];
    const R dtm = R(p.dt * p.mobil), g2 = R(2.0 * p.gamma), kap = R(p.grcoef);
    for (int k = 0; k < p.q; ++k) {
        const R e = eta[k * n + i], e2 = e * e;
        const R dfd = e * (e2 - R(1) + g2 * (S - e2));
        out[k * n + i] = e - dtm * (dfd - kap * gg_lap(eta + k * n, x, y, p));
    }
}

// input cotangents of all q fields; adds dL/d(L, kappa, gamma) into gparams
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) gg_adj_kernel(GgAdj p, const R *eta, const R *gout, R *gin,
                                                             double *gparams)
{
    __shared__ double red[kAdjThreads / 32];
    const int64_t n = (int64_t)p.nx * p.ny;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    R gl = R(0), gkap = R(0), ggam = R(0);
    if (i < n) {
        const int x = (int)(i % p.nx), y = (int)(i / p.nx);
        R S = R(0), P = R(0);
        for (int k = 0; k < p.q; ++k) {
            S += eta[k * n + i] * eta[k * n + i];
            P += gout[k * n + i] * eta[k * n + i];
        }
        const R dt = R(p.dt), dtm = R(p.dt * p.mobil), g = R(p.gamma), kap = R(p.grcoef);
        for (int k = 0; k < p.q; ++k) {
            const R e = eta[k * n + i], e2 = e * e, gk = gout[k * n + i];
            const R jac = R(3) * e2 - R(1) + R(2) * g * (S - e2);  // d dfd_k / d eta_k
            gin[k * n + i] = gk - dtm * (gk * jac + R(4) * g * e * (P - gk * e)) + dtm * kap * gg_lap_t(gout + k * n, x, y, p);
            const R lap = gg_lap(eta + k * n, x, y, p);
            const R dfd = e * (e2 - R(1) + R(2) * g * (S - e2));
            gl += gk * (-dt) * (dfd - kap * lap);
            gkap += gk * dtm * lap;
            ggam += gk * (-dtm) * R(2) * e * (S - e2);
        }
    }
    const double a = block_sum(gl, red);
    const double b = block_sum(gkap, red);
    const double c = block_sum(ggam, red);
    if (threadIdx.x == 0) {
        atomicAdd(&gparams[0], a);
        atomicAdd(&gparams[1], b);
        atomicAdd(&gparams[2], c);
    }
}

KobAdj kob_args(const amps_params *p, int64_t step)
{
    KobAdj k;
    k.nx = p->nx; k.ny = p->ny; k.bc = p->bc;
    k.dx = p->dx; k.dy = p->dy; k.dxdy = p->dx * p->dy; k.dt = p->dt; k.tau = p->tau; k.epsb = p->epsb;
    k.delta = p->delta; k.aniso = p->aniso; k.theta0 = p->theta0; k.alpha = p->alpha; k.gama = p->gama;
    k.teq = p->teq; k.pi = p->pi; k.kappa = p->kappa; k.noise = p->noise; k.seed = p->seed; k.step = step;
    return k;
}

GgAdj gg_args(const amps_params *p)
{
    GgAdj g;
    g.nx = p->nx; g.ny = p->ny; g.bc = p->bc; g.q = p->nfields; g.stencil = p->stencil;
    g.dxdy = p->dx * p->dy; g.dt = p->dt; g.mobil = p->mobil; g.grcoef = p->grcoef; g.gamma = p->gamma;
    return g;
}

int check(const amps_params *p, int dtype)
{
    if (!p || (dtype != AMPS_F64 && dtype != AMPS_F32) || p->nx < 5 || p->ny < 5) return AMPS_ERR_INVALID;
    if (p->model == AMPS_SINTERING) return AMPS_ERR_UNSUPPORTED;
    if (p->model == AMPS_GRAINGROWTH && (p->nfields < 1 || p->nfields > 32)) return AMPS_ERR_INVALID;
    if (p->bc != AMPS_BC_PERIODIC && p->bc != AMPS_BC_NOFLUX) return AMPS_ERR_INVALID;
    return AMPS_OK;
}

template <typename R>
int forward_t(const amps_params *p, const void *in, void *out, void *ws, int64_t step, cudaStream_t s)
{
    const int64_t n = (int64_t)p->nx * p->ny;
    const int grid = (int)((n + kAdjThreads - 1) / kAdjThreads);
    if (p->model == AMPS_KOBAYASHI) {
        const KobAdj k = kob_args(p, step);
        const R *phi = (const R *)in, *T = phi + n;
        R *w = (R *)ws;
        kob_inter_kernel<R><<<grid, kAdjThreads, 0, s>>>(k, phi, w);
        kob_update_kernel<R><<<grid, kAdjThreads, 0, s>>>(k, phi, T, w, (R *)out, (R *)out + n);
    } else {
        gg_fwd_kernel<R><<<grid, kAdjThreads, 0, s>>>(gg_args(p), (const R *)in, (R *)out);
    }
    return cudaGetLastError() == cudaSuccess ? AMPS_OK : AMPS_ERR_CUDA;
}

template <typename R>
int adjoint_t(const amps_params *p, const void *in, const void *gout, void *gin, double *gparams, void *ws,
              int64_t step, cudaStream_t s)
{
    const int64_t n = (int64_t)p->nx * p->ny;
    const int grid = (int)((n + kAdjThreads - 1) / kAdjThreads);
    if (p->model == AMPS_KOBAYASHI) {
        const KobAdj k = kob_args(p, step);
        const R *phi = (const R *)in, *T = phi + n;
        const R *gphi_out = (const R *)gout, *gT_out = gphi_out + n;
        R *w = (R *)ws, *mu = w + 5 * n, *v = mu + n;
        kob_inter_kernel<R><<<grid, kAdjThreads, 0, s>>>(k, phi, w);
        kob_mu_kernel<R><<<grid, kAdjThreads, 0, s>>>(k, gphi_out, gT_out, mu);
        kob_adj_inter_kernel<R><<<grid, kAdjThreads, 0, s>>>(k, w, mu, v, gparams);
        kob_adj_out_kernel<R><<<grid, kAdjThreads, 0, s>>>(k, phi, T, w, mu, v, gphi_out, gT_out, (R *)gin,
                                                             (R *)gin + n, gparams);
    } else {
        gg_adj_kernel<R><<<grid, kAdjThreads, 0, s>>>(gg_args(p), (const R *)in, (const R *)gout, (R *)gin, gparams);
    }
    return cudaGetLastError() == cudaSuccess ? AMPS_OK : AMPS_ERR_CUDA;
}

}  // namespace

extern "C" size_t amps_adjoint_workspace_bytes(const amps_params *p, int dtype)
{
    if (check(p, dtype) != AMPS_OK) return 0;
    const size_t n = (size_t)p->nx * p->ny, r = dtype == AMPS_F64 ? 8 : 4;
    return p->model == AMPS_KOBAYASHI ? 9 * n * r : 0;
}

extern "C" int amps_step_forward(const amps_params *p, int dtype, const void *state_in, void *state_out,
                                 void *workspace, int64_t step, void *stream)
{
    if (int r = check(p, dtype)) return r;
    if (!state_in || !state_out || state_in == state_out || (p->model == AMPS_KOBAYASHI && !workspace))
        return AMPS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    return dtype == AMPS_F64 ? forward_t<double>(p, state_in, state_out, workspace, step, s)
                             : forward_t<float>(p, state_in, state_out, workspace, step, s);
}

extern "C" int amps_step_adjoint(const amps_params *p, int dtype, const void *state_in, const void *grad_out,
                                 void *grad_in, double *grad_params, void *workspace, int64_t step, void *stream)
{
    if (int r = check(p, dtype)) return r;
    if (!state_in || !grad_out || !grad_in || !grad_params || grad_in == grad_out ||
        (p->model == AMPS_KOBAYASHI && !workspace))
        return AMPS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    return dtype == AMPS_F64 ? adjoint_t<double>(p, state_in, grad_out, grad_in, grad_params, workspace, step, s)
                             : adjoint_t<float>(p, state_in, grad_out, grad_in, grad_params, workspace, step, s);
}
