// k_adjoint.cu -- explicit time step, its hand-written adjoint, and a
// checkpointed rollout for the Kobayashi dendrite and grain growth, on
// row-major device arrays (float or double).  No reference counterpart (the
// reference is forward-only); the step restated is snowflake/function.h:5-60
// and graingrowth/function.h:5-30.
//
// Kobayashi step, per cell (periodic or zero-flux neighbour map M):
//   px = (phi[M(x+1)] - phi[M(x-1)]) / 2dx,  py likewise,  a = aniso*(atan2(py,px) - theta0)
//   eps = epsb*(1 + delta*cos a),  epd = -epsb*aniso*delta*sin a
//   lap = (sum of phi at the 8 radius-2 cross neighbours - 8 phi) / dxdy
//   term1 = ((eps*epd*px)[M(y+1)] - (eps*epd*px)[M(y-1)]) / 2dy
//   term2 = -((eps*epd*py)[M(x+1)] - (eps*epd*py)[M(x-1)]) / 2dx
//   m = alpha/pi*atan(gama*(teq - T)),  g = phi*(1-phi)*(phi - 1/2 + m + noise*chi)
//   phi' = phi + dt/tau*(term1 + term2 + eps^2*lap + g),  T' = T + dt*lapT + K*(phi' - phi)
// The adjoint maps output cotangents (gphi', gT') to input cotangents and adds
// dL/d(delta, K, epsb) into a device double[3].  Each step is ONE fused
// kernel: a CTA stages its tile plus halo (radius 2 forward, 3 adjoint) in
// shared memory, computes the intermediates there, and applies the stencil
// transposes from shared memory.  A transpose gathers over every preimage of
// the neighbour map, so zero-flux (mirror) boundaries are differentiated
// exactly: intermediate cotangents are zero outside the domain and the
// mirrored preimages of a boundary cell are added explicitly.
//
// Grain growth: eta_k' = eta_k - dt*L*(dfd_k - kappa*lap eta_k),
//   dfd_k = eta_k*(eta_k^2 - 1 + 2*gamma*(S - eta_k^2)),  S = sum_j eta_j^2;
// gradients w.r.t. (L, kappa, gamma).
//
// Parameter values and the noise step origin can come from device memory
// (ParamSrc), so a captured CUDA graph of a whole rollout stays valid when
// they change between calls.
#include "../../include/amps.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <new>
#include <vector>

namespace {

constexpr int kAdjThreads = 256;
constexpr int kMaxAdjSmem = 226 * 1024;  // dynamic shared memory opt-in limit

struct KobAdj {
    int nx, ny, bc;
    double dx, dy, dxdy, dt, tau, aniso, theta0, alpha, gama, teq, pi, noise;
    uint64_t seed;
};

struct GgAdj {
    int nx, ny, bc, q, stencil;
    double dxdy, dt;
};

// The three differentiable parameters and the noise step index: by value,
// or (dev / dstep non-null) read from device memory at kernel start.
struct ParamSrc {
    double v[3];
    const double *dev;
    int64_t step;          // step index, or offset added to *dstep
    const int64_t *dstep;
};

__device__ __forceinline__ void load_params(const ParamSrc &s, double &a, double &b, double &c, int64_t &step)
{
    if (s.dev) {
        a = s.dev[0];
        b = s.dev[1];
        c = s.dev[2];
    } else {
        a = s.v[0];
        b = s.v[1];
        c = s.v[2];
    }
    step = s.dstep ? *s.dstep + s.step : s.step;
}

__device__ __forceinline__ int nbmap(int i, int n, int bc)
{
    if (bc == 0) return i < 0 ? i + n : (i >= n ? i - n : i);
    return i < 0 ? -i - 1 : (i >= n ? 2 * n - i - 1 : i);
}

// Cells j with M(j + k) = c along one axis of the zero-flux map (direct
// j = c - k, plus the mirrored preimages of a boundary cell); at most two.
__device__ __forceinline__ int preimages_noflux(int c, int k, int n, int *j)
{
    int m = 0;
    if (c - k >= 0 && c - k < n) j[m++] = c - k;
    if (-1 - c - k >= 0) j[m++] = -1 - c - k;
    if (2 * n - 1 - c - k < n) j[m++] = 2 * n - 1 - c - k;
    return m;
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

// A tile of TX x TY cells with a halo of H cells, row-major in shared memory.
template <int TX, int TY, int H> struct Reg {
    static constexpr int W = TX + 2 * H, HT = TY + 2 * H, N = W * HT;
};

// Sum over the preimages of cell (cx, cy) for offset (kx, ky) of a shared
// array holding a region with halo H around the tile at (x0, y0).  Periodic:
// the one preimage sits at region position c - k (the halo holds wrapped
// values).  Zero-flux: the array is zero outside the domain, so the direct
// term is the region value at c - k; mirrored preimages are added.
template <int TX, int TY, int H, typename R>
__device__ __forceinline__ R fold_s(const R *a, int x0, int y0, int cx, int cy, int kx, int ky, int nx, int ny,
                                    int bc)
{
    using G = Reg<TX, TY, H>;
    const int rx = cx - kx - x0 + H, ry = cy - ky - y0 + H;
    if (bc == 0 || (cx - kx >= 0 && cx - kx < nx && cy - ky >= 0 && cy - ky < ny &&
                    cx >= 2 && cx < nx - 2 && cy >= 2 && cy < ny - 2))
        return a[ry * G::W + rx];
    int jx[3], jy[3];
    const int mx = preimages_noflux(cx, kx, nx, jx), my = preimages_noflux(cy, ky, ny, jy);
    R s = R(0);
    for (int b = 0; b < my; ++b)
        for (int c = 0; c < mx; ++c) s += a[(jy[b] - y0 + H) * G::W + (jx[c] - x0 + H)];
    return s;
}

// ------------------------------------------------------------ Kobayashi ----
// Forward step.  Shared: phi, T over the halo-2 region; eps*epd*px,
// eps*epd*py and eps over the halo-1 region (at an out-of-domain zero-flux
// position: the values of the mirrored cell, as the map M looks them up).
template <typename R, int TX, int TY>
__global__ void __launch_bounds__(kAdjThreads) kob_fwd_kernel(KobAdj p, ParamSrc ps, const R *__restrict__ in,
                                                              R *__restrict__ out)
{
    using R2 = Reg<TX, TY, 2>;
    using R1 = Reg<TX, TY, 1>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *sphi = reinterpret_cast<R *>(smem_raw), *sT = sphi + R2::N;
    R *sP1 = sT + R2::N, *sP2 = sP1 + R1::N, *seps = sP2 + R1::N;
    double delta, kappa, epsb;
    int64_t step;
    load_params(ps, delta, kappa, epsb, step);
    const int nx = p.nx, ny = p.ny, bc = p.bc;
    const int64_t n = (int64_t)nx * ny;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const R *phi = in, *T = in + n;
    for (int u = threadIdx.x; u < R2::N; u += kAdjThreads) {
        const int gx = x0 - 2 + u % R2::W, gy = y0 - 2 + u / R2::W;
        R a = R(0), b = R(0);
        if (gx < nx + 2 && gy < ny + 2) {
            const int64_t j = (int64_t)nbmap(gy, ny, bc) * nx + nbmap(gx, nx, bc);
            a = phi[j];
            b = T[j];
        }
        sphi[u] = a;
        sT[u] = b;
    }
    __syncthreads();
    const R aniso = R(p.aniso), th0 = R(p.theta0);
    for (int u = threadIdx.x; u < R1::N; u += kAdjThreads) {
        int gx = x0 - 1 + u % R1::W, gy = y0 - 1 + u / R1::W;
        R P1 = R(0), P2 = R(0), e = R(0);
        if (gx <= nx && gy <= ny) {
            if (bc == 1) {
                gx = nbmap(gx, nx, 1);
                gy = nbmap(gy, ny, 1);
            }
            const int o = (gy - y0 + 2) * R2::W + (gx - x0 + 2);
            const R px = (sphi[o + 1] - sphi[o - 1]) * R(0.5 / p.dx);
            const R py = (sphi[o + R2::W] - sphi[o - R2::W]) * R(0.5 / p.dy);
            const R a = aniso * (atan2(py, px) - th0);
            e = R(epsb) * (R(1) + R(delta) * cos(a));
            const R ed = R(-epsb * p.aniso * delta) * sin(a);
            P1 = e * ed * px;
            P2 = e * ed * py;
        }
        sP1[u] = P1;
        sP2[u] = P2;
        seps[u] = e;
    }
    __syncthreads();
    const R dtt = R(p.dt / p.tau), inv = R(1.0 / p.dxdy);
    for (int u = threadIdx.x; u < TX * TY; u += kAdjThreads) {
        const int i = u % TX, jj = u / TX, gx = x0 + i, gy = y0 + jj;
        if (gx >= nx || gy >= ny) continue;
        const int o = (jj + 2) * R2::W + i + 2, o1 = (jj + 1) * R1::W + i + 1;
        constexpr int W = R2::W;
        const R ph = sphi[o], t0 = sT[o];
        const R sp = (sphi[o - 1] + sphi[o + 1]) + (sphi[o - 2] + sphi[o + 2]) + (sphi[o - W] + sphi[o + W]) +
                     (sphi[o - 2 * W] + sphi[o + 2 * W]);
        const R lap = (sp - R(8) * ph) * inv;
        const R st = (sT[o - 1] + sT[o + 1]) + (sT[o - 2] + sT[o + 2]) + (sT[o - W] + sT[o + W]) +
                     (sT[o - 2 * W] + sT[o + 2 * W]);
        const R lapT = (st - R(8) * t0) * inv;
        const R term1 = (sP1[o1 + R1::W] - sP1[o1 - R1::W]) * R(0.5 / p.dy);
        const R term2 = -(sP2[o1 + 1] - sP2[o1 - 1]) * R(0.5 / p.dx);
        const R m = R(p.alpha / p.pi) * atan(R(p.gama) * (R(p.teq) - t0));
        R drive = ph - R(0.5) + m;
        const int64_t g = (int64_t)gy * nx + gx;
        if (p.noise != 0.0) drive += R(p.noise) * (R(u01(p.seed, (uint64_t)step, (uint64_t)g)) - R(0.5));
        const R e = seps[o1];
        const R d = dtt * (term1 + term2 + e * e * lap + ph * (R(1) - ph) * drive);
        out[g] = ph + d;
        out[n + g] = t0 + R(p.dt) * lapT + R(kappa) * d;
    }
}

// Adjoint step.  Shared (halo 3 for phi, 2 for the rest, 1 for the
// anisotropy cotangents):
//   phi (R3); mu = gphi' + K gT' and gT' (R2, zero outside a zero-flux domain);
//   sin a, cos a, px, py (R2, at out-of-domain positions the mirrored cell's;
//   eps and epd are rebuilt from them exactly as the forward computes them);
//   Q = dt/tau*mu*eps^2/dxdy (R2, zero outside); lpx, lpy (R1, zero outside):
//   the cotangents of px, py including the path through theta = atan2(py, px).
template <typename R, int TX, int TY>
__global__ void __launch_bounds__(kAdjThreads)
    kob_adj_kernel(KobAdj p, ParamSrc ps, const R *__restrict__ in, const R *__restrict__ gout, R *__restrict__ gin,
                   double *__restrict__ gparams)
{
    using R3 = Reg<TX, TY, 3>;
    using R2 = Reg<TX, TY, 2>;
    using R1 = Reg<TX, TY, 1>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[kAdjThreads / 32];
    R *sphi = reinterpret_cast<R *>(smem_raw);
    R *smu = sphi + R3::N, *sgT = smu + R2::N, *ssa = sgT + R2::N, *sca = ssa + R2::N;
    R *spx = sca + R2::N, *spy = spx + R2::N, *sQ = spy + R2::N, *slpx = sQ + R2::N, *slpy = slpx + R1::N;
    double delta, kappa, epsb;
    int64_t step;
    load_params(ps, delta, kappa, epsb, step);
    const int nx = p.nx, ny = p.ny, bc = p.bc;
    const int64_t n = (int64_t)nx * ny;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const R *phi = in, *T = in + n, *gpo = gout, *gTo = gout + n;
    const R K = R(kappa);
    for (int u = threadIdx.x; u < R3::N; u += kAdjThreads) {
        const int gx = x0 - 3 + u % R3::W, gy = y0 - 3 + u / R3::W;
        sphi[u] = (gx < nx + 3 && gy < ny + 3) ? phi[(int64_t)nbmap(gy, ny, bc) * nx + nbmap(gx, nx, bc)] : R(0);
    }
    for (int u = threadIdx.x; u < R2::N; u += kAdjThreads) {
        const int gx = x0 - 2 + u % R2::W, gy = y0 - 2 + u / R2::W;
        const bool dom = gx >= 0 && gx < nx && gy >= 0 && gy < ny;
        R m = R(0), t = R(0);
        if (gx < nx + 2 && gy < ny + 2 && (bc == 0 || dom)) {
            const int64_t j = (int64_t)nbmap(gy, ny, bc) * nx + nbmap(gx, nx, bc);
            t = gTo[j];
            m = gpo[j] + K * t;
        }
        smu[u] = m;
        sgT[u] = t;
    }
    __syncthreads();
    const R aniso = R(p.aniso), th0 = R(p.theta0), dtt = R(p.dt / p.tau), inv = R(1.0 / p.dxdy);
    const R eb = R(epsb), dl = R(delta), ebd = R(-epsb * p.aniso * delta);
    auto EPS = [&](R ca) { return eb * (R(1) + dl * ca); };
    auto EPD = [&](R sa) { return ebd * sa; };
    // sin a, cos a, px, py and Q over R2
    for (int u = threadIdx.x; u < R2::N; u += kAdjThreads) {
        const int gx = x0 - 2 + u % R2::W, gy = y0 - 2 + u / R2::W;
        R sa = R(0), ca = R(0), px = R(0), py = R(0), q = R(0);
        if (gx <= nx + 1 && gy <= ny + 1) {
            const bool dom = gx >= 0 && gx < nx && gy >= 0 && gy < ny;
            const int sx = bc == 1 ? nbmap(gx, nx, 1) : gx, sy = bc == 1 ? nbmap(gy, ny, 1) : gy;
            const int o = (sy - y0 + 3) * R3::W + (sx - x0 + 3);
            px = (sphi[o + 1] - sphi[o - 1]) * R(0.5 / p.dx);
            py = (sphi[o + R3::W] - sphi[o - R3::W]) * R(0.5 / p.dy);
            const R a = aniso * (atan2(py, px) - th0);
            sa = sin(a);
            ca = cos(a);
            const R e = EPS(ca);
            if (bc == 0 || dom) q = dtt * smu[u] * e * e * inv;
        }
        ssa[u] = sa;
        sca[u] = ca;
        spx[u] = px;
        spy[u] = py;
        sQ[u] = q;
    }
    __syncthreads();
    // anisotropy cotangents over R1; parameter gradients of the tile's own cells
    R gd = R(0), ge = R(0), gk = R(0);
    for (int u = threadIdx.x; u < R1::N; u += kAdjThreads) {
        const int rx = u % R1::W, ry = u / R1::W, gx = x0 - 1 + rx, gy = y0 - 1 + ry;
        const bool dom = gx >= 0 && gx < nx && gy >= 0 && gy < ny;
        R lpx = R(0), lpy = R(0);
        if (gx <= nx && gy <= ny && (bc == 0 || dom)) {
            const int o3 = (ry + 2) * R3::W + rx + 2, o2 = (ry + 1) * R2::W + rx + 1;
            constexpr int W = R3::W;
            const R sp = (sphi[o3 - 1] + sphi[o3 + 1]) + (sphi[o3 - 2] + sphi[o3 + 2]) + (sphi[o3 - W] + sphi[o3 + W]) +
                         (sphi[o3 - 2 * W] + sphi[o3 + 2 * W]);
            const R lap = (sp - R(8) * sphi[o3]) * inv;
            const R A = dtt * R(0.5 / p.dy) *
                        (fold_s<TX, TY, 2>(smu, x0, y0, gx, gy, 0, 1, nx, ny, bc) -
                         fold_s<TX, TY, 2>(smu, x0, y0, gx, gy, 0, -1, nx, ny, bc));
            const R B = dtt * R(0.5 / p.dx) *
                        (fold_s<TX, TY, 2>(smu, x0, y0, gx, gy, -1, 0, nx, ny, bc) -
                         fold_s<TX, TY, 2>(smu, x0, y0, gx, gy, 1, 0, nx, ny, bc));
            const R C = dtt * smu[o2] * lap;
            const R sa = ssa[o2], ca = sca[o2], px = spx[o2], py = spy[o2];
            const R e = EPS(ca), ed = EPD(sa);
            const R le = A * ed * px + B * ed * py + R(2) * C * e;
            const R led = A * e * px + B * e * py;
            lpx = A * e * ed;
            lpy = B * e * ed;
            const R la = le * R(-epsb * delta) * sa + led * R(-epsb * p.aniso * delta) * ca;
            const R lth = aniso * la;
            const R r2 = px * px + py * py;
            if (r2 > R(0)) {  // atan2 has no derivative where the gradient vanishes
                lpx += lth * (-py / r2);
                lpy += lth * (px / r2);
            }
            if (rx >= 1 && rx <= TX && ry >= 1 && ry <= TY && gx < nx && gy < ny) {
                gd += le * R(epsb) * ca + led * R(-epsb * p.aniso) * sa;
                ge += le * (R(1) + R(delta) * ca) + led * R(-p.aniso * delta) * sa;
            }
        }
        slpx[u] = lpx;
        slpy[u] = lpy;
    }
    __syncthreads();
    for (int u = threadIdx.x; u < TX * TY; u += kAdjThreads) {
        const int i = u % TX, jj = u / TX, gx = x0 + i, gy = y0 + jj;
        if (gx >= nx || gy >= ny) continue;
        const int o3 = (jj + 3) * R3::W + i + 3, o2 = (jj + 2) * R2::W + i + 2;
        constexpr int W = R3::W;
        // transposes: radius-2 cross of Q (eps^2 lap phi) and of gT' (lap T)
        R lq = -R(8) * sQ[o2], lt = -R(8) * sgT[o2];
        const int off[4] = {-2, -1, 1, 2};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            lq += fold_s<TX, TY, 2>(sQ, x0, y0, gx, gy, off[k], 0, nx, ny, bc) +
                  fold_s<TX, TY, 2>(sQ, x0, y0, gx, gy, 0, off[k], nx, ny, bc);
            lt += fold_s<TX, TY, 2>(sgT, x0, y0, gx, gy, off[k], 0, nx, ny, bc) +
                  fold_s<TX, TY, 2>(sgT, x0, y0, gx, gy, 0, off[k], nx, ny, bc);
        }
        const R dpx = (fold_s<TX, TY, 1>(slpx, x0, y0, gx, gy, 1, 0, nx, ny, bc) -
                       fold_s<TX, TY, 1>(slpx, x0, y0, gx, gy, -1, 0, nx, ny, bc)) *
                      R(0.5 / p.dx);
        const R dpy = (fold_s<TX, TY, 1>(slpy, x0, y0, gx, gy, 0, 1, nx, ny, bc) -
                       fold_s<TX, TY, 1>(slpy, x0, y0, gx, gy, 0, -1, nx, ny, bc)) *
                      R(0.5 / p.dy);
        // the forward increment d = phi' - phi at this cell (for dL/dK)
        auto P1 = [&](int o) { return EPS(sca[o]) * EPD(ssa[o]) * spx[o]; };
        auto P2 = [&](int o) { return EPS(sca[o]) * EPD(ssa[o]) * spy[o]; };
        const R term1 = (P1(o2 + R2::W) - P1(o2 - R2::W)) * R(0.5 / p.dy);
        const R term2 = -(P2(o2 + 1) - P2(o2 - 1)) * R(0.5 / p.dx);
        const R ph = sphi[o3];
        const R sp = (sphi[o3 - 1] + sphi[o3 + 1]) + (sphi[o3 - 2] + sphi[o3 + 2]) + (sphi[o3 - W] + sphi[o3 + W]) +
                     (sphi[o3 - 2 * W] + sphi[o3 + 2 * W]);
        const R lap = (sp - R(8) * ph) * inv;
        const int64_t g = (int64_t)gy * nx + gx;
        const R t0 = T[g];
        const R m = R(p.alpha / p.pi) * atan(R(p.gama) * (R(p.teq) - t0));
        R drive = ph - R(0.5) + m;
        if (p.noise != 0.0) drive += R(p.noise) * (R(u01(p.seed, (uint64_t)step, (uint64_t)g)) - R(0.5));
        const R e = EPS(sca[o2]);
        const R d = dtt * (term1 + term2 + e * e * lap + ph * (R(1) - ph) * drive);
        const R mu = smu[o2];
        const R dg = (R(1) - R(2) * ph) * drive + ph * (R(1) - ph);
        gin[g] = gpo[g] + dtt * mu * dg + lq + dpx + dpy;
        const R z = R(p.gama) * (R(p.teq) - t0);
        const R dm = R(p.alpha / p.pi) * (-R(p.gama)) / (R(1) + z * z);
        gin[n + g] = gTo[g] + R(p.dt * inv) * lt + dtt * mu * ph * (R(1) - ph) * dm;
        gk += gTo[g] * d;
    }
    const double sd = block_sum(gd, red);
    const double sk = block_sum(gk, red);
    const double se = block_sum(ge, red);
    if (threadIdx.x == 0) {
        atomicAdd(&gparams[0], sd);
        atomicAdd(&gparams[1], sk);
        atomicAdd(&gparams[2], se);
    }
}

// --------------------------------------------------------- grain growth ----
// One cell per thread on a kGX x kGY tile; every field of the tile plus a
// halo of one staged in shared memory (field-major).
constexpr int kGX = 32, kGY = 8;
using GReg = Reg<kGX, kGY, 1>;

// One element from global to shared memory by an asynchronous copy (the
// copies of all rows stay in flight until gg_stage_wait).
template <typename R> __device__ __forceinline__ void cp_elem(R *d, const R *g)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(d);
    if constexpr (sizeof(R) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(g) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(g) : "memory");
}

__device__ __forceinline__ void gg_stage_wait()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Stage q fields of f (row-major [q][n]) over the halo-1 region, one warp
// per region row (a coalesced copy of the row's kGX interior cells, two
// lanes for its halo cells); complete after gg_stage_wait.  zero_out:
// zero-flux cotangents are zero outside the domain (the transpose adds the
// mirrored preimages itself).
template <typename R>
__device__ __forceinline__ void gg_stage(R *s, const R *f, int q, int x0, int y0, const GgAdj &p, bool zero_out)
{
    static_assert(kGX == 32, "one lane per interior column");
    const int64_t n = (int64_t)p.nx * p.ny;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool zf = zero_out && p.bc == 1;
    for (int rr = warp; rr < q * GReg::HT; rr += kAdjThreads / 32) {
        const int k = rr / GReg::HT, ry = rr - k * GReg::HT;
        const int gy = y0 - 1 + ry;
        const bool rowok = gy <= p.ny && !(zf && (gy < 0 || gy >= p.ny));
        const R *row = f + k * n + (int64_t)(rowok ? nbmap(gy, p.ny, p.bc) : 0) * p.nx;
        R *dst = s + k * GReg::N + ry * GReg::W;
        const int gx = x0 + lane;
        if (rowok && gx <= p.nx && !(zf && gx >= p.nx))
            cp_elem(dst + 1 + lane, row + nbmap(gx, p.nx, p.bc));
        else
            dst[1 + lane] = R(0);
        if (lane < 2) {
            const int hx = lane == 0 ? x0 - 1 : x0 + kGX;
            R *d = dst + (lane == 0 ? 0 : GReg::W - 1);
            if (rowok && hx <= p.nx && !(zf && (hx < 0 || hx >= p.nx)))
                cp_elem(d, row + nbmap(hx, p.nx, p.bc));
            else
                *d = R(0);
        }
    }
}

// 8-neighbour (graingrowth/function.h:20) or 5-point Laplacian at region offset o, / dxdy
template <typename R> __device__ __forceinline__ R gg_lap_s(const R *s, int o, int stencil, R inv)
{
    constexpr int W = GReg::W;
    R v;
    if (stencil == 0)
        v = s[o - W - 1] + s[o - W] + s[o - W + 1] + s[o - 1] + s[o + 1] + s[o + W - 1] + s[o + W] + s[o + W + 1] -
            R(8) * s[o];
    else
        v = s[o - 1] + s[o + 1] + s[o - W] + s[o + W] - R(4) * s[o];
    return v * inv;
}

// transpose of gg_lap_s at cell (gx, gy) (exact for both boundary maps)
template <typename R>
__device__ __forceinline__ R gg_lap_t_s(const R *s, int o, int x0, int y0, int gx, int gy, const GgAdj &p, R inv)
{
    // the stencil is symmetric: where no mirrored preimage exists (periodic
    // grids, and cells off a zero-flux edge) its transpose is itself
    if (p.bc == 0 || (gx >= 1 && gx < p.nx - 1 && gy >= 1 && gy < p.ny - 1)) return gg_lap_s(s, o, p.stencil, inv);
    R v;
    if (p.stencil == 0) {
        v = -R(8) * s[o];
        for (int ky = -1; ky <= 1; ++ky)
            for (int kx = -1; kx <= 1; ++kx)
                if (kx || ky) v += fold_s<kGX, kGY, 1>(s, x0, y0, gx, gy, kx, ky, p.nx, p.ny, p.bc);
    } else {
        v = fold_s<kGX, kGY, 1>(s, x0, y0, gx, gy, -1, 0, p.nx, p.ny, p.bc) +
            fold_s<kGX, kGY, 1>(s, x0, y0, gx, gy, 1, 0, p.nx, p.ny, p.bc) +
            fold_s<kGX, kGY, 1>(s, x0, y0, gx, gy, 0, -1, p.nx, p.ny, p.bc) +
            fold_s<kGX, kGY, 1>(s, x0, y0, gx, gy, 0, 1, p.nx, p.ny, p.bc) - R(4) * s[o];
    }
    return v * inv;
}

template <typename R>
__global__ void __launch_bounds__(kAdjThreads) gg_fwd_kernel(GgAdj p, ParamSrc ps, const R *__restrict__ eta,
                                                             R *__restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *se = reinterpret_cast<R *>(smem_raw);
    double mobil, grcoef, gamma;
    int64_t step;
    load_params(ps, mobil, grcoef, gamma, step);
    const int x0 = blockIdx.x * kGX, y0 = blockIdx.y * kGY;
    gg_stage(se, eta, p.q, x0, y0, p, false);
    gg_stage_wait();
    __syncthreads();
    const int i = threadIdx.x % kGX, j = threadIdx.x / kGX, gx = x0 + i, gy = y0 + j;
    if (gx >= p.nx || gy >= p.ny) return;
    const int64_t n = (int64_t)p.nx * p.ny, g = (int64_t)gy * p.nx + gx;
    const int o = (j + 1) * GReg::W + i + 1;
    R S = R(0);
    for (int k = 0; k < p.q; ++k) S += se[k * GReg::N + o] * se[k * GReg::N + o];
    const R dtm = R(p.dt * mobil), g2 = R(2.0 * gamma), kap = R(grcoef), inv = R(1.0 / p.dxdy);
    for (int k = 0; k < p.q; ++k) {
        const R *sk = se + k * GReg::N;
        const R e = sk[o], e2 = e * e;
        const R dfd = e * (e2 - R(1) + g2 * (S - e2));
        out[k * n + g] = e - dtm * (dfd - kap * gg_lap_s(sk, o, p.stencil, inv));
    }
}

// input cotangents of all q fields; adds dL/d(L, kappa, gamma) into gparams
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) gg_adj_kernel(GgAdj p, ParamSrc ps, const R *__restrict__ eta,
                                                             const R *__restrict__ gout, R *__restrict__ gin,
                                                             double *__restrict__ gparams)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[kAdjThreads / 32];
    R *se = reinterpret_cast<R *>(smem_raw), *sg = se + p.q * GReg::N;
    double mobil, grcoef, gamma;
    int64_t step;
    load_params(ps, mobil, grcoef, gamma, step);
    const int x0 = blockIdx.x * kGX, y0 = blockIdx.y * kGY;
    gg_stage(se, eta, p.q, x0, y0, p, false);
    gg_stage(sg, gout, p.q, x0, y0, p, true);
    gg_stage_wait();
    __syncthreads();
    const int i = threadIdx.x % kGX, j = threadIdx.x / kGX, gx = x0 + i, gy = y0 + j;
    R gl = R(0), gkap = R(0), ggam = R(0);
    if (gx < p.nx && gy < p.ny) {
        const int64_t n = (int64_t)p.nx * p.ny, g = (int64_t)gy * p.nx + gx;
        const int o = (j + 1) * GReg::W + i + 1;
        R S = R(0), P = R(0);
        for (int k = 0; k < p.q; ++k) {
            const R e = se[k * GReg::N + o];
            S += e * e;
            P += sg[k * GReg::N + o] * e;
        }
        const R dt = R(p.dt), dtm = R(p.dt * mobil), gm = R(gamma), kap = R(grcoef), inv = R(1.0 / p.dxdy);
        for (int k = 0; k < p.q; ++k) {
            const R *ek = se + k * GReg::N, *gk_s = sg + k * GReg::N;
            const R e = ek[o], e2 = e * e, gk = gk_s[o];
            const R jac = R(3) * e2 - R(1) + R(2) * gm * (S - e2);  // d dfd_k / d eta_k
            gin[k * n + g] = gk - dtm * (gk * jac + R(4) * gm * e * (P - gk * e)) +
                             dtm * kap * gg_lap_t_s(gk_s, o, x0, y0, gx, gy, p, inv);
            const R lap = gg_lap_s(ek, o, p.stencil, inv);
            const R dfd = e * (e2 - R(1) + R(2) * gm * (S - e2));
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

// ---- grain growth, periodic grids, 32x32 tiles ----------------------------
// The forward step and its adjoint for periodic grids whose sides are
// multiples of 32 (the Laplacian is then its own transpose): every field of a
// 32x32 tile plus its halo staged by asynchronous copies in a 16-byte-aligned
// row layout, the per-cell sums (S = sum e^2; the adjoint's P = sum g e)
// formed once into shared tiles, then each warp advances one field at a
// time, a lane sweeping 8 rows x 4 cells with a 3-row register window (the
// grain-growth step kernel's layout).  The neighbour sums keep gg_lap_s's
// left-to-right order, so the forward results are gg_fwd_kernel's.
constexpr int kG32Rows = 8;  // rows per lane

template <typename R> struct G32 {
    static constexpr int T = 32, O = 16 / (int)sizeof(R) >= 1 ? 16 / (int)sizeof(R) : 1;
    static constexpr int P = T + 2 * O, ROWS = T + 2, FIELD = ROWS * P;
    static size_t smem(int nfields, int sums) { return sizeof(R) * ((size_t)nfields * FIELD + (size_t)sums * T * T); }
};

// Stage q fields (periodic) of tile (tx, ty): one warp per staged row.
template <typename R>
__device__ __forceinline__ void gg_stage32(R *s, const R *f, int q, int tx, int ty, const GgAdj &p)
{
    using L = G32<R>;
    const int64_t n = (int64_t)p.nx * p.ny;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x0 = tx * L::T;
    for (int rr = warp; rr < q * L::ROWS; rr += kAdjThreads / 32) {
        const int k = rr / L::ROWS, ry = rr - k * L::ROWS;
        int gy = ty * L::T - 1 + ry;
        gy = gy < 0 ? gy + p.ny : (gy >= p.ny ? gy - p.ny : gy);
        const R *row = f + k * n + (int64_t)gy * p.nx;
        R *dst = s + k * L::FIELD + ry * L::P + L::O;
        cp_elem(dst + lane, row + x0 + lane);
        if (lane < 2) {
            int hx = lane == 0 ? x0 - 1 : x0 + L::T;
            hx = hx < 0 ? hx + p.nx : (hx >= p.nx ? hx - p.nx : hx);
            cp_elem(dst + (lane == 0 ? -1 : L::T), row + hx);
        }
    }
}

// Cells [c-1, c+4] of one staged row into w[0..5].
template <typename R> __device__ __forceinline__ void ld_row6r(const R *p, R *w)
{
    if constexpr (sizeof(R) == 4) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        w[1] = v.x; w[2] = v.y; w[3] = v.z; w[4] = v.w;
    } else {
        const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
        w[1] = a.x; w[2] = a.y; w[3] = b.x; w[4] = b.y;
    }
    w[0] = p[-1];
    w[5] = p[4];
}

// gg_lap_s's neighbour sum, from the window rows up / md / dn around column k+1
template <typename R> __device__ __forceinline__ R lap_w(const R *up, const R *md, const R *dn, int k, int stencil, R inv)
{
    R v;
    if (stencil == 0)
        v = up[k] + up[k + 1] + up[k + 2] + md[k] + md[k + 2] + dn[k] + dn[k + 1] + dn[k + 2] - R(8) * md[k + 1];
    else
        v = md[k] + md[k + 2] + up[k + 1] + dn[k + 1] - R(4) * md[k + 1];
    return v * inv;
}

template <typename R>
__global__ void __launch_bounds__(kAdjThreads) gg_fwd32_kernel(GgAdj p, ParamSrc ps, const R *__restrict__ eta,
                                                               R *__restrict__ out)
{
    using L = G32<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *se = reinterpret_cast<R *>(smem_raw), *sS = se + p.q * L::FIELD;
    double mobil, grcoef, gamma;
    int64_t step;
    load_params(ps, mobil, grcoef, gamma, step);
    const int ntx = p.nx / L::T, tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
    gg_stage32(se, eta, p.q, tx, ty, p);
    gg_stage_wait();
    __syncthreads();
    {
        const int row = threadIdx.x / 8, c = (threadIdx.x % 8) * 4;
        R acc[4] = {R(0), R(0), R(0), R(0)};
        for (int k = 0; k < p.q; ++k) {
            const R *q = se + k * L::FIELD + (row + 1) * L::P + L::O + c;
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] += q[j] * q[j];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) sS[row * L::T + c + j] = acc[j];
    }
    __syncthreads();
    const int64_t n = (int64_t)p.nx * p.ny;
    const R dtm = R(p.dt * mobil), g2 = R(2.0 * gamma), kap = R(grcoef), inv = R(1.0 / p.dxdy);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = (lane & 7) * 4, r0 = (lane >> 3) * kG32Rows;
    const int64_t gbase = (int64_t)(ty * L::T + r0) * p.nx + tx * L::T + c0;
    for (int f = warp; f < p.q; f += kAdjThreads / 32) {
        const R *fs = se + f * L::FIELD + L::O + c0;
        R w[3][6];
        ld_row6r(fs + r0 * L::P, w[0]);
        ld_row6r(fs + (r0 + 1) * L::P, w[1]);
#pragma unroll
        for (int i = 0; i < kG32Rows; ++i) {
            const R *up = w[i % 3], *md = w[(i + 1) % 3];
            R *dn = w[(i + 2) % 3];
            ld_row6r(fs + (r0 + i + 2) * L::P, dn);
            R o4[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const R e = md[k + 1], e2 = e * e, S = sS[(r0 + i) * L::T + c0 + k];
                const R dfd = e * (e2 - R(1) + g2 * (S - e2));
                o4[k] = e - dtm * (dfd - kap * lap_w(up, md, dn, k, p.stencil, inv));
            }
            R *dst = out + f * n + gbase + (int64_t)i * p.nx;
#pragma unroll
            for (int k = 0; k < 4; ++k) dst[k] = o4[k];
        }
    }
}

// Input cotangents of all q fields and dL/d(L, kappa, gamma) into gparams
// (gg_adj_kernel's arithmetic; the parameter sums are grouped differently).
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) gg_adj32_kernel(GgAdj p, ParamSrc ps, const R *__restrict__ eta,
                                                               const R *__restrict__ gout, R *__restrict__ gin,
                                                               double *__restrict__ gparams)
{
    using L = G32<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[kAdjThreads / 32];
    R *se = reinterpret_cast<R *>(smem_raw), *sg = se + p.q * L::FIELD;
    R *sS = sg + p.q * L::FIELD, *sP = sS + L::T * L::T;
    double mobil, grcoef, gamma;
    int64_t step;
    load_params(ps, mobil, grcoef, gamma, step);
    const int ntx = p.nx / L::T, tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
    gg_stage32(se, eta, p.q, tx, ty, p);
    gg_stage32(sg, gout, p.q, tx, ty, p);
    gg_stage_wait();
    __syncthreads();
    {
        const int row = threadIdx.x / 8, c = (threadIdx.x % 8) * 4;
        R S[4] = {R(0), R(0), R(0), R(0)}, P[4] = {R(0), R(0), R(0), R(0)};
        for (int k = 0; k < p.q; ++k) {
            const int o = k * L::FIELD + (row + 1) * L::P + L::O + c;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const R e = se[o + j];
                S[j] += e * e;
                P[j] += sg[o + j] * e;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sS[row * L::T + c + j] = S[j];
            sP[row * L::T + c + j] = P[j];
        }
    }
    __syncthreads();
    const int64_t n = (int64_t)p.nx * p.ny;
    const R dt = R(p.dt), dtm = R(p.dt * mobil), gm = R(gamma), kap = R(grcoef), inv = R(1.0 / p.dxdy);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = (lane & 7) * 4, r0 = (lane >> 3) * kG32Rows;
    const int64_t gbase = (int64_t)(ty * L::T + r0) * p.nx + tx * L::T + c0;
    R gl = R(0), gkap = R(0), ggam = R(0);
    for (int f = warp; f < p.q; f += kAdjThreads / 32) {
        const R *fe = se + f * L::FIELD + L::O + c0, *fg = sg + f * L::FIELD + L::O + c0;
        R we[3][6], wg[3][6];
        ld_row6r(fe + r0 * L::P, we[0]);
        ld_row6r(fe + (r0 + 1) * L::P, we[1]);
        ld_row6r(fg + r0 * L::P, wg[0]);
        ld_row6r(fg + (r0 + 1) * L::P, wg[1]);
#pragma unroll
        for (int i = 0; i < kG32Rows; ++i) {
            const R *eu = we[i % 3], *em = we[(i + 1) % 3], *gu = wg[i % 3], *gmr = wg[(i + 1) % 3];
            R *ed = we[(i + 2) % 3], *gd = wg[(i + 2) % 3];
            ld_row6r(fe + (r0 + i + 2) * L::P, ed);
            ld_row6r(fg + (r0 + i + 2) * L::P, gd);
            R o4[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int so = (r0 + i) * L::T + c0 + k;
                const R S = sS[so], P = sP[so];
                const R e = em[k + 1], e2 = e * e, gk = gmr[k + 1];
                const R jac = R(3) * e2 - R(1) + R(2) * gm * (S - e2);  // d dfd_k / d eta_k
                o4[k] = gk - dtm * (gk * jac + R(4) * gm * e * (P - gk * e)) +
                        dtm * kap * lap_w(gu, gmr, gd, k, p.stencil, inv);
                const R lap = lap_w(eu, em, ed, k, p.stencil, inv);
                const R dfd = e * (e2 - R(1) + R(2) * gm * (S - e2));
                gl += gk * (-dt) * (dfd - kap * lap);
                gkap += gk * dtm * lap;
                ggam += gk * (-dtm) * R(2) * e * (S - e2);
            }
            R *dst = gin + f * n + gbase + (int64_t)i * p.nx;
#pragma unroll
            for (int k = 0; k < 4; ++k) dst[k] = o4[k];
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

// The 32x32 periodic path applies (and its staging fits in shared memory)?
template <typename R> bool gg_use32(const amps_params *p, int sums)
{
    return p->bc == AMPS_BC_PERIODIC && p->nx % 32 == 0 && p->ny % 32 == 0 &&
           G32<R>::smem(sums == 2 ? 2 * p->nfields : p->nfields, sums) <= (size_t)kMaxAdjSmem;
}

// ------------------------------------------------------------- launches ----
constexpr int kTX = 32;

template <typename R, int TY> constexpr size_t kob_fwd_smem()
{
    return (2 * Reg<kTX, TY, 2>::N + 3 * Reg<kTX, TY, 1>::N) * sizeof(R);
}
template <typename R, int TY> constexpr size_t kob_adj_smem()
{
    return (Reg<kTX, TY, 3>::N + 7 * Reg<kTX, TY, 2>::N + 2 * Reg<kTX, TY, 1>::N) * sizeof(R);
}

// 32x16 tiles, or 32x8 where that leaves fewer than two CTAs per SM.
bool small_tiles(int nx, int ny) { return (int64_t)((nx + 31) / 32) * ((ny + 15) / 16) < 2 * 152; }

// Largest dynamic shared memory of any launch (grain growth with 32 fields
// in double: 2 * 32 * 340 * 8 = 174 KB).
template <typename R> cudaError_t kob_prepare()
{
    const cudaFuncAttribute attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(kob_adj_kernel<R, kTX, 16>, attr, (int)kob_adj_smem<R, 16>());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kob_adj_kernel<R, kTX, 8>, attr, (int)kob_adj_smem<R, 8>());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_fwd_kernel<R>, attr, (int)(32 * GReg::N * sizeof(R)));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_adj_kernel<R>, attr, (int)(2 * 32 * GReg::N * sizeof(R)));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_fwd32_kernel<R>, attr, kMaxAdjSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_adj32_kernel<R>, attr, kMaxAdjSmem);
    return e;
}

KobAdj kob_args(const amps_params *p)
{
    KobAdj k;
    k.nx = p->nx; k.ny = p->ny; k.bc = p->bc;
    k.dx = p->dx; k.dy = p->dy; k.dxdy = p->dx * p->dy; k.dt = p->dt; k.tau = p->tau;
    k.aniso = p->aniso; k.theta0 = p->theta0; k.alpha = p->alpha; k.gama = p->gama;
    k.teq = p->teq; k.pi = p->pi; k.noise = p->noise; k.seed = p->seed;
    return k;
}

GgAdj gg_args(const amps_params *p)
{
    GgAdj g;
    g.nx = p->nx; g.ny = p->ny; g.bc = p->bc; g.q = p->nfields; g.stencil = p->stencil;
    g.dxdy = p->dx * p->dy; g.dt = p->dt;
    return g;
}

ParamSrc param_src(const amps_params *p, int64_t step)
{
    ParamSrc s;
    if (p->model == AMPS_KOBAYASHI) {
        s.v[0] = p->delta; s.v[1] = p->kappa; s.v[2] = p->epsb;
    } else {
        s.v[0] = p->mobil; s.v[1] = p->grcoef; s.v[2] = p->gamma;
    }
    s.dev = nullptr; s.step = step; s.dstep = nullptr;
    return s;
}

int check(const amps_params *p, int dtype)
{
    if (!p || (dtype != AMPS_F64 && dtype != AMPS_F32) || p->nx < 5 || p->ny < 5) return AMPS_ERR_INVALID;
    if (p->model == AMPS_SINTERING) return AMPS_ERR_UNSUPPORTED;
    if (p->model != AMPS_KOBAYASHI && p->model != AMPS_GRAINGROWTH) return AMPS_ERR_INVALID;
    if (p->model == AMPS_GRAINGROWTH && (p->nfields < 1 || p->nfields > 32)) return AMPS_ERR_INVALID;
    if (p->bc != AMPS_BC_PERIODIC && p->bc != AMPS_BC_NOFLUX) return AMPS_ERR_INVALID;
    if (p->model == AMPS_KOBAYASHI && (p->tau == 0.0 || p->pi == 0.0 || p->dx == 0.0 || p->dy == 0.0))
        return AMPS_ERR_INVALID;
    return AMPS_OK;
}

int64_t state_elems(const amps_params *p)
{
    return (int64_t)p->nx * p->ny * (p->model == AMPS_KOBAYASHI ? 2 : p->nfields);
}

template <typename R>
void launch_forward(const amps_params *p, const ParamSrc &ps, const void *in, void *out, cudaStream_t s)
{
    const int nx = p->nx, ny = p->ny;
    if (p->model == AMPS_KOBAYASHI) {
        if (small_tiles(nx, ny)) {
            const dim3 grid((nx + kTX - 1) / kTX, (ny + 7) / 8);
            kob_fwd_kernel<R, kTX, 8><<<grid, kAdjThreads, kob_fwd_smem<R, 8>(), s>>>(kob_args(p), ps, (const R *)in,
                                                                                      (R *)out);
        } else {
            const dim3 grid((nx + kTX - 1) / kTX, (ny + 15) / 16);
            kob_fwd_kernel<R, kTX, 16><<<grid, kAdjThreads, kob_fwd_smem<R, 16>(), s>>>(kob_args(p), ps,
                                                                                        (const R *)in, (R *)out);
        }
    } else if (gg_use32<R>(p, 1)) {
        gg_fwd32_kernel<R><<<(nx / 32) * (ny / 32), kAdjThreads, G32<R>::smem(p->nfields, 1), s>>>(
            gg_args(p), ps, (const R *)in, (R *)out);
    } else {
        const dim3 grid((nx + kGX - 1) / kGX, (ny + kGY - 1) / kGY);
        gg_fwd_kernel<R><<<grid, kAdjThreads, (size_t)p->nfields * GReg::N * sizeof(R), s>>>(gg_args(p), ps,
                                                                                            (const R *)in, (R *)out);
    }
}

template <typename R>
void launch_adjoint(const amps_params *p, const ParamSrc &ps, const void *in, const void *gout, void *gin,
                    double *gparams, cudaStream_t s)
{
    const int nx = p->nx, ny = p->ny;
    if (p->model == AMPS_KOBAYASHI) {
        if (small_tiles(nx, ny)) {
            const dim3 grid((nx + kTX - 1) / kTX, (ny + 7) / 8);
            kob_adj_kernel<R, kTX, 8><<<grid, kAdjThreads, kob_adj_smem<R, 8>(), s>>>(
                kob_args(p), ps, (const R *)in, (const R *)gout, (R *)gin, gparams);
        } else {
            const dim3 grid((nx + kTX - 1) / kTX, (ny + 15) / 16);
            kob_adj_kernel<R, kTX, 16><<<grid, kAdjThreads, kob_adj_smem<R, 16>(), s>>>(
                kob_args(p), ps, (const R *)in, (const R *)gout, (R *)gin, gparams);
        }
    } else if (gg_use32<R>(p, 2)) {
        gg_adj32_kernel<R><<<(nx / 32) * (ny / 32), kAdjThreads, G32<R>::smem(2 * p->nfields, 2), s>>>(
            gg_args(p), ps, (const R *)in, (const R *)gout, (R *)gin, gparams);
    } else {
        const dim3 grid((nx + kGX - 1) / kGX, (ny + kGY - 1) / kGY);
        gg_adj_kernel<R><<<grid, kAdjThreads, 2 * (size_t)p->nfields * GReg::N * sizeof(R), s>>>(
            gg_args(p), ps, (const R *)in, (const R *)gout, (R *)gin, gparams);
    }
}

cudaError_t prepare(int dtype)
{
    static cudaError_t done[2] = {cudaErrorNotReady, cudaErrorNotReady};
    const int k = dtype == AMPS_F64 ? 0 : 1;
    if (done[k] != cudaSuccess) done[k] = k == 0 ? kob_prepare<double>() : kob_prepare<float>();
    return done[k];
}

void forward_any(int dtype, const amps_params *p, const ParamSrc &ps, const void *in, void *out, cudaStream_t s)
{
    if (dtype == AMPS_F64) launch_forward<double>(p, ps, in, out, s);
    else launch_forward<float>(p, ps, in, out, s);
}

void adjoint_any(int dtype, const amps_params *p, const ParamSrc &ps, const void *in, const void *gout, void *gin,
                 double *gparams, cudaStream_t s)
{
    if (dtype == AMPS_F64) launch_adjoint<double>(p, ps, in, gout, gin, gparams, s);
    else launch_adjoint<float>(p, ps, in, gout, gin, gparams, s);
}

}  // namespace

extern "C" int amps_step_forward(const amps_params *p, int dtype, const void *state_in, void *state_out, int64_t step,
                                 void *stream)
{
    if (int r = check(p, dtype)) return r;
    if (!state_in || !state_out || state_in == state_out) return AMPS_ERR_INVALID;
    if (prepare(dtype) != cudaSuccess) return AMPS_ERR_CUDA;
    forward_any(dtype, p, param_src(p, step), state_in, state_out, (cudaStream_t)stream);
    return cudaGetLastError() == cudaSuccess ? AMPS_OK : AMPS_ERR_CUDA;
}

extern "C" int amps_step_adjoint(const amps_params *p, int dtype, const void *state_in, const void *grad_out,
                                 void *grad_in, double *grad_params, int64_t step, void *stream)
{
    if (int r = check(p, dtype)) return r;
    if (!state_in || !grad_out || !grad_in || !grad_params || grad_in == grad_out || grad_in == state_in)
        return AMPS_ERR_INVALID;
    if (prepare(dtype) != cudaSuccess) return AMPS_ERR_CUDA;
    adjoint_any(dtype, p, param_src(p, step), state_in, grad_out, grad_in, grad_params, (cudaStream_t)stream);
    return cudaGetLastError() == cudaSuccess ? AMPS_OK : AMPS_ERR_CUDA;
}

// ------------------------------------------------------ rollout handle ----
namespace {

__global__ void set_params_kernel(double *pv, double a, double b, double c, int64_t *dstep, int64_t step0)
{
    pv[0] = a;
    pv[1] = b;
    pv[2] = c;
    *dstep = step0;
}

int auto_segment(int nsteps)
{
    int s = 1;
    while ((int64_t)s * s < nsteps) ++s;
    return s;
}

}  // namespace

struct amps_adjoint {
    amps_params p;
    int dtype = AMPS_F64, nsteps = 0, seg = 1, nseg = 1;
    size_t state_bytes = 0;
    cudaStream_t stream = nullptr, capture = nullptr;
    char *mem = nullptr;  // one allocation: checkpoints, replay states, ping-pong, params
    std::vector<char *> ckpt, segbuf;
    char *tmp[2] = {nullptr, nullptr}, *g[2] = {nullptr, nullptr};
    double *dpv = nullptr, *dgp = nullptr;
    int64_t *dstep = nullptr;
    const char *final_state = nullptr, *final_grad = nullptr;
    bool graphs = true, have_forward = false;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};  // forward sweep, backward sweep
    char err[160] = "";

    ParamSrc src(int64_t off) const
    {
        ParamSrc s;
        s.v[0] = s.v[1] = s.v[2] = 0.0;
        s.dev = dpv;
        s.step = off;
        s.dstep = dstep;
        return s;
    }

    // The whole forward sweep; step k reads the previous output, checkpoint
    // slots take every seg-th state so nothing is copied.
    void enqueue_forward(cudaStream_t s)
    {
        const char *src_p = ckpt[0];
        for (int k = 0; k < nsteps; ++k) {
            char *dst = ((k + 1) % seg == 0 && k + 1 < nsteps) ? ckpt[(k + 1) / seg]
                                                                : (src_p == tmp[0] ? tmp[1] : tmp[0]);
            forward_any(dtype, &p, src(k), src_p, dst, s);
            src_p = dst;
        }
        final_state = src_p;
    }

    // Segments in reverse: replay the segment from its checkpoint (keeping
    // every step's input), then run its adjoint steps backwards.
    void enqueue_backward(cudaStream_t s)
    {
        int cur = 0;
        std::vector<const char *> st(seg);
        for (int sg = nseg - 1; sg >= 0; --sg) {
            const int first = sg * seg, count = nsteps - first < seg ? nsteps - first : seg;
            st[0] = ckpt[sg];
            for (int k = 1; k < count; ++k) {
                forward_any(dtype, &p, src(first + k - 1), st[k - 1], segbuf[k - 1], s);
                st[k] = segbuf[k - 1];
            }
            for (int k = count - 1; k >= 0; --k) {
                adjoint_any(dtype, &p, src(first + k), st[k], g[cur], g[cur ^ 1], dgp, s);
                cur ^= 1;
            }
        }
        final_grad = g[cur];
    }

    int fail(int code, const char *what)
    {
        snprintf(err, sizeof err, "%s", what);
        return code;
    }

    int run_sweep(int which)
    {
        if (!graphs) {
            if (which == 0) enqueue_forward(stream);
            else enqueue_backward(stream);
            return cudaGetLastError() == cudaSuccess ? AMPS_OK : fail(AMPS_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
        }
        if (!exec[which]) {
            cudaGraph_t graph = nullptr;
            if (cudaStreamBeginCapture(capture, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return fail(AMPS_ERR_CUDA, "cudaStreamBeginCapture failed");
            if (which == 0) enqueue_forward(capture);
            else enqueue_backward(capture);
            const cudaError_t e1 = cudaStreamEndCapture(capture, &graph);
            if (e1 != cudaSuccess || !graph) return fail(AMPS_ERR_CUDA, cudaGetErrorString(e1));
            const cudaError_t e2 = cudaGraphInstantiate(&exec[which], graph, 0);
            cudaGraphDestroy(graph);
            if (e2 != cudaSuccess) {
                exec[which] = nullptr;
                return fail(AMPS_ERR_CUDA, cudaGetErrorString(e2));
            }
        }
        return cudaGraphLaunch(exec[which], stream) == cudaSuccess ? AMPS_OK : fail(AMPS_ERR_CUDA, "cudaGraphLaunch failed");
    }

    ~amps_adjoint()
    {
        for (auto &e : exec)
            if (e) cudaGraphExecDestroy(e);
        if (capture) cudaStreamDestroy(capture);
        if (mem) cudaFree(mem);
    }
};

namespace {

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t layout_bytes(const amps_params *p, int dtype, int nsteps, int seg, size_t *state_bytes, int *nseg)
{
    const size_t sb = align256((size_t)state_elems(p) * (dtype == AMPS_F64 ? 8 : 4));
    const int ns = (nsteps + seg - 1) / seg;
    if (state_bytes) *state_bytes = sb;
    if (nseg) *nseg = ns;
    // checkpoints + (seg - 1) replay states + 2 forward + 2 cotangent buffers + params/step/grads
    return sb * ((size_t)ns + (size_t)(seg - 1) + 4) + 256;
}

}  // namespace

extern "C" size_t amps_adjoint_memory_bytes(const amps_params *p, int dtype, int nsteps, int segment)
{
    if (check(p, dtype) != AMPS_OK || nsteps < 1 || segment < 0) return 0;
    const int seg = segment == 0 ? auto_segment(nsteps) : (segment > nsteps ? nsteps : segment);
    return layout_bytes(p, dtype, nsteps, seg, nullptr, nullptr);
}

extern "C" int amps_adjoint_create(const amps_params *p, int dtype, int nsteps, int segment, amps_adjoint **out)
{
    if (!out) return AMPS_ERR_INVALID;
    *out = nullptr;
    if (int r = check(p, dtype)) return r;
    if (nsteps < 1 || segment < 0) return AMPS_ERR_INVALID;
    if (prepare(dtype) != cudaSuccess) return AMPS_ERR_CUDA;
    amps_adjoint *a = new (std::nothrow) amps_adjoint;
    if (!a) return AMPS_ERR_ALLOC;
    a->p = *p;
    a->dtype = dtype;
    a->nsteps = nsteps;
    a->seg = segment == 0 ? auto_segment(nsteps) : (segment > nsteps ? nsteps : segment);
    const size_t total = layout_bytes(p, dtype, nsteps, a->seg, &a->state_bytes, &a->nseg);
    if (cudaMalloc(&a->mem, total) != cudaSuccess) {
        cudaGetLastError();
        delete a;
        return AMPS_ERR_ALLOC;
    }
    char *q = a->mem;
    for (int i = 0; i < a->nseg; ++i, q += a->state_bytes) a->ckpt.push_back(q);
    for (int i = 0; i < a->seg - 1; ++i, q += a->state_bytes) a->segbuf.push_back(q);
    a->tmp[0] = q; q += a->state_bytes;
    a->tmp[1] = q; q += a->state_bytes;
    a->g[0] = q; q += a->state_bytes;
    a->g[1] = q; q += a->state_bytes;
    a->dpv = (double *)q;
    a->dgp = a->dpv + 4;
    a->dstep = (int64_t *)(a->dpv + 8);
    if (cudaStreamCreateWithFlags(&a->capture, cudaStreamNonBlocking) != cudaSuccess) {
        delete a;
        return AMPS_ERR_CUDA;
    }
    *out = a;
    return AMPS_OK;
}

extern "C" int amps_adjoint_destroy(amps_adjoint *a)
{
    if (!a) return AMPS_ERR_INVALID;
    if (a->stream) cudaStreamSynchronize(a->stream);
    else cudaDeviceSynchronize();
    delete a;
    return AMPS_OK;
}

extern "C" int amps_adjoint_set_stream(amps_adjoint *a, void *stream)
{
    if (!a) return AMPS_ERR_INVALID;
    a->stream = (cudaStream_t)stream;
    return AMPS_OK;
}

extern "C" int amps_adjoint_set_graphs(amps_adjoint *a, int enable)
{
    if (!a) return AMPS_ERR_INVALID;
    a->graphs = enable != 0;
    return AMPS_OK;
}

extern "C" int amps_adjoint_segment(const amps_adjoint *a) { return a ? a->seg : -1; }

extern "C" const char *amps_adjoint_last_error(const amps_adjoint *a) { return a ? a->err : "null handle"; }

extern "C" int amps_adjoint_forward(amps_adjoint *a, const double *param_values, const void *state0,
                                    void *state_final, int64_t step0)
{
    if (!a || !param_values || !state0) return AMPS_ERR_INVALID;
    set_params_kernel<<<1, 1, 0, a->stream>>>(a->dpv, param_values[0], param_values[1], param_values[2], a->dstep,
                                             step0);
    if (cudaMemcpyAsync(a->ckpt[0], state0, (size_t)state_elems(&a->p) * (a->dtype == AMPS_F64 ? 8 : 4),
                        cudaMemcpyDeviceToDevice, a->stream) != cudaSuccess)
        return a->fail(AMPS_ERR_CUDA, "state0 copy failed");
    if (int r = a->run_sweep(0)) return r;
    if (state_final &&
        cudaMemcpyAsync(state_final, a->final_state, (size_t)state_elems(&a->p) * (a->dtype == AMPS_F64 ? 8 : 4),
                        cudaMemcpyDeviceToDevice, a->stream) != cudaSuccess)
        return a->fail(AMPS_ERR_CUDA, "final state copy failed");
    a->have_forward = true;
    return AMPS_OK;
}

extern "C" int amps_adjoint_backward(amps_adjoint *a, const void *grad_final, void *grad_state0, double *grad_params)
{
    if (!a || !grad_final) return AMPS_ERR_INVALID;
    if (!a->have_forward) return a->fail(AMPS_ERR_INVALID, "amps_adjoint_backward before amps_adjoint_forward");
    const size_t bytes = (size_t)state_elems(&a->p) * (a->dtype == AMPS_F64 ? 8 : 4);
    if (cudaMemsetAsync(a->dgp, 0, 3 * sizeof(double), a->stream) != cudaSuccess ||
        cudaMemcpyAsync(a->g[0], grad_final, bytes, cudaMemcpyDeviceToDevice, a->stream) != cudaSuccess)
        return a->fail(AMPS_ERR_CUDA, "cotangent copy failed");
    if (int r = a->run_sweep(1)) return r;
    if (grad_state0 &&
        cudaMemcpyAsync(grad_state0, a->final_grad, bytes, cudaMemcpyDeviceToDevice, a->stream) != cudaSuccess)
        return a->fail(AMPS_ERR_CUDA, "gradient copy failed");
    if (grad_params &&
        cudaMemcpyAsync(grad_params, a->dgp, 3 * sizeof(double), cudaMemcpyDeviceToDevice, a->stream) != cudaSuccess)
        return a->fail(AMPS_ERR_CUDA, "parameter gradient copy failed");
    return AMPS_OK;
}
