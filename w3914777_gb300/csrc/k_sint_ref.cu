// k_sint_ref.cu -- sintering step in the reference's own mixed-precision
// arithmetic (amps_params.half_arith = AMPS_HALF_REF): half tiles compute in
// binary16, every operation rounded on its own in the reference's order
// (sintering/function.h:161-774, con1_mix / con2_mix / phi1_mix / phi2_mix,
// low branches), FP64 tiles in the reference's double order (the same
// expressions as the plain kernels, sintering/function.h:51-159).
//
// Two launches a step, as the reference's data flow needs: the chemical
// potential mu of every cell is computed by the cell's owner tile at that
// tile's tier (pass 1), and c' = c + dt*M*lap(mu) and every eta' read their
// neighbours' mu (pass 2).  A half tile sees every neighbour's value --
// state or mu -- as the half rounding of its float rounding, as the
// reference's __float2half / __floats2half2_rn patching gives it
// (sintering/function.h:221-224, the high tiles' edge patches at :310-315,
// :469-474); an FP64 tile sees every value exactly (half values widen
// exactly, as the reference's ring write-backs give them).  mu is kept in
// one double array: exact for the half owners' values.
//
// The reference packs a tile's half2 as columns x and x+8
// (sintering/tools.h:73-86); the lanes compute independently, so one cell per
// thread in scalar binary16 gives the same bits.  N particles generalise
// eta1/eta2 as the plain path does: sums over every particle in order, and
// sum_{p<q} 2 eta_p eta_q for the grain-boundary mobility.
#include "amps_internal.cuh"
#include "amps_kernels.h"

namespace amps {

namespace {

// the value a half tile reads: half(float(v))
__device__ __forceinline__ __half to_half(double v) { return __float2half_rn((float)v); }
__device__ __forceinline__ __half hk(const Phys &ph, int i) { return __ushort_as_half(ph.sn_h[i]); }
__device__ __forceinline__ __half hadd(__half a, __half b) { return __hadd_rn(a, b); }
__device__ __forceinline__ __half hsub(__half a, __half b) { return __hsub_rn(a, b); }
__device__ __forceinline__ __half hmul(__half a, __half b) { return __hmul_rn(a, b); }
__device__ __forceinline__ __half hc(float v) { return __float2half_rn(v); }

// value of field f at grid cell (x, y), read at its owner tile's input tier
template <int T> __device__ __forceinline__ double cell(const StepArgs &a, int f, int x, int y)
{
    const int t = (y / T) * a.ntx + x / T;
    return load_tier<double>(a, a.tier_in[t], (int64_t)f * a.n + (int64_t)y * a.nx + x);
}

}  // namespace

// Pass 1: mu at every cell of tile blockIdx.x, at the tile's tier.
template <int T>
__global__ void __launch_bounds__(kThreads) sint_ref_mu_kernel(StepArgs a, double *mu)
{
    const int tile = blockIdx.x, tx = tile % a.ntx, ty = tile / a.ntx;
    const bool high = a.tier_out[tile] == TIER_FP64;
    const int np = a.nf - 1;
    const Phys &ph = a.ph;
    for (int u = threadIdx.x; u < T * T; u += kThreads) {
        const int gx = tx * T + u % T, gy = ty * T + u / T;
        const int xs1 = bc_map(gx - 1, a.nx, a.bc), xa1 = bc_map(gx + 1, a.nx, a.bc);
        const int ys1 = bc_map(gy - 1, a.ny, a.bc), ya1 = bc_map(gy + 1, a.ny, a.bc);
        const double c = cell<T>(a, 0, gx, gy), cw = cell<T>(a, 0, xs1, gy), ce = cell<T>(a, 0, xa1, gy),
                     cs = cell<T>(a, 0, gx, ys1), cn = cell<T>(a, 0, gx, ya1);
        double m;
        if (high) {
            // sintering/function.h:67-71 (con1_pure; the high branch of con1_mix)
            const double lap = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(cw, ce), cs), cn), __dmul_rn(4.0, c)),
                                         ph.dxdy);
            const double e0 = cell<T>(a, 1, gx, gy);
            double s2 = __dmul_rn(e0, e0), s3 = cube_rn(e0);
            for (int k = 1; k < np; ++k) {
                const double e = cell<T>(a, 1 + k, gx, gy);
                s2 = __dadd_rn(s2, __dmul_rn(e, e));
                s3 = __dadd_rn(s3, cube_rn(e));
            }
            const double A2 = 2.0 * ph.A;
            const double dfdc = __dadd_rn(
                __dsub_rn(__dmul_rn(ph.B, __dsub_rn(__dadd_rn(__dmul_rn(2.0, c), __dmul_rn(4.0, s3)), __dmul_rn(6.0, s2))),
                          __dmul_rn(__dmul_rn(A2, __dmul_rn(c, c)), __dsub_rn(1.0, c))),
                __dmul_rn(__dmul_rn(A2, c), __dmul_rn(__dsub_rn(1.0, c), __dsub_rn(1.0, c))));
            m = __dsub_rn(dfdc, __dmul_rn(0.5 * ph.coefm, lap));
        } else {
            // sintering/function.h:245-249 (con1_mix, low branch)
            const __half h = to_half(c);
            const __half lap = __hdiv(hsub(hadd(hadd(hadd(to_half(cw), to_half(ce)), to_half(cs)), to_half(cn)),
                                           hmul(hc(4.f), h)),
                                      hk(ph, SH_DXDY));
            __half s2 = hc(0.f), s3 = hc(0.f);
            for (int k = 0; k < np; ++k) {
                const __half e = to_half(cell<T>(a, 1 + k, gx, gy));
                const __half e2 = hmul(e, e), e3 = hmul(hmul(e, e), e);
                s2 = k ? hadd(s2, e2) : e2;
                s3 = k ? hadd(s3, e3) : e3;
            }
            const __half one_c = hsub(hc(1.f), h);
            const __half x = hsub(hadd(hmul(hc(2.f), h), hmul(hc(4.f), s3)), hmul(hc(6.f), s2));
            const __half dfdc = hadd(hsub(hmul(hk(ph, SH_B), x), hmul(hmul(hk(ph, SH_A2), hmul(h, h)), one_c)),
                                     hmul(hmul(hk(ph, SH_A2), h), hmul(one_c, one_c)));
            m = (double)__half2float(hsub(dfdc, hmul(hmul(hc(0.5f), hk(ph, SH_COEFM)), lap)));
        }
        mu[(int64_t)gy * a.nx + gx] = m;
    }
}

// Pass 2: c' (con2_mix) then every eta' (phi1_mix / phi2_mix) at every cell
// of tile blockIdx.x, at the tile's tier; on monitor steps the tile metric
// of c'.
template <int T>
__global__ void __launch_bounds__(kThreads) sint_ref_update_kernel(StepArgs a, const double *mu)
{
    __shared__ double red[kThreads / 32];
    const int tile = blockIdx.x, tx = tile % a.ntx, ty = tile / a.ntx;
    const bool high = a.tier_out[tile] == TIER_FP64;
    const int np = a.nf - 1;
    const Phys &ph = a.ph;
    MonAcc mon;
    const bool mon_on = a.monitor_now != 0;
    if (mon_on) mon_reset(a, mon);
    for (int u = threadIdx.x; u < T * T; u += kThreads) {
        const int i = u % T, j = u / T;
        const int gx = tx * T + i, gy = ty * T + j;
        const int xs1 = bc_map(gx - 1, a.nx, a.bc), xa1 = bc_map(gx + 1, a.nx, a.bc);
        const int ys1 = bc_map(gy - 1, a.ny, a.bc), ya1 = bc_map(gy + 1, a.ny, a.bc);
        const int64_t g = (int64_t)gy * a.nx + gx;
        const double m0 = mu[g], mw = mu[(int64_t)gy * a.nx + xs1], me = mu[(int64_t)gy * a.nx + xa1],
                     ms = mu[(int64_t)ys1 * a.nx + gx], mn = mu[(int64_t)ya1 * a.nx + gx];
        const double c = cell<T>(a, 0, gx, gy);
        double cnew;
        if (high) {
            // sintering/function.h:90-101 (con2_pure; the high branch of con2_mix)
            const double lapm = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(mw, me), ms), mn), __dmul_rn(4.0, m0)),
                                          ph.dxdy);
            const double phi = __dmul_rn(cube_rn(c), __dadd_rn(__dsub_rn(10.0, __dmul_rn(15.0, c)), __dmul_rn(6.0, __dmul_rn(c, c))));
            double sum = 0.0;
            for (int p = 0; p < np; ++p)
                for (int q = p + 1; q < np; ++q)
                    sum = __dadd_rn(sum, __dmul_rn(__dmul_rn(cell<T>(a, 1 + p, gx, gy), cell<T>(a, 1 + q, gx, gy)), 2.0));
            const double mob = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(ph.dvol, phi), __dmul_rn(ph.dvap, __dsub_rn(1.0, phi))),
                                                   __dmul_rn(__dmul_rn(ph.dsur, c), __dsub_rn(1.0, c))),
                                         __dmul_rn(ph.dgrb, sum));
            double v = __dadd_rn(c, __dmul_rn(__dmul_rn(ph.dt, mob), lapm));
            if (v >= 1) v = 1;
            else if (v < 0) v = 0;
            cnew = v;
            ((double *)a.out[TIER_FP64])[g] = cnew;
        } else {
            // sintering/function.h:401-411 (con2_mix, low branch)
            const __half h = to_half(c);
            const __half lapm = __hdiv(hsub(hadd(hadd(hadd(to_half(mw), to_half(me)), to_half(ms)), to_half(mn)),
                                            hmul(hc(4.f), to_half(m0))),
                                       hk(ph, SH_DXDY));
            const __half phi = hmul(hmul(hmul(h, h), h), hadd(hsub(hc(10.f), hmul(hc(15.f), h)), hmul(hc(6.f), hmul(h, h))));
            __half sum = hc(0.f);
            bool first = true;
            for (int p = 0; p < np; ++p)
                for (int q = p + 1; q < np; ++q) {
                    const __half t = hmul(hmul(to_half(cell<T>(a, 1 + p, gx, gy)), to_half(cell<T>(a, 1 + q, gx, gy))),
                                          hc(2.f));
                    sum = first ? t : hadd(sum, t);
                    first = false;
                }
            const __half one_c = hsub(hc(1.f), h), one_phi = hsub(hc(1.f), phi);
            const __half mob = hadd(hadd(hadd(hmul(hk(ph, SH_DVOL), phi), hmul(hk(ph, SH_DVAP), one_phi)),
                                         hmul(hmul(hk(ph, SH_DSUR), h), one_c)),
                                    hmul(hk(ph, SH_DGRB), sum));
            __half v = hadd(h, hmul(hmul(hk(ph, SH_DT), mob), lapm));
            v = __hmax(hc(0.f), __hmin(hc(1.f), v));
            cnew = (double)__half2float(v);
            ((__half *)a.out[TIER_HALF])[g] = v;
        }
        if (mon_on && a.mfield <= 0) mon_add<T>(a, mon, 0, tile, j, i, g, cnew, c, snap_prefetch<T>(a, 0, tile, j, i, g));
        // eta' of every particle (sintering/function.h:126-131; phi1_mix low branch :556-565)
        if (high) {
            const double e0 = cell<T>(a, 1, gx, gy);
            double s2 = __dmul_rn(e0, e0);
            for (int k = 1; k < np; ++k) {
                const double e = cell<T>(a, 1 + k, gx, gy);
                s2 = __dadd_rn(s2, __dmul_rn(e, e));
            }
            for (int k = 0; k < np; ++k) {
                const double e = cell<T>(a, 1 + k, gx, gy);
                const double lap = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(cell<T>(a, 1 + k, xs1, gy),
                                                                                      cell<T>(a, 1 + k, xa1, gy)),
                                                                             cell<T>(a, 1 + k, gx, ys1)),
                                                                    cell<T>(a, 1 + k, gx, ya1)),
                                                          __dmul_rn(4.0, e)),
                                             ph.dxdy);
                const double dfd = __dmul_rn(ph.B, __dadd_rn(__dadd_rn(
                    __dmul_rn(__dmul_rn(-12.0, __dmul_rn(e, e)), __dsub_rn(2.0, cnew)),
                    __dmul_rn(__dmul_rn(12.0, e), __dsub_rn(1.0, cnew))), __dmul_rn(__dmul_rn(12.0, e), s2)));
                double v = __dsub_rn(e, __dmul_rn(ph.dt * ph.coefl, __dsub_rn(dfd, __dmul_rn(0.5 * ph.coefk, lap))));
                if (v >= 1) v = 1;
                else if (v < 0) v = 0;
                ((double *)a.out[TIER_FP64])[(int64_t)(1 + k) * a.n + g] = v;
            }
        } else {
            const __half hcn = to_half(cnew);
            __half s2 = hc(0.f);
            for (int k = 0; k < np; ++k) {
                const __half e = to_half(cell<T>(a, 1 + k, gx, gy));
                s2 = k ? hadd(s2, hmul(e, e)) : hmul(e, e);
            }
            for (int k = 0; k < np; ++k) {
                const __half e = to_half(cell<T>(a, 1 + k, gx, gy));
                const __half lap = __hdiv(hsub(hadd(hadd(hadd(to_half(cell<T>(a, 1 + k, xs1, gy)),
                                                              to_half(cell<T>(a, 1 + k, xa1, gy))),
                                                         to_half(cell<T>(a, 1 + k, gx, ys1))),
                                                    to_half(cell<T>(a, 1 + k, gx, ya1))),
                                               hmul(hc(4.f), e)),
                                          hk(ph, SH_DXDY));
                const __half t1 = hmul(hmul(__hneg(hc(12.f)), hmul(e, e)), hsub(hc(2.f), hcn));
                const __half t2 = hmul(hmul(hc(12.f), e), hsub(hc(1.f), hcn));
                const __half t3 = hmul(hmul(hc(12.f), e), s2);
                const __half dfd = hmul(hk(ph, SH_B), hadd(hadd(t1, t2), t3));
                __half v = hsub(e, hmul(hmul(hk(ph, SH_DT), hk(ph, SH_COEFL)),
                                        hsub(dfd, hmul(hmul(hc(0.5f), hk(ph, SH_COEFK)), lap))));
                v = __hmax(hc(0.f), __hmin(hc(1.f), v));
                ((__half *)a.out[TIER_HALF])[(int64_t)(1 + k) * a.n + g] = v;
            }
        }
    }
    if (mon_on) {
        const double metric = mon_finish(a, mon, red, 0.0);
        if (threadIdx.x == 0) a.metric[tile] = metric;
    }
}

cudaError_t sint_ref_launch(int tile, const StepArgs &a, double *mu, int grid, cudaStream_t s)
{
    if (tile == 32) {
        sint_ref_mu_kernel<32><<<grid, kThreads, 0, s>>>(a, mu);
        sint_ref_update_kernel<32><<<grid, kThreads, 0, s>>>(a, mu);
    } else {
        sint_ref_mu_kernel<16><<<grid, kThreads, 0, s>>>(a, mu);
        sint_ref_update_kernel<16><<<grid, kThreads, 0, s>>>(a, mu);
    }
    return cudaGetLastError();
}

}  // namespace amps
