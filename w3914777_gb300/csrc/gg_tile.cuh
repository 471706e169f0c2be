// gg_tile.cuh -- the per-tile body of the fused grain-growth step, shared by
// the single-run step kernel (k_graingrowth.cu), its binary16-arithmetic
// instantiations (k_gg_half.cu) and the ensemble's tile-queue kernel.
//
// Reference: graingrowth/function.h:5-30 (kernel1_pure) and
// graingrowth/function.h:33-277 (kernel1_mix), generalised from Q=2 to Q
// fields with cross coefficient gamma:
//   dfd_i = 2*gamma*eta_i*sum_{j!=i} eta_j^2 + eta_i^3 - eta_i
//   eta_i' = eta_i - dt*L*(dfd_i - kappa*lap(eta_i)).
#pragma once
#include "amps_internal.cuh"

namespace amps {

// Half / FP32 tile: staged float neighbourhood, float arithmetic.  Each
// thread advances CPT consecutive cells of one row (CPT = 4 for 32x32 tiles:
// one 128-bit shared load plus two halo scalars per row, shared row sums,
// 128-bit / 64-bit global stores).
template <int TIER, int CPT>
__device__ __forceinline__ void store_cells(const StepArgs &a, int64_t idx, const float *v)
{
    if (CPT == 4 && TIER == TIER_FP32) {
        *reinterpret_cast<float4 *>((float *)a.out[TIER_FP32] + idx) = make_float4(v[0], v[1], v[2], v[3]);
    } else if (CPT == 4 && TIER == TIER_HALF) {
        __half2 h0 = __floats2half2_rn(v[0], v[1]), h1 = __floats2half2_rn(v[2], v[3]);
        uint2 u;
        u.x = *reinterpret_cast<unsigned *>(&h0);
        u.y = *reinterpret_cast<unsigned *>(&h1);
        *reinterpret_cast<uint2 *>((__half *)a.out[TIER_HALF] + idx) = u;
    } else {
#pragma unroll
        for (int k = 0; k < CPT; ++k) store_tier<TIER>(a, idx + k, v[k]);
    }
}

// MON: this step evaluates the monitor (compiled out of the other steps, so
// their loop carries no monitor state).
template <int T, int TIER, bool MON>
__device__ __forceinline__ void gg_tile_lo_impl(const StepArgs &a, const float *sm, int tile, int tx, int ty,
                                                double *red)
{
    using S = Stage<float, T, 1>;
    constexpr int CPT = T * T / kThreads;  // cells per thread, along x
    constexpr int GPR = T / CPT;           // thread groups per row
    const int row = threadIdx.x / GPR;
    const int c0 = (threadIdx.x % GPR) * CPT;
    const int nf = a.nf;
    const Phys &ph = a.ph;
    float *smm = const_cast<float *>(sm);
    float ssum[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) ssum[k] = 0.f;
    for (int f = 0; f < nf; ++f) {
        float c[CPT];
        const float *ctr = &S::at(smm, f, row + 1, S::O + c0);
#pragma unroll
        for (int k = 0; k < CPT; ++k) c[k] = ctr[k];
#pragma unroll
        for (int k = 0; k < CPT; ++k) ssum[k] = fmaf(c[k], c[k], ssum[k]);
    }
    const float dtm = ph.gg_dtm, g2 = ph.gg_g2, kap = ph.gg_kap, inv = ph.gg_inv;
    const int64_t gbase = (int64_t)(ty * T + row) * a.px + tx * T + c0;
    double metric = 0.0;
    MonAccF mon;
    for (int f = 0; f < nf; ++f) {
        const bool mon_f = MON && (a.mfield < 0 || a.mfield == f);
        const int mslot = a.mfield < 0 ? f : 0;
        double snapv[CPT];
        if (mon_f) {
            mon_reset(a, mon);
#pragma unroll
            for (int k = 0; k < CPT; ++k) snapv[k] = snap_prefetch<T>(a, mslot, tile, row, c0 + k, gbase + k);
        }
        float w[3][CPT + 2];
#pragma unroll
        for (int rr = 0; rr < 3; ++rr) {
            const float *p = &S::at(smm, f, row + rr, S::O + c0);
            if (CPT == 4) {
                const float4 q = *reinterpret_cast<const float4 *>(p);
                w[rr][1] = q.x; w[rr][2] = q.y; w[rr][3] = q.z; w[rr][4] = q.w;
            } else {
#pragma unroll
                for (int k = 0; k < CPT; ++k) w[rr][k + 1] = p[k];
            }
            w[rr][0] = p[-1];
            w[rr][CPT + 1] = p[CPT];
        }
        float out[CPT];
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            const float e = w[1][k + 1];
            float s;
            if (a.stencil == 0)
                s = (w[0][k] + w[0][k + 1] + w[0][k + 2]) + (w[1][k] + w[1][k + 2]) + (w[2][k] + w[2][k + 1] + w[2][k + 2])
                  - 8.f * e;
            else
                s = (w[1][k] + w[1][k + 2]) + (w[0][k + 1] + w[2][k + 1]) - 4.f * e;
            const float lap = s * inv;
            const float e2 = e * e;
            const float dfd = e * fmaf(g2, ssum[k] - e2, e2 - 1.f);
            out[k] = fmaf(-dtm, fmaf(-kap, lap, dfd), e);
        }
        store_cells<TIER, CPT>(a, (int64_t)f * a.n + gbase, out);
        if (mon_f) {
            // a ragged grid's edge tile: cells past the domain are not samples
            const int vw = min(T, a.nx - tx * T), vh = min(T, a.ny - ty * T);
#pragma unroll
            for (int k = 0; k < CPT; ++k)
                if (row < vh && c0 + k < vw)
                    mon_add<T>(a, mon, mslot, tile, row, c0 + k, gbase + k, round_to_tier<TIER>(out[k]), w[1][k + 1],
                               snapv[k]);
            metric = mon_finish(a, mon, red, metric);
        }
    }
    if (MON && threadIdx.x == 0) a.metric[tile] = metric;
}

template <int T, int TIER>
__device__ __forceinline__ void gg_tile_lo(const StepArgs &a, const float *sm, int tile, int tx, int ty, double *red)
{
    if (a.monitor_now) gg_tile_lo_impl<T, TIER, true>(a, sm, tile, tx, ty, red);
    else gg_tile_lo_impl<T, TIER, false>(a, sm, tile, tx, ty, red);
}

// Half/FP32 tile, 32^2 tiles: the sum of squares over fields is formed once
// per cell into shared memory (ss, 32x32 floats, after the staged fields),
// then each thread advances RPT rows x 4 cells of a field from RPT + 2 staged
// rows with a 3-row register window (RPT = 4: 1.5 row reads per output row,
// 8: 1.25, against 2 for two rows a thread), the CTA's RPT groups on fields
// g, g+RPT, ...  Per cell the arithmetic, and its order, is
// gg_tile_lo_impl's.  MK, the monitor kind of a monitor step (0: none, 2:
// temporal, 3: rate; the spatial range takes gg_tile_lo_impl): the tile
// metric is a maximum over fields and cells, so each thread folds every
// field it computes into one accumulator and the block reduces once.
// PH > 0: one CTA of a split tile -- staging slots 0..PH-1 hold fields
// [f0, f0 + PH), and the caller has formed `ss` over every field.
template <int TIER, int RPT, int MK = 0, int PH = 0>
__device__ __forceinline__ void gg_tile_lo_rows(const StepArgs &a, const float *sm, float *ss, int tile, int tx,
                                                int ty, double *red, int f0 = 0)
{
    static_assert(PH == 0 || MK == 0, "split tiles run the steps without a monitor");
    constexpr int T = 32, CPT = 4, GPR = T / CPT;
    using S = Stage<float, T, 1>;
    float *smm = const_cast<float *>(sm);
    const int nf = PH ? PH : a.nf;
    if constexpr (PH == 0) {
        const int row = threadIdx.x / GPR, c = (threadIdx.x % GPR) * CPT;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int f = 0; f < nf; ++f) {
            const float4 q = *reinterpret_cast<const float4 *>(&S::at(smm, f, row + 1, S::O + c));
            acc.x = fmaf(q.x, q.x, acc.x);
            acc.y = fmaf(q.y, q.y, acc.y);
            acc.z = fmaf(q.z, q.z, acc.z);
            acc.w = fmaf(q.w, q.w, acc.w);
        }
        *reinterpret_cast<float4 *>(ss + row * T + c) = acc;
        __syncthreads();
    }
    static_assert(T % RPT == 0 && (T / RPT) * GPR * RPT == kThreads, "RPT groups of T/RPT x GPR threads");
    const int group = threadIdx.x / (kThreads / RPT), t = threadIdx.x % (kThreads / RPT);
    const int r0 = RPT * (t / GPR), c0 = (t % GPR) * CPT;  // tile-local rows r0 .. r0+RPT-1
    const Phys &ph = a.ph;
    const float dtm = ph.gg_dtm, g2 = ph.gg_g2, kap = ph.gg_kap, inv = ph.gg_inv;
    const int64_t gbase = (int64_t)(ty * T + r0) * a.px + tx * T + c0;
    MonAccF mon;
    if (MK) mon_reset(a, mon);
    for (int f = group; f < nf; f += RPT) {
        const bool mon_f = MK && (a.mfield < 0 || a.mfield == f);
        const int mslot = a.mfield < 0 ? f : 0;
        float w[3][CPT + 2];
        auto load_row = [&](int sr, float *d) {
            const float *p = &S::at(smm, f, sr, S::O + c0);
            const float4 q = *reinterpret_cast<const float4 *>(p);
            d[0] = p[-1];
            d[1] = q.x; d[2] = q.y; d[3] = q.z; d[4] = q.w;
            d[CPT + 1] = p[CPT];
        };
        load_row(r0, w[0]);
        load_row(r0 + 1, w[1]);
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            float *up = w[i % 3], *md = w[(i + 1) % 3], *dn = w[(i + 2) % 3];
            load_row(r0 + i + 2, dn);
            const float4 sq = *reinterpret_cast<const float4 *>(ss + (r0 + i) * T + c0);
            const float ssum[CPT] = {sq.x, sq.y, sq.z, sq.w};
            float out[CPT];
#pragma unroll
            for (int k = 0; k < CPT; ++k) {
                const float e = md[k + 1];
                float sv;
                if (a.stencil == 0)
                    sv = (up[k] + up[k + 1] + up[k + 2]) + (md[k] + md[k + 2]) + (dn[k] + dn[k + 1] + dn[k + 2]) -
                         8.f * e;
                else
                    sv = (md[k] + md[k + 2]) + (up[k + 1] + dn[k + 1]) - 4.f * e;
                const float lap = sv * inv;
                const float e2 = e * e;
                const float dfd = e * fmaf(g2, ssum[k] - e2, e2 - 1.f);
                out[k] = fmaf(-dtm, fmaf(-kap, lap, dfd), e);
            }
            const int64_t gi = gbase + (int64_t)i * a.px;
            store_cells<TIER, CPT>(a, (int64_t)(f0 + f) * a.n + gi, out);
            if constexpr (MK != 0) {
                // a ragged grid's edge tile: cells past the domain are not samples
                if (mon_f && r0 + i < min(T, a.ny - ty * T)) {
                    const int vw = min(T, a.nx - tx * T);
#pragma unroll
                    for (int k = 0; k < CPT; ++k)
                        if (c0 + k < vw)
                            mon_add_k<T, MK>(a, mon, mslot, tile, r0 + i, c0 + k, gi + k, round_to_tier<TIER>(out[k]),
                                             md[k + 1]);
                }
            }
        }
    }
    if constexpr (MK != 0) {
        const double metric = mon_finish_k<MK>(a, mon, red);
        if (threadIdx.x == 0) a.metric[tile] = metric;
    }
}

// One cell of the FP64 tile's neighbourhood at tile-local (ly, lx), read at
// its owner tile's input tier: the tile of the 3x3 neighbourhood at that
// position, or (own: a ragged grid's edge tile, whose boundary-mapped halo
// can lie in another tile) the tile that holds the mapped cell.
template <int T>
__device__ __forceinline__ double ld_nb64(const StepArgs &a, const uint8_t *nt, int f, int x0, int y0, int ly, int lx,
                                          bool own = false)
{
    const int gy = bc_map(y0 + ly, a.ny, a.bc), gx = bc_map(x0 + lx, a.nx, a.bc);
    const int cls = (ly < 0 ? 0 : (ly < T ? 3 : 6)) + (lx < 0 ? 0 : (lx < T ? 1 : 2));
    const int tier = own ? a.tier_in[(gy / T) * a.ntx + gx / T] : nt[cls];
    return load_tier<double>(a, tier, (int64_t)f * a.n + (int64_t)gy * a.px + gx);
}

// FP64 tile: direct loads through L1 with a rolling 3-row window, FP64
// arithmetic; REF keeps the reference's expression order and rounding
// (graingrowth/function.h:20-23).
// PH > 0: this CTA updates fields [f0, f0 + PH) of the tile (one CTA of a
// split tile; the sum of squares still covers every field).
template <int T, bool REF, bool PARTIAL = false, int PH = 0>
__device__ __forceinline__ void gg_tile_fp64(const StepArgs &a, const uint8_t *nt, int tile, int tx, int ty, double *red,
                                             int f0 = 0)
{
    constexpr bool partial = PARTIAL;  // a ragged grid's edge tile: owner-tier loads
    constexpr int RPT = T * T / kThreads;
    const int col = threadIdx.x % T;
    const int r0 = (threadIdx.x / T) * RPT;
    const int x0 = tx * T, y0 = ty * T;
    const int nf = a.nf;
    const Phys &ph = a.ph;
    double ssum[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) ssum[j] = 0.0;
    if (!REF)
        for (int f = 0; f < nf; ++f)
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const double v = ld_nb64<T>(a, nt, f, x0, y0, r0 + j, col, partial);
                ssum[j] = fma(v, v, ssum[j]);
            }
    const int64_t gbase = (int64_t)(y0 + r0) * a.px + x0 + col;
    double metric = 0.0;
    MonAcc mon;
    for (int f = PH ? f0 : 0; f < (PH ? f0 + PH : nf); ++f) {
        const bool mon_f = a.monitor_now && (a.mfield < 0 || a.mfield == f);
        const int mslot = a.mfield < 0 ? f : 0;
        if (mon_f) mon_reset(a, mon);
        double rd[3], rc[3], ru[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            rd[k] = ld_nb64<T>(a, nt, f, x0, y0, r0 - 1, col + k - 1, partial);
            rc[k] = ld_nb64<T>(a, nt, f, x0, y0, r0, col + k - 1, partial);
        }
#pragma unroll 1
        for (int j = 0; j < RPT; ++j) {
#pragma unroll
            for (int k = 0; k < 3; ++k) ru[k] = ld_nb64<T>(a, nt, f, x0, y0, r0 + j + 1, col + k - 1, partial);
            const int64_t g = gbase + (int64_t)j * a.px;
            const double snapv = mon_f ? snap_prefetch<T>(a, mslot, tile, r0 + j, col, g) : 0.0;
            const double e = rc[1];
            double out;
            if (REF) {
                double lap;
                if (a.stencil == 0)
                    lap = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(
                                      rd[0], rd[1]), rd[2]), rc[0]), rc[2]), ru[0]), ru[1]), ru[2]),
                                      __dmul_rn(8.0, e)), ph.dxdy);
                else
                    lap = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(rc[0], rc[2]), rd[1]), ru[1]),
                                              __dmul_rn(4.0, e)), ph.dxdy);
                double sum = 0.0;
                bool first = true;
                for (int b = 0; b < nf; ++b) {
                    if (b == f) continue;
                    const double v = ld_nb64<T>(a, nt, b, x0, y0, r0 + j, col, partial);
                    const double s2 = __dmul_rn(v, v);
                    sum = first ? s2 : __dadd_rn(sum, s2);
                    first = false;
                }
                const double dfd = __dsub_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0 * ph.gamma, e), sum), pow(e, 3.0)), e);
                out = __dsub_rn(e, __dmul_rn(ph.dt * ph.mobil, __dsub_rn(dfd, __dmul_rn(ph.grcoef, lap))));
            } else {
                double s;
                if (a.stencil == 0) s = (rd[0] + rd[1] + rd[2]) + (rc[0] + rc[2]) + (ru[0] + ru[1] + ru[2]) - 8.0 * e;
                else s = (rc[0] + rc[2]) + (rd[1] + ru[1]) - 4.0 * e;
                const double lap = s * ph.inv_dxdy;
                const double e2 = e * e;
                double sj = ssum[0];
#pragma unroll
                for (int q = 1; q < RPT; ++q) sj = j == q ? ssum[q] : sj;
                const double dfd = e * fma(2.0 * ph.gamma, sj - e2, e2 - 1.0);
                out = fma(-(ph.dt * ph.mobil), fma(-ph.grcoef, lap, dfd), e);
            }
            ((double *)a.out[TIER_FP64])[(int64_t)f * a.n + g] = out;
            // a ragged grid's edge tile: cells past the domain are not samples
            if (mon_f && (!PARTIAL || (r0 + j < a.ny - y0 && col < a.nx - x0)))
                mon_add<T>(a, mon, mslot, tile, r0 + j, col, g, out, e, snapv);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                rd[k] = rc[k];
                rc[k] = ru[k];
            }
        }
        if (mon_f) metric = mon_finish(a, mon, red, metric);
    }
    if (a.monitor_now && threadIdx.x == 0) a.metric[tile] = metric;
}

// The FP64 tile of a ragged grid's edge, out of line (off the whole tiles' registers).
template <int T, bool REF, int PH = 0>
__device__ __noinline__ void gg_tile_fp64_partial(const StepArgs &a, const uint8_t *nt, int tile, int tx, int ty,
                                                  double *red, int f0 = 0)
{
    gg_tile_fp64<T, REF, true, PH>(a, nt, tile, tx, ty, red, f0);
}

__device__ __forceinline__ __half2 gg_hconst(const Phys &ph, int i)
{
    const __half h = __ushort_as_half(ph.gg_h[i]);
    return __halves2half2(h, h);
}

// Half tile in binary16 arithmetic on pairs of adjacent columns, packed as
// the reference packs its half2 tiles (graingrowth/tools.h:165).  Each cell
// enters as the half rounding of its staged float, itself the float rounding
// of the owner tile's input -- the reference's __float2half(double) halo
// patching and its __floats2half2_rn demotion (graingrowth/function.h:87-161,
// graingrowth/tools.h:256-271).
//   HA == AMPS_HALF_REF: graingrowth/function.h:163-166 as written, every
//     +, -, *, / rounded on its own (the _rn intrinsics are never contracted
//     into fused multiply-adds) and in the reference's order; Q fields
//     generalise `hetab*hetab` to the left-to-right sum over j != i, and
//     `htwo*hone` to 2*gamma.  The 5-point stencil follows the FP64
//     reference-order tiles' order.
//   HA == AMPS_HALF_HFMA2: the same update as packed fused multiply-adds,
//     eta*(2*gamma*S + eta^2 - 1) and eta - dt*L*(dfd - kappa/dxdy * s).
// MK != 0: a monitor step; the epilogue folds each stored value (exact in
// double) into the per-field accumulator as the other tiers do.
template <int T, int MK, int HA>
__device__ __forceinline__ void gg_tile_half2(const StepArgs &a, const float *sm, int tile, int tx, int ty, double *red)
{
    using S = Stage<float, T, 1>;
    constexpr int PPR = T / 2, NP = T * PPR;  // pairs per row, per tile
    float *smm = const_cast<float *>(sm);
    const int nf = a.nf;
    const Phys &ph = a.ph;
    const __half2 h1 = __float2half2_rn(1.f), h2 = __float2half2_rn(2.f), h4 = __float2half2_rn(4.f),
                  h8 = __float2half2_rn(8.f);
    auto pair = [&](int f, int sr, int c) {  // staged row sr, tile columns c and c+1
        return __floats2half2_rn(S::at(smm, f, sr, S::O + c), S::at(smm, f, sr, S::O + c + 1));
    };
    double metric = 0.0;
    for (int f = 0; f < nf; ++f) {
        const bool mon_f = MK != 0 && (a.mfield < 0 || a.mfield == f);
        const int mslot = a.mfield < 0 ? f : 0;
        MonAcc mon;
        if (mon_f) mon_reset(a, mon);
        for (int p = threadIdx.x; p < NP; p += kThreads) {
            const int row = p / PPR, c = 2 * (p % PPR);
            const __half2 dl = pair(f, row, c - 1), dc = pair(f, row, c), dr = pair(f, row, c + 1);
            const __half2 ml = pair(f, row + 1, c - 1), ctr = pair(f, row + 1, c), mr = pair(f, row + 1, c + 1);
            const __half2 ul = pair(f, row + 2, c - 1), uc = pair(f, row + 2, c), ur = pair(f, row + 2, c + 1);
            __half2 out;
            if constexpr (HA == 1) {
                __half2 s;
                if (a.stencil == 0) {
                    s = __hadd2_rn(dl, dc);
                    s = __hadd2_rn(s, dr);
                    s = __hadd2_rn(s, ml);
                    s = __hadd2_rn(s, mr);
                    s = __hadd2_rn(s, ul);
                    s = __hadd2_rn(s, uc);
                    s = __hadd2_rn(s, ur);
                    s = __hsub2_rn(s, __hmul2_rn(h8, ctr));
                } else {
                    s = __hsub2_rn(__hadd2_rn(__hadd2_rn(__hadd2_rn(ml, mr), dc), uc), __hmul2_rn(h4, ctr));
                }
                const __half2 lap = __h2div(s, gg_hconst(ph, GH_DXDY));
                __half2 sum = __float2half2_rn(0.f);
                bool first = true;
                for (int b = 0; b < nf; ++b) {
                    if (b == f) continue;
                    const __half2 v = pair(b, row + 1, c);
                    const __half2 s2 = __hmul2_rn(v, v);
                    sum = first ? s2 : __hadd2_rn(sum, s2);
                    first = false;
                }
                __half2 dfd = __hmul2_rn(__hmul2_rn(__hmul2_rn(h2, gg_hconst(ph, GH_GAM)), ctr), sum);
                dfd = __hsub2_rn(__hadd2_rn(dfd, __hmul2_rn(__hmul2_rn(ctr, ctr), ctr)), ctr);
                dfd = __hmul2_rn(h1, dfd);
                out = __hsub2_rn(ctr, __hmul2_rn(__hmul2_rn(gg_hconst(ph, GH_DT), gg_hconst(ph, GH_MOB)),
                                                 __hsub2_rn(dfd, __hmul2_rn(gg_hconst(ph, GH_KAP), lap))));
            } else {
                __half2 s = a.stencil == 0 ? __hadd2(__hadd2(__hadd2(dl, dc), dr), __hadd2(ml, mr)) +
                                                 __hadd2(__hadd2(ul, uc), ur)
                                           : __hadd2(__hadd2(ml, mr), __hadd2(dc, uc));
                s = __hfma2(a.stencil == 0 ? __hneg2(h8) : __hneg2(h4), ctr, s);
                __half2 sum = __float2half2_rn(0.f);
                for (int b = 0; b < nf; ++b) {
                    if (b == f) continue;
                    const __half2 v = pair(b, row + 1, c);
                    sum = __hfma2(v, v, sum);
                }
                const __half2 dfd = __hmul2(ctr, __hfma2(gg_hconst(ph, GH_G2), sum, __hfma2(ctr, ctr, __hneg2(h1))));
                out = __hfma2(__hneg2(gg_hconst(ph, GH_DTM)), __hfma2(__hneg2(gg_hconst(ph, GH_KINV)), s, dfd), ctr);
            }
            const int64_t g = (int64_t)(ty * T + row) * a.px + tx * T + c;
            *reinterpret_cast<__half2 *>((__half *)a.out[TIER_HALF] + (int64_t)f * a.n + g) = out;
            if (mon_f) {
                const double s0 = snap_prefetch<T>(a, mslot, tile, row, c, g);
                const double s1 = snap_prefetch<T>(a, mslot, tile, row, c + 1, g + 1);
                mon_add<T>(a, mon, mslot, tile, row, c, g, (double)__low2float(out), (double)__low2float(ctr), s0);
                mon_add<T>(a, mon, mslot, tile, row, c + 1, g + 1, (double)__high2float(out),
                           (double)__high2float(ctr), s1);
            }
        }
        if (mon_f) metric = mon_finish(a, mon, red, metric);
    }
    if (MK != 0 && threadIdx.x == 0) a.metric[tile] = metric;
}

// ---- ragged grids ----------------------------------------------------------------
// A grid whose sides are not multiples of the tile keeps whole tiles in
// storage (row pitch px = ntx*T, nty*T rows): the last tile column and row
// reach past the domain into that padding.  Such a partial tile is staged and
// computed as a whole tile -- its cells past the domain compute from padding
// and store into padding, which no cell inside the domain ever reads, and
// the monitor skips them -- with one correction: the staged slots of column
// w and row h (w x h: the tile's cells inside the domain), the right and
// lower halo of its last valid cells, held padding and are re-read across
// the boundary map (periodic: column 0 / row 0 of the domain) at the input
// tier of the tile that owns them.  Every access stays inside the storage:
// rows and halo columns are boundary-mapped (nx, ny >= T), interior row
// segments end at most at the padded pitch.
__device__ __forceinline__ bool gg_partial_tile(const StepArgs &a, int T, int tx, int ty)
{
    return (tx + 1) * T > a.nx || (ty + 1) * T > a.ny;
}

// The patch of a partial tile's staging (Stage<CT, T, 1> layout, fields
// [f0, f0 + nfs) in slots 0..nfs-1; nfs < 0: all); the caller synchronises
// before and after.
template <typename CT, int T>
__device__ __noinline__ void patch_ragged(const StepArgs &a, CT *sm, int tx, int ty, int f0 = 0, int nfs = -1)
{
    using S = Stage<CT, T, 1>;
    const int x0 = tx * T, y0 = ty * T;
    const int w = min(T, a.nx - x0), h = min(T, a.ny - y0);
    // column w for rows -1..h (when w < T); row h for columns -1..w-1, or
    // -1..T when the tile is whole in x (the corner (w, h) once)
    const int nc = w < T ? h + 2 : 0;
    const int nr = h < T ? (w < T ? w + 1 : w + 2) : 0;
    for (int u = threadIdx.x; u < nc + nr; u += kThreads) {
        const int lx = u < nc ? w : u - nc - 1, ly = u < nc ? u - 1 : h;
        const int gx = bc_map(x0 + lx, a.nx, a.bc), gy = bc_map(y0 + ly, a.ny, a.bc);
        const int tier = a.tier_in[(gy / T) * a.ntx + gx / T];
        const int64_t o = (int64_t)gy * a.px + gx;
        CT *d = &S::at(sm, 0, ly + 1, S::O + lx);
        const int nl = nfs < 0 ? a.nf : nfs;
        for (int f = 0; f < nl; ++f) d[f * S::FIELD] = load_tier<CT>(a, tier, (int64_t)(f0 + f) * a.n + o);
    }
}

// Fused all-tier step: at most 64 registers, so that four CTAs share an SM
// and the half/FP32 tiles (the common case) keep their occupancy.
// every tile of the 3x3 neighbourhood (after the boundary map) holds FP32 input
__device__ __forceinline__ bool all_fp32(const uint8_t *nt)
{
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 9; ++k) ok &= nt[k] == TIER_FP32;
    return ok;
}

// One tile of the fused step (every tier), by the whole CTA: neighbourhood
// tiers, staging, update (and the monitor on monitor steps).  Shared by the
// single-run step kernel and the ensemble's tile-queue kernel, so that a
// member of an ensemble gets exactly the results of a single run.  MK: 0 for
// a step without the monitor, 1/2/3 a monitor step of that monitor kind
// (spatial / temporal / rate), -1 a monitor step of the kind in `a`.
// NC = false: no read-only-path loads (the persistent multi-step kernel
// reads values that other CTAs of the same launch wrote).  RG: the grid may
// be ragged (its edge tiles partial); compiled out of the whole-tile grids'
// kernels, whose registers it would otherwise spill.
// tm, bar (T = 32): a tensor map of this step's FP32 input and an mbarrier;
// tiles whose halo needs no wrap or mirror then fetch the whole FP32
// neighbourhood -- every field, 34 rows x 40 columns, the staging layout --
// by one bulk tensor copy issued by one thread (sm 128-byte aligned).
template <int T, bool REF, int MK, int HA = 0, bool NC = true, bool RG = false>
__device__ __forceinline__ void gg_tile_step(const StepArgs &a, float *sm, uint8_t *ntier, double *red, int tile,
                                             const CUtensorMap *tm = nullptr, uint64_t *bar = nullptr)
{
    constexpr bool MON = MK != 0;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    load_neighbour_tiers(a, tx, ty, ntier);
    // the copy of the FP32 neighbourhood (the common case) starts before the
    // tiers are known, so that its latency overlaps theirs; where the tile
    // turns out FP64 or its neighbourhood mixed, the copies are drained and
    // their data (in-bounds reads of the full-size FP32 store) discarded
    const bool spec = T == 32 && a.in[TIER_FP32] != nullptr;
    const bool bulk = spec && tm != nullptr && tx >= 1 && ty >= 1 && tx <= a.ntx - 2 && ty <= a.nty - 2;
    if (bulk) {
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
            mbar_arrive_expect_tx(bar, (uint32_t)(Stage<float, T, 1>::FIELD * a.nf * sizeof(float)));
            tma_load_3d(sm, tm, tx * T - Stage<float, T, 1>::O, ty * T - 1, 0, bar);
        }
    } else if (spec) {
        stage_tile_async32<T, 1, false>(a, sm, tx, ty, a.nf);
    }
    // the staging copies have landed (false: a bounded wait on the tensor
    // copy gave up -- flagged; the CTA waits once more for it and returns)
    auto spec_done = [&]() -> bool {
        if (!bulk) {
            cp_async_wait_all();
            return true;
        }
        const bool ok = mbar_wait_bounded(bar, 0);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.flags, 2);
                if (!ok) mbar_wait_bounded(bar, 0);
            }
            return false;
        }
        return true;
    };
    const int tier = a.tier_out[tile];
    __syncthreads();
    if (tier == TIER_FP64) {
        // the FP64 path reads through L1, not the staging area: the discarded
        // copies land while it computes, before the CTA exits
        if (RG && gg_partial_tile(a, T, tx, ty)) gg_tile_fp64_partial<T, REF>(a, ntier, tile, tx, ty, red);
        else gg_tile_fp64<T, REF>(a, ntier, tile, tx, ty, red);
        if (spec) spec_done();
        return;
    }
    const bool all32 = all_fp32(ntier);
    if (spec) {
        if (!spec_done()) return;
        // mixed neighbourhood: the FP32-owned slots are in place; each thread
        // overwrites its own other slots with their converted values
        if (!all32) stage_tile<float, T, 1, true, NC>(a, sm, ntier, tx, ty, 0, a.nf);
    } else if (all32) {
        stage_tile_async32<T, 1>(a, sm, tx, ty, a.nf);
    } else {
        stage_tile<float, T, 1, false, NC>(a, sm, ntier, tx, ty, 0, a.nf);
    }
    __syncthreads();
    if (RG && gg_partial_tile(a, T, tx, ty)) {  // a ragged grid's edge tile: its wrapped halo
        patch_ragged<float, T>(a, sm, tx, ty);
        __syncthreads();
    }
    if constexpr (HA != 0) {
        if (tier == TIER_HALF) {
            gg_tile_half2<T, MK, HA>(a, sm, tile, tx, ty, red);
            return;
        }
    }
    if constexpr (T == 32) {
        // the spatial range needs one reduction per field: gg_tile_lo_impl
        float *ss = sm + a.nf * Stage<float, T, 1>::FIELD;  // gg_smem_bytes reserves it
        if (!MON) {
            // 8 rows a thread when the fields come in eights (one warp a field)
            if (a.nf % 8 == 0) {
                if (tier == TIER_FP32) gg_tile_lo_rows<TIER_FP32, 8>(a, sm, ss, tile, tx, ty, red);
                else gg_tile_lo_rows<TIER_HALF, 8>(a, sm, ss, tile, tx, ty, red);
            } else {
                if (tier == TIER_FP32) gg_tile_lo_rows<TIER_FP32, 4>(a, sm, ss, tile, tx, ty, red);
                else gg_tile_lo_rows<TIER_HALF, 4>(a, sm, ss, tile, tx, ty, red);
            }
            return;
        }
        if (MK == 3 && a.nf % 8 == 0) {
            if (tier == TIER_FP32) gg_tile_lo_rows<TIER_FP32, 8, 3>(a, sm, ss, tile, tx, ty, red);
            else gg_tile_lo_rows<TIER_HALF, 8, 3>(a, sm, ss, tile, tx, ty, red);
            return;
        }
        if (MK == 3 || (MK == -1 && a.monitor_kind == 3)) {
            if (tier == TIER_FP32) gg_tile_lo_rows<TIER_FP32, 4, 3>(a, sm, ss, tile, tx, ty, red);
            else gg_tile_lo_rows<TIER_HALF, 4, 3>(a, sm, ss, tile, tx, ty, red);
            return;
        }
        if (MK == 2 || (MK == -1 && a.monitor_kind == 2)) {
            if (tier == TIER_FP32) gg_tile_lo_rows<TIER_FP32, 4, 2>(a, sm, ss, tile, tx, ty, red);
            else gg_tile_lo_rows<TIER_HALF, 4, 2>(a, sm, ss, tile, tx, ty, red);
            return;
        }
    }
    if (tier == TIER_FP32) gg_tile_lo_impl<T, TIER_FP32, MON>(a, sm, tile, tx, ty, red);
    else gg_tile_lo_impl<T, TIER_HALF, MON>(a, sm, tile, tx, ty, red);
}

// Fused all-tier step: at most 64 registers, so that four CTAs share an SM.
// The monitor steps (one in `cadence`) are separate instantiations, one per
// monitor kind MK, so the other steps' kernel carries no monitor code and
// each monitor step's kernel only its own kind's.  Half/FP32 tiles stage
// their neighbourhood in shared memory (reading it directly through L1
// measured 18.1 against 15.8 us per adaptive 1024^2 Q=8 step).
// tm: the tensor map of the step's FP32 input, valid when a.tma_stage.
template <int T, bool REF, int MK, int HA = 0, bool RG = false>
__global__ void __launch_bounds__(kThreads, 4) gg_step_kernel(StepArgs a, const __grid_constant__ CUtensorMap tm)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    __shared__ __align__(8) uint64_t bar;
    // 128-byte aligned staging (gg_smem_bytes adds the slack), as tensor copies need
    float *sm = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smraw) + 127) & ~uintptr_t(127));
    // programmatic dependent launch (gg_launch): the next step's CTAs may be
    // scheduled into the slots this grid's last wave leaves free; every CTA
    // waits for the previous grid to complete, its writes visible, before
    // its first global read (both are no-ops for a plain launch)
    pdl_trigger();
    pdl_wait();
    const int tile = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    gg_tile_step<T, REF, MK, HA, true, RG>(a, sm, ntier, red, tile, a.tma_stage ? &tm : nullptr, &bar);
}


}  // namespace amps
