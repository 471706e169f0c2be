// k_graingrowth.cu -- fused multi-order-parameter Allen-Cahn (grain growth) step.
//
// One launch per step covers every tile; each CTA advances one tile in that
// tile's own tier.  Half and FP32 tiles stage all Q fields plus a 1-cell halo
// in shared memory as float (each cell converted from its owner tile's input
// tier) and store at half/float; FP64 tiles are bound by the FP64 pipes, so
// they skip the staging and read their neighbourhood straight through L1.
// Shared memory is therefore sized by the float staging alone.  On monitor
// steps the epilogue reduces the per-tile metric.
//
// Reference: graingrowth/function.h:5-30 (kernel1_pure, launched once per
// field, graingrowth/purehigh.cu:31-32) and graingrowth/function.h:33-277
// (kernel1_mix with its half2 halo patching and ring write-back), generalised
// from Q=2 to Q fields with cross coefficient gamma:
//   dfd_i = 2*gamma*eta_i*sum_{j!=i} eta_j^2 + eta_i^3 - eta_i
//   eta_i' = eta_i - dt*L*(dfd_i - kappa*lap(eta_i)).
#include "amps_internal.cuh"
#include "amps_kernels.h"

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
    const int64_t gbase = (int64_t)(ty * T + row) * a.nx + tx * T + c0;
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
#pragma unroll
            for (int k = 0; k < CPT; ++k)
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
template <int TIER, int RPT, int MK = 0>
__device__ __forceinline__ void gg_tile_lo_rows(const StepArgs &a, const float *sm, float *ss, int tile, int tx,
                                                int ty, double *red)
{
    constexpr int T = 32, CPT = 4, GPR = T / CPT;
    using S = Stage<float, T, 1>;
    float *smm = const_cast<float *>(sm);
    const int nf = a.nf;
    {
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
    }
    __syncthreads();
    static_assert(T % RPT == 0 && (T / RPT) * GPR * RPT == kThreads, "RPT groups of T/RPT x GPR threads");
    const int group = threadIdx.x / (kThreads / RPT), t = threadIdx.x % (kThreads / RPT);
    const int r0 = RPT * (t / GPR), c0 = (t % GPR) * CPT;  // tile-local rows r0 .. r0+RPT-1
    const Phys &ph = a.ph;
    const float dtm = ph.gg_dtm, g2 = ph.gg_g2, kap = ph.gg_kap, inv = ph.gg_inv;
    const int64_t gbase = (int64_t)(ty * T + r0) * a.nx + tx * T + c0;
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
            const int64_t gi = gbase + (int64_t)i * a.nx;
            store_cells<TIER, CPT>(a, (int64_t)f * a.n + gi, out);
            if constexpr (MK != 0) {
                if (mon_f) {
#pragma unroll
                    for (int k = 0; k < CPT; ++k)
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
// its owner tile's input tier.
template <int T>
__device__ __forceinline__ double ld_nb64(const StepArgs &a, const uint8_t *nt, int f, int x0, int y0, int ly, int lx)
{
    const int gy = bc_map(y0 + ly, a.ny, a.bc), gx = bc_map(x0 + lx, a.nx, a.bc);
    const int cls = (ly < 0 ? 0 : (ly < T ? 3 : 6)) + (lx < 0 ? 0 : (lx < T ? 1 : 2));
    return load_tier<double>(a, nt[cls], (int64_t)f * a.n + (int64_t)gy * a.nx + gx);
}

// FP64 tile: direct loads through L1 with a rolling 3-row window, FP64
// arithmetic; REF keeps the reference's expression order and rounding
// (graingrowth/function.h:20-23).
template <int T, bool REF>
__device__ __forceinline__ void gg_tile_fp64(const StepArgs &a, const uint8_t *nt, int tile, int tx, int ty, double *red)
{
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
                const double v = ld_nb64<T>(a, nt, f, x0, y0, r0 + j, col);
                ssum[j] = fma(v, v, ssum[j]);
            }
    const int64_t gbase = (int64_t)(y0 + r0) * a.nx + x0 + col;
    double metric = 0.0;
    MonAcc mon;
    for (int f = 0; f < nf; ++f) {
        const bool mon_f = a.monitor_now && (a.mfield < 0 || a.mfield == f);
        const int mslot = a.mfield < 0 ? f : 0;
        if (mon_f) mon_reset(a, mon);
        double rd[3], rc[3], ru[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            rd[k] = ld_nb64<T>(a, nt, f, x0, y0, r0 - 1, col + k - 1);
            rc[k] = ld_nb64<T>(a, nt, f, x0, y0, r0, col + k - 1);
        }
#pragma unroll 1
        for (int j = 0; j < RPT; ++j) {
#pragma unroll
            for (int k = 0; k < 3; ++k) ru[k] = ld_nb64<T>(a, nt, f, x0, y0, r0 + j + 1, col + k - 1);
            const int64_t g = gbase + (int64_t)j * a.nx;
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
                    const double v = ld_nb64<T>(a, nt, b, x0, y0, r0 + j, col);
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
            if (mon_f) mon_add<T>(a, mon, mslot, tile, r0 + j, col, g, out, e, snapv);
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
template <int T, bool REF, int MK>
__device__ __forceinline__ void gg_tile_step(const StepArgs &a, float *sm, uint8_t *ntier, double *red, int tile)
{
    constexpr bool MON = MK != 0;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    load_neighbour_tiers(a, tx, ty, ntier);
    // the copy of the FP32 neighbourhood (the common case) starts before the
    // tiers are known, so that its latency overlaps theirs; where the tile
    // turns out FP64 or its neighbourhood mixed, the copies are drained and
    // their data (in-bounds reads of the full-size FP32 store) discarded
    const bool spec = T == 32 && a.in[TIER_FP32] != nullptr;
    if (spec) stage_tile_async32<T, 1, false>(a, sm, tx, ty, a.nf);
    const int tier = a.tier_out[tile];
    __syncthreads();
    if (tier == TIER_FP64) {
        // the FP64 path reads through L1, not the staging area: the discarded
        // copies land while it computes, before the CTA exits
        gg_tile_fp64<T, REF>(a, ntier, tile, tx, ty, red);
        if (spec) cp_async_wait_all();
        return;
    }
    const bool all32 = all_fp32(ntier);
    if (spec) {
        cp_async_wait_all();
        // mixed neighbourhood: the FP32-owned slots are in place; each thread
        // overwrites its own other slots with their converted values
        if (!all32) stage_tile<float, T, 1, true>(a, sm, ntier, tx, ty, 0, a.nf);
    } else if (all32) {
        stage_tile_async32<T, 1>(a, sm, tx, ty, a.nf);
    } else {
        stage_tile<float, T, 1>(a, sm, ntier, tx, ty, 0, a.nf);
    }
    __syncthreads();
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

// gg_tile_step out of line, for callers whose StepArgs live in shared
// memory (inlined, their loads are hoisted and spill).
template <int T, bool REF, bool MON>
__device__ __noinline__ void gg_tile_step_call(const StepArgs &a, float *sm, uint8_t *ntier, double *red, int tile)
{
    gg_tile_step<T, REF, MON ? -1 : 0>(a, sm, ntier, red, tile);
}

// Fused all-tier step: at most 64 registers, so that four CTAs share an SM.
// The monitor steps (one in `cadence`) are separate instantiations, one per
// monitor kind MK, so the other steps' kernel carries no monitor code and
// each monitor step's kernel only its own kind's.  Half/FP32 tiles stage
// their neighbourhood in shared memory (reading it directly through L1
// measured 18.1 against 15.8 us per adaptive 1024^2 Q=8 step).
template <int T, bool REF, int MK>
__global__ void __launch_bounds__(kThreads, 4) gg_step_kernel(StepArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    float *sm = reinterpret_cast<float *>(smraw);
    // programmatic dependent launch (gg_launch): the next step's CTAs may be
    // scheduled into the slots this grid's last wave leaves free; every CTA
    // waits for the previous grid to complete, its writes visible, before
    // its first global read (both are no-ops for a plain launch)
    pdl_trigger();
    pdl_wait();
    const int tile = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    gg_tile_step<T, REF, MK>(a, sm, ntier, red, tile);
}

// All-FP64 step (plain FP64 mode): the FP64 neighbourhood is staged in
// shared memory, which suits the FP64-pipe-bound arithmetic better than the
// fused kernel's direct loads.
template <int T, bool REF>
__global__ void __launch_bounds__(kThreads) gg_step_f64_kernel(StepArgs a)
{
    using S = Stage<double, T, 1>;
    constexpr int RPT = T * T / kThreads;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    double *sm = reinterpret_cast<double *>(smraw);
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    load_neighbour_tiers(a, tx, ty, ntier);
    __syncthreads();
    stage_tile<double, T, 1>(a, sm, ntier, tx, ty, 0, a.nf);
    __syncthreads();
    const int col = threadIdx.x % T;
    const int r0 = (threadIdx.x / T) * RPT;
    const int c = S::O + col;
    const int nf = a.nf;
    const Phys &ph = a.ph;
    double ssum[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) ssum[j] = 0.0;
    if (!REF)
        for (int f = 0; f < nf; ++f)
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const double v = S::at(sm, f, r0 + j + 1, c);
                ssum[j] = fma(v, v, ssum[j]);
            }
    const int64_t gbase = (int64_t)(ty * T + r0) * a.nx + tx * T + col;
    for (int f = 0; f < nf; ++f) {
        double w[RPT + 2][3];
#pragma unroll
        for (int j = 0; j < RPT + 2; ++j) {
            w[j][0] = S::at(sm, f, r0 + j, c - 1);
            w[j][1] = S::at(sm, f, r0 + j, c);
            w[j][2] = S::at(sm, f, r0 + j, c + 1);
        }
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const double *rd = w[j], *rc = w[j + 1], *ru = w[j + 2];
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
                    const double v = S::at(sm, b, r0 + j + 1, c);
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
                const double dfd = e * fma(2.0 * ph.gamma, ssum[j] - e2, e2 - 1.0);
                out = fma(-(ph.dt * ph.mobil), fma(-ph.grcoef, lap, dfd), e);
            }
            ((double *)a.out[TIER_FP64])[(int64_t)f * a.n + gbase + (int64_t)j * a.nx] = out;
        }
    }
}

// tier: TIER_FP64 selects the all-FP64 staged kernel; anything else the fused one.
size_t gg_smem_bytes(int tile, int tier, int nf)
{
    if (tier == TIER_FP64)
        return (size_t)nf * (tile == 32 ? Stage<double, 32, 1>::FIELD : Stage<double, 16, 1>::FIELD) * sizeof(double);
    // 32^2: + the sum-of-squares tile of gg_tile_lo_4row
    if (tile == 32) return ((size_t)nf * Stage<float, 32, 1>::FIELD + 32 * 32) * sizeof(float);
    return (size_t)nf * Stage<float, 16, 1>::FIELD * sizeof(float);
}

template <typename K> static cudaError_t launch_pdl(K kernel, int grid, size_t smem, cudaStream_t s, const StepArgs &a)
{
    return launch_kernel(kernel, grid, smem, s, true, a);
}

cudaError_t gg_launch(int tile, int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s)
{
    const size_t smem = gg_smem_bytes(tile, tier, a.nf);
#define AMPS_GGL(K, TT)                                                         \
    do {                                                                        \
        if (ref) K<TT, true><<<grid, kThreads, smem, s>>>(a);                   \
        else K<TT, false><<<grid, kThreads, smem, s>>>(a);                      \
    } while (0)
#define AMPS_GGM(TT)                                                                                  \
    do {                                                                                              \
        switch (a.monitor_now ? a.monitor_kind : 0) {                                                 \
        case 0:                                                                                       \
            if (ref) return launch_pdl(gg_step_kernel<TT, true, 0>, grid, smem, s, a);                \
            return launch_pdl(gg_step_kernel<TT, false, 0>, grid, smem, s, a);                        \
        case 1:                                                                                       \
            if (ref) return launch_pdl(gg_step_kernel<TT, true, 1>, grid, smem, s, a);                \
            return launch_pdl(gg_step_kernel<TT, false, 1>, grid, smem, s, a);                        \
        case 2:                                                                                       \
            if (ref) return launch_pdl(gg_step_kernel<TT, true, 2>, grid, smem, s, a);                \
            return launch_pdl(gg_step_kernel<TT, false, 2>, grid, smem, s, a);                        \
        default:                                                                                      \
            if (ref) return launch_pdl(gg_step_kernel<TT, true, 3>, grid, smem, s, a);                \
            return launch_pdl(gg_step_kernel<TT, false, 3>, grid, smem, s, a);                        \
        }                                                                                             \
    } while (0)
    if (tier == TIER_FP64) {
        if (tile == 32) AMPS_GGL(gg_step_f64_kernel, 32);
        else AMPS_GGL(gg_step_f64_kernel, 16);
    } else {
        if (tile == 32) AMPS_GGM(32);
        else AMPS_GGM(16);
    }
#undef AMPS_GGL
#undef AMPS_GGM
    return cudaGetLastError();
}

cudaError_t gg_prepare(int tile, int tier, bool ref)
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (tier == TIER_FP64) {
        if (tile == 32) return ref ? cudaFuncSetAttribute(gg_step_f64_kernel<32, true>, attr, lim)
                                   : cudaFuncSetAttribute(gg_step_f64_kernel<32, false>, attr, lim);
        return ref ? cudaFuncSetAttribute(gg_step_f64_kernel<16, true>, attr, lim)
                   : cudaFuncSetAttribute(gg_step_f64_kernel<16, false>, attr, lim);
    }
    cudaError_t e = cudaSuccess;
#define AMPS_GGP(TT, MK)                                                                                     \
    if (e == cudaSuccess)                                                                                    \
        e = ref ? cudaFuncSetAttribute(gg_step_kernel<TT, true, MK>, attr, lim)                              \
                : cudaFuncSetAttribute(gg_step_kernel<TT, false, MK>, attr, lim)
    if (tile == 32) {
        AMPS_GGP(32, 0); AMPS_GGP(32, 1); AMPS_GGP(32, 2); AMPS_GGP(32, 3);
    } else {
        AMPS_GGP(16, 0); AMPS_GGP(16, 1); AMPS_GGP(16, 2); AMPS_GGP(16, 3);
    }
#undef AMPS_GGP
    return e;
}

// Persistent, TMA-pipelined fused step for 32x32 tiles (nf <= kTmaMaxFields).
// Each CTA walks tiles blockIdx.x, +gridDim.x, ...  A tile whose input
// neighbourhood is entirely FP32 and inside the domain (no wrap, no mirror)
// is fetched by one 3-D tensor copy -- all nf fields, 34 rows x 40 columns --
// straight into the float staging layout, issued one tile ahead into the
// other of two buffers so that the copy overlaps the current tile's
// arithmetic.  Every other tile (domain edge, a neighbour at another tier,
// FP64 output) takes the generic staged / direct path.
template <bool REF>
__global__ void __launch_bounds__(kThreads, 2)
    gg_step_tma_kernel(const __grid_constant__ CUtensorMap tm, StepArgs a, int bufstride)
{
    constexpr int T = 32;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    __shared__ int fast_s[2];
    float *buf0 = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const int ntiles = a.ntx * a.nty;
    const uint32_t bytes = 40u * 34u * (uint32_t)a.nf * 4u;
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // thread 0 only: can tile t come by tensor copy?
    auto is_fast = [&](int t) -> int {
        const int tx = t % a.ntx, ty = t / a.ntx;
        if (tx < 1 || ty < 1 || tx > a.ntx - 2 || ty > a.nty - 2) return 0;
        if (a.tier_out[t] == TIER_FP64) return 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
                if (a.tier_in[(ty + dy) * a.ntx + tx + dx] != TIER_FP32) return 0;
        return 1;
    };
    auto issue = [&](int t, int b) {
        const int tx = t % a.ntx, ty = t / a.ntx;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&mbar[b], bytes);
        tma_load_3d(buf0 + b * bufstride, &tm, tx * T - 4, ty * T - 1, 0, &mbar[b]);
    };
    uint32_t ph0 = 0, ph1 = 0;
    int t = blockIdx.x;
    if (threadIdx.x == 0) {
        const int f = t < ntiles ? is_fast(t) : 0;
        if (f) issue(t, 0);
        fast_s[0] = f;
    }
    __syncthreads();
    for (int i = 0; t < ntiles; ++i, t += gridDim.x) {
        const int b = i & 1;
        const int tn = t + gridDim.x;
        if (threadIdx.x == 0) {  // prefetch the next tile into the other buffer (free since the last barrier)
            const int f = tn < ntiles ? is_fast(tn) : 0;
            if (f) issue(tn, b ^ 1);
            fast_s[b ^ 1] = f;
        }
        const int fast = fast_s[b];
        const int tx = t % a.ntx, ty = t / a.ntx;
        const int tier = a.tier_out[t];
        float *sm = buf0 + b * bufstride;
        if (fast) {
            const uint32_t par = b ? ph1 : ph0;
            const bool ok = mbar_wait_bounded(&mbar[b], par);
            if (b) ph1 ^= 1u; else ph0 ^= 1u;
            if (__syncthreads_or(!ok)) {
                // Give up: flag it, then give both copies that may still be in
                // flight -- this buffer's (the one that timed out) and the
                // prefetch into the other -- a second bounded wait before the
                // CTA leaves, so that neither lands in shared memory after it.
                // A copy that never completes cannot be recovered here: the
                // flag makes the host report AMPS_ERR_TIMEOUT.
                // The CTA's shared memory stays allocated while thread 0 waits.
                if (threadIdx.x == 0) {
                    atomicOr(a.flags, 2);
                    if (!ok) mbar_wait_bounded(&mbar[b], par);
                    if (fast_s[b ^ 1]) mbar_wait_bounded(&mbar[b ^ 1], b ? ph0 : ph1);
                }
                return;
            }
            if (tier == TIER_FP32) gg_tile_lo<T, TIER_FP32>(a, sm, t, tx, ty, red);
            else gg_tile_lo<T, TIER_HALF>(a, sm, t, tx, ty, red);
        } else {
            load_neighbour_tiers(a, tx, ty, ntier);
            __syncthreads();
            if (tier == TIER_FP64) {
                gg_tile_fp64<T, REF>(a, ntier, t, tx, ty, red);
            } else {
                stage_tile<float, T, 1>(a, sm, ntier, tx, ty, 0, a.nf);
                __syncthreads();
                if (tier == TIER_FP32) gg_tile_lo<T, TIER_FP32>(a, sm, t, tx, ty, red);
                else gg_tile_lo<T, TIER_HALF>(a, sm, t, tx, ty, red);
            }
        }
        fence_proxy_async_smem();  // this buffer's reads/writes before its next tensor copy
        __syncthreads();
    }
    // a prefetch is issued only for tiles the loop reaches, so nothing is in flight here
}

int gg_tma_buffer_floats(int nf) { return ((nf * Stage<float, 32, 1>::FIELD * 4 + 1023) / 1024) * 256; }
size_t gg_tma_smem_bytes(int nf) { return (size_t)2 * gg_tma_buffer_floats(nf) * 4 + 1024; }

cudaError_t gg_launch_tma(bool ref, const CUtensorMap &tm, const StepArgs &a, int grid, cudaStream_t s)
{
    const int bs = gg_tma_buffer_floats(a.nf);
    const size_t smem = gg_tma_smem_bytes(a.nf);
    if (ref) gg_step_tma_kernel<true><<<grid, kThreads, smem, s>>>(tm, a, bs);
    else gg_step_tma_kernel<false><<<grid, kThreads, smem, s>>>(tm, a, bs);
    return cudaGetLastError();
}

cudaError_t gg_prepare_tma(bool ref, int nf, int *blocks_per_sm)
{
    const size_t smem = gg_tma_smem_bytes(nf);
    cudaError_t e = ref ? cudaFuncSetAttribute(gg_step_tma_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                        : cudaFuncSetAttribute(gg_step_tma_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return ref ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gg_step_tma_kernel<true>, kThreads, smem)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gg_step_tma_kernel<false>, kThreads, smem);
}

// Ensemble step: persistent CTAs take (member, tile) work items from a
// global counter; items are ordered by cost (most fields first), so the
// dynamic queue approximates longest-first scheduling across members of
// different sizes and field counts.  A tile is gg_tile_step, the fused
// kernel's per-tile code (same results); the member's arguments are
// copied into shared memory when the member changes.  No waits: the counter
// only hands out indices, and the last CTA to finish resets it.
template <int T, bool REF, bool MON>
__global__ void __launch_bounds__(kThreads, 2)
    gg_ens_kernel(const StepArgs *__restrict__ table, const int2 *__restrict__ items, int nitems, int *queue)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    __shared__ __align__(16) StepArgs sa;
    __shared__ int sw;
    float *sm = reinterpret_cast<float *>(smraw);
    static_assert(sizeof(StepArgs) % 4 == 0, "StepArgs copied as 32-bit words");
    int member = -1;
    for (;;) {
        if (threadIdx.x == 0) sw = atomicAdd(&queue[0], 1);
        __syncthreads();
        const int w = sw;
        if (w >= nitems) break;
        const int2 it = items[w];
        if (it.x != member) {
            const int *src = reinterpret_cast<const int *>(table + it.x);
            int *dst = reinterpret_cast<int *>(&sa);
            for (int k = threadIdx.x; k < (int)(sizeof(StepArgs) / 4); k += kThreads) dst[k] = src[k];
            member = it.x;
        }
        __syncthreads();
        gg_tile_step_call<T, REF, MON>(sa, sm, ntier, red, it.y);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&queue[1], 1) == (int)gridDim.x - 1) {
            queue[0] = 0;
            queue[1] = 0;
            __threadfence();
        }
    }
}

// staging for the member with the most fields
size_t gg_ens_smem_bytes(int tile, int max_nf) { return gg_smem_bytes(tile, -1, max_nf); }

cudaError_t gg_prepare_ens(int tile, bool ref, int max_nf, int *blocks_per_sm)
{
    const size_t smem = gg_ens_smem_bytes(tile, max_nf);
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaSuccess;
#define AMPS_GGE(TT, RR)                                                                                   \
    do {                                                                                                   \
        e = cudaFuncSetAttribute(gg_ens_kernel<TT, RR, false>, attr, (int)smem);                           \
        if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_ens_kernel<TT, RR, true>, attr, (int)smem);      \
        if (e != cudaSuccess) return e;                                                                    \
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gg_ens_kernel<TT, RR, false>, kThreads, smem); \
    } while (0)
    if (tile == 32) {
        if (ref) AMPS_GGE(32, true);
        AMPS_GGE(32, false);
    }
    if (ref) AMPS_GGE(16, true);
    AMPS_GGE(16, false);
#undef AMPS_GGE
}

cudaError_t gg_launch_ens(int tile, bool ref, bool monitor, const StepArgs *table, const int2 *items, int nitems,
                          int *queue, int grid, size_t smem, cudaStream_t s)
{
#define AMPS_GGEL(TT, RR)                                                                                      \
    do {                                                                                                       \
        if (monitor) gg_ens_kernel<TT, RR, true><<<grid, kThreads, smem, s>>>(table, items, nitems, queue);    \
        else gg_ens_kernel<TT, RR, false><<<grid, kThreads, smem, s>>>(table, items, nitems, queue);           \
    } while (0)
    if (tile == 32) {
        if (ref) AMPS_GGEL(32, true);
        else AMPS_GGEL(32, false);
    } else {
        if (ref) AMPS_GGEL(16, true);
        else AMPS_GGEL(16, false);
    }
#undef AMPS_GGEL
    return cudaGetLastError();
}

}  // namespace amps
