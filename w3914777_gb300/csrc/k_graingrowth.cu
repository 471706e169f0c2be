// k_graingrowth.cu -- fused multi-order-parameter Allen-Cahn (grain growth) step.
//
// One CTA per tile.  All Q fields of the tile plus a 1-cell halo are staged in
// shared memory at the tile's compute precision (each cell converted from its
// owner tile's input tier), then every thread advances one column of
// T*T/256 cells for all Q fields and stores them at the tile's output tier.
// On monitor steps the epilogue also reduces the per-tile monitor metric.
//
// Reference: graingrowth/function.h:5-30 (kernel1_pure, launched once per
// field, graingrowth/purehigh.cu:31-32) and graingrowth/function.h:33-277
// (kernel1_mix with its half2 halo patching and ring write-back), generalised
// from Q=2 to Q fields with cross coefficient gamma:
//   dfd_i = 2*gamma*eta_i*sum_{j!=i} eta_j^2 + eta_i^3 - eta_i
//   eta_i' = eta_i - dt*L*(dfd_i - kappa*lap(eta_i)).
#include "amps_internal.cuh"
#include "amps_kernels.h"
#include <type_traits>

namespace amps {

template <int T, int TIER, bool REF>
__global__ void __launch_bounds__(kThreads) gg_step_kernel(StepArgs a)
{
    using CT = typename std::conditional<TIER == TIER_FP64, double, float>::type;
    constexpr int R = 1;
    using S = Stage<CT, T, R>;
    constexpr int RG = kThreads / T;  // row groups
    constexpr int RPT = T / RG;       // rows per thread
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    CT *sm = reinterpret_cast<CT *>(smraw);

    if ((int)blockIdx.x >= a.count[TIER]) return;
    const int tile = a.list[blockIdx.x];
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    load_neighbour_tiers(a, tx, ty, ntier);
    __syncthreads();
    stage_tile<CT, T, R>(a, sm, ntier, tx, ty, 0, a.nf);
    __syncthreads();

    const int col = threadIdx.x % T;
    const int r0 = (threadIdx.x / T) * RPT;
    const int c = S::O + col;
    const int nf = a.nf;
    const Phys &ph = a.ph;

    // sum of squares of every field at this thread's cells (FAST form)
    CT ssum[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) ssum[j] = CT(0);
    if (!REF) {
        for (int f = 0; f < nf; ++f) {
#pragma unroll
            for (int j = 0; j < RPT; ++j) {
                const CT v = S::at(sm, f, r0 + j + R, c);
                ssum[j] = fma(v, v, ssum[j]);
            }
        }
    }

    const CT dtm = CT(ph.dt * ph.mobil);
    const CT g2 = CT(2.0 * ph.gamma);
    const CT kap = CT(ph.grcoef);
    const CT inv = CT(ph.inv_dxdy);
    const int64_t gbase = (int64_t)(ty * T + r0) * a.nx + tx * T + col;
    double metric = 0.0;
    MonAcc mon;

    for (int f = 0; f < nf; ++f) {
        const bool mon_f = a.monitor_now && (a.mfield < 0 || a.mfield == f);
        if (mon_f) mon_reset(a, mon);
        CT w[RPT + 2][3];
#pragma unroll
        for (int j = 0; j < RPT + 2; ++j) {
            w[j][0] = S::at(sm, f, r0 + j, c - 1);
            w[j][1] = S::at(sm, f, r0 + j, c);
            w[j][2] = S::at(sm, f, r0 + j, c + 1);
        }
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const CT *rd = w[j], *rc = w[j + 1], *ru = w[j + 2];
            const CT e = rc[1];
            CT out;
            if (REF) {
                // graingrowth/function.h:20-23, rounding every operation as written
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
                    const double v = S::at(sm, b, r0 + j + R, c);
                    const double s2 = __dmul_rn(v, v);
                    sum = first ? s2 : __dadd_rn(sum, s2);
                    first = false;
                }
                const double dfd = __dsub_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0 * ph.gamma, e), sum), pow((double)e, 3.0)), e);
                out = (CT)__dsub_rn(e, __dmul_rn(ph.dt * ph.mobil, __dsub_rn(dfd, __dmul_rn(ph.grcoef, lap))));
            } else {
                CT s;
                if (a.stencil == 0) s = (rd[0] + rd[1] + rd[2]) + (rc[0] + rc[2]) + (ru[0] + ru[1] + ru[2]) - CT(8) * e;
                else s = (rc[0] + rc[2]) + (rd[1] + ru[1]) - CT(4) * e;
                const CT lap = s * inv;
                const CT e2 = e * e;
                const CT dfd = e * fma(g2, ssum[j] - e2, e2 - CT(1));
                out = fma(-dtm, fma(-kap, lap, dfd), e);
            }
            const int64_t gidx = (int64_t)f * a.n + gbase + (int64_t)j * a.nx;
            store_tier<TIER>(a, gidx, out);
            if (mon_f)
                mon_add<T>(a, mon, a.mfield < 0 ? f : 0, tile, r0 + j, col, gbase + (int64_t)j * a.nx,
                           (double)round_to_tier<TIER>(out));
        }
        if (mon_f) metric = mon_finish(a, mon, red, metric);
    }
    if (a.monitor_now && threadIdx.x == 0) a.metric[tile] = metric;
}

template <int T, int TIER, bool REF> static size_t gg_smem(int nf)
{
    using CT = typename std::conditional<TIER == TIER_FP64, double, float>::type;
    return (size_t)nf * Stage<CT, T, 1>::FIELD * sizeof(CT);
}

template <int T, int TIER, bool REF>
static cudaError_t gg_launch_t(const StepArgs &a, int grid, cudaStream_t s)
{
    const size_t smem = gg_smem<T, TIER, REF>(a.nf);
    gg_step_kernel<T, TIER, REF><<<grid, kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

size_t gg_smem_bytes(int tile, int tier, int nf)
{
    const int T = tile;
    if (T == 32) return tier == TIER_FP64 ? gg_smem<32, TIER_FP64, false>(nf) : gg_smem<32, TIER_FP32, false>(nf);
    return tier == TIER_FP64 ? gg_smem<16, TIER_FP64, false>(nf) : gg_smem<16, TIER_FP32, false>(nf);
}

cudaError_t gg_launch(int tile, int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s)
{
#define AMPS_GG(TT)                                                                 \
    switch (tier) {                                                                 \
    case TIER_HALF: return gg_launch_t<TT, TIER_HALF, false>(a, grid, s);           \
    case TIER_FP32: return gg_launch_t<TT, TIER_FP32, false>(a, grid, s);           \
    default:                                                                        \
        return ref ? gg_launch_t<TT, TIER_FP64, true>(a, grid, s)                   \
                   : gg_launch_t<TT, TIER_FP64, false>(a, grid, s);                 \
    }
    if (tile == 32) { AMPS_GG(32) }
    AMPS_GG(16)
#undef AMPS_GG
}

cudaError_t gg_prepare(int tile, int tier, bool ref)
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
#define AMPS_GGP(TT)                                                                              \
    switch (tier) {                                                                               \
    case TIER_HALF: return cudaFuncSetAttribute(gg_step_kernel<TT, TIER_HALF, false>, attr, lim);  \
    case TIER_FP32: return cudaFuncSetAttribute(gg_step_kernel<TT, TIER_FP32, false>, attr, lim);  \
    default:                                                                                      \
        return ref ? cudaFuncSetAttribute(gg_step_kernel<TT, TIER_FP64, true>, attr, lim)         \
                   : cudaFuncSetAttribute(gg_step_kernel<TT, TIER_FP64, false>, attr, lim);       \
    }
    if (tile == 32) { AMPS_GGP(32) }
    AMPS_GGP(16)
#undef AMPS_GGP
}

}  // namespace amps
