// k_sintering.cu -- fused solid-state sintering step: Cahn-Hilliard density c
// plus one Allen-Cahn order parameter per particle.
//
// The reference runs four kernels per step with full-size intermediates
// (sintering/function.h:51-79 con1_pure: mu; :80-108 con2_pure: c update;
// :110-159 phi1/phi2_pure: eta updates; sequenced in sintering/main.cu:136-147).
// Here one CTA per tile stages c with a 2-cell halo and every eta with a
// 1-cell halo, computes the chemical potential mu on the tile plus a 1-cell
// ring (phase A), then c' from lap(mu) and every eta' from c' and the old
// etas (phase B) -- the reference's operator splitting, in one pass.
// Generalised to N particles: sum_{i<j} 2 eta_i eta_j for the grain-boundary
// mobility term (the reference's 2*eta1*eta2, sintering/function.h:97) and
// sums over all eta in the bulk terms.
#include "amps_internal.cuh"
#include "amps_kernels.h"
#include <type_traits>

namespace amps {

// ---- per-cell arithmetic (non-reference order), shared by the whole-tile
// and the row-band paths.  C points at a cell's c with row stride cs; E at the
// cell's eta_0, field stride es, row stride rs.

// Chemical potential mu at one cell (sintering/function.h:67-71), in MT.
template <typename CT, typename MT>
__device__ __forceinline__ MT sint_mu(const CT *C, int cs, const CT *E, int es, int np, const Phys &ph)
{
    const CT cc = C[0];
    MT lap, s2 = 0, s3 = 0;
    bool exact = false;
    if constexpr (sizeof(MT) == 8 && sizeof(CT) == 4) {
        // double mu from float inputs.  Where c and every eta are 0 or 1
        // (the bulk), the sums below are small integers, exact in float:
        // form them there and keep the FP64 pipe for the other cells.
        // The results are the double path's to the bit.
        bool bin = (cc == 0.f || cc == 1.f);
        float s2f = 0.f, s3f = 0.f;
        for (int k = 0; k < np; ++k) {
            const float e = E[k * es];
            bin &= (e == 0.f || e == 1.f);
            const float e2 = e * e;
            s2f += e2;
            s3f = fmaf(e2, e, s3f);
        }
        const float csum = C[-1] + C[1] + C[-cs] + C[cs];
        bin &= (C[-1] == 0.f || C[-1] == 1.f) && (C[1] == 0.f || C[1] == 1.f) && (C[-cs] == 0.f || C[-cs] == 1.f) &&
               (C[cs] == 0.f || C[cs] == 1.f);
        if (bin) {
            exact = true;
            s2 = s2f;
            s3 = s3f;
            lap = ((MT)csum - MT(4) * (MT)cc) * kc<MT>(ph, SN_INV);
        }
    }
    if (!exact) {
        lap = ((MT)C[-1] + (MT)C[1] + (MT)C[-cs] + (MT)C[cs] - MT(4) * (MT)cc) * kc<MT>(ph, SN_INV);
        for (int k = 0; k < np; ++k) {
            // FP64 inputs: a +0 order parameter adds +0 to either sum, which
            // never holds -0 (float inputs: the test costs more than the arithmetic)
            const CT ek = E[k * es];
            if (sizeof(CT) == 8 && pos_zero(ek)) continue;
            const MT e = ek;
            const MT e2 = e * e;
            s2 += e2;
            s3 = fma(e2, e, s3);
        }
    }
    const MT c1 = MT(1) - (MT)cc;
    const MT A2 = kc<MT>(ph, SN_A2);
    const MT dfdc = kc<MT>(ph, SN_B) * (MT(2) * (MT)cc + MT(4) * s3 - MT(6) * s2) + A2 * (MT)cc * c1 * (c1 - (MT)cc);
    return dfdc - kc<MT>(ph, SN_HCM) * lap;
}

// c' at one cell (sintering/function.h:90-100) from the mu region M (row
// stride ms, M at the cell) and the old etas; s2f: sum of eta^2 at the cell.
template <typename CT, typename MT>
__device__ __forceinline__ CT sint_c_new(CT cc, const MT *M, int ms, const CT *E, int es, int np, const Phys &ph,
                                         CT &s2f)
{
    const MT lapm = (M[-1] + M[1] + M[-ms] + M[ms] - MT(4) * M[0]) * kc<MT>(ph, SN_INV);
    const CT phi = cc * cc * cc * fma(CT(6) * cc, cc, CT(10) - CT(15) * cc);
    CT se = 0;
    s2f = 0;
    for (int k = 0; k < np; ++k) {
        const CT e = E[k * es];
        if (sizeof(CT) == 8 && pos_zero(e)) continue;  // adds +0 to sums that never hold -0
        se += e;
        s2f = fma(e, e, s2f);
    }
    const CT sum = se * se - s2f;  // sum_{i != j} eta_i eta_j
    const CT mob = kc<CT>(ph, SN_DVOL) * phi + kc<CT>(ph, SN_DVAP) * (CT(1) - phi) +
                   kc<CT>(ph, SN_DSUR) * cc * (CT(1) - cc) + kc<CT>(ph, SN_DGRB) * sum;
    const CT v = (CT)((MT)cc + (MT)(kc<CT>(ph, SN_DT) * mob) * lapm);
    return v >= CT(1) ? CT(1) : (v < CT(0) ? CT(0) : v);
}

// eta' of one particle at one cell (sintering/function.h:126-131); Ep at the
// cell's eta, row stride rs.
template <typename CT>
__device__ __forceinline__ CT sint_eta_new(const CT *Ep, int rs, CT cn, CT s2f, const Phys &ph)
{
    const CT e = Ep[0];
    if (sizeof(CT) == 8 && pos_zero(e) && pos_zero(Ep[-1]) && pos_zero(Ep[1]) && pos_zero(Ep[-rs]) &&
        pos_zero(Ep[rs])) {
        // a particle absent from the whole stencil stays absent: below, lap
        // is +0, dfd and the inner term signed zeros, and v = -DTL*(+-0) + (+0)
        // = +0 -- the same bits, without the arithmetic
        return CT(0);
    }
    const CT lap = (Ep[-1] + Ep[1] + Ep[-rs] + Ep[rs] - CT(4) * e) * kc<CT>(ph, SN_INV);
    const CT dfd = kc<CT>(ph, SN_B12) * e * (s2f + (CT(1) - cn) - e * (CT(2) - cn));
    const CT v = fma(-kc<CT>(ph, SN_DTL), fma(-kc<CT>(ph, SN_HCK), lap, dfd), e);
    return v >= CT(1) ? CT(1) : (v < CT(0) ? CT(0) : v);
}

// One tile of one step at tier TIER (smraw: the kernel's dynamic shared
// memory, sint_smem<T, TIER, MU64> bytes; red / ntier: its static scratch).
template <int T, int TIER, bool REF, bool MU64>
__device__ __forceinline__ void sint_tile(const StepArgs &a, unsigned char *smraw, double *red, uint8_t *ntier,
                                          int tile)
{
    using CT = typename std::conditional<TIER == TIER_FP64, double, float>::type;
    using MT = typename std::conditional<MU64, double, CT>::type;  // type of mu and lap(mu)
    using SC = Stage<CT, T, 2>;
    using SE = Stage<CT, T, 1>;
    constexpr int E = T + 2;
    MT *mu = reinterpret_cast<MT *>(smraw);                       // [E*E]
    CT *smc = reinterpret_cast<CT *>(smraw + sizeof(MT) * E * E);  // c, 2-cell halo
    CT *sme = smc + SC::FIELD;                                     // etas, 1-cell halo
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int x0 = tx * T, y0 = ty * T;
    const int np = a.nf - 1;
    load_neighbour_tiers(a, tx, ty, ntier);
    __syncthreads();
    stage_tile<CT, T, 2>(a, smc, ntier, tx, ty, 0, 1);
    stage_tile<CT, T, 1>(a, sme, ntier, tx, ty, 1, np);
    __syncthreads();
    const Phys &ph = a.ph;

    // phase A: mu on the tile + ring (sintering/function.h:67-71)
    for (int u = threadIdx.x; u < E * E; u += kThreads) {
        int i = u % E - 1, j = u / E - 1;
        if (a.bc != 0) {
            i = bc_map(x0 + i, a.nx, 1) - x0;
            j = bc_map(y0 + j, a.ny, 1) - y0;
        }
        const CT *C = &SC::at(smc, 0, j + 2, i + SC::O);
        const CT cc = C[0];
        MT m;
        if (REF) {
            const double lap = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(C[-1], C[1]), C[-SC::P]), C[SC::P]),
                                                   __dmul_rn(4.0, cc)), ph.dxdy);
            double e0 = SE::at(sme, 0, j + 1, i + SE::O);
            double s2 = __dmul_rn(e0, e0), s3 = cube_rn(e0);
            for (int k = 1; k < np; ++k) {
                const double e = SE::at(sme, k, j + 1, i + SE::O);
                s2 = __dadd_rn(s2, __dmul_rn(e, e));
                s3 = __dadd_rn(s3, cube_rn(e));
            }
            const double A2 = 2.0 * ph.A;
            const double dfdc = __dadd_rn(
                __dsub_rn(__dmul_rn(ph.B, __dsub_rn(__dadd_rn(__dmul_rn(2.0, cc), __dmul_rn(4.0, s3)), __dmul_rn(6.0, s2))),
                          __dmul_rn(__dmul_rn(A2, __dmul_rn(cc, cc)), __dsub_rn(1.0, cc))),
                __dmul_rn(__dmul_rn(A2, cc), __dmul_rn(__dsub_rn(1.0, cc), __dsub_rn(1.0, cc))));
            m = __dsub_rn(dfdc, __dmul_rn(0.5 * ph.coefm, lap));
        } else {
            m = sint_mu<CT, MT>(C, SC::P, &SE::at(sme, 0, j + 1, i + SE::O), SE::FIELD, np, ph);
        }
        mu[u] = m;
    }
    __syncthreads();

    // phase B: c' (sintering/function.h:90-100), then eta_i' (:126-131)
    double metric = 0.0;
    // half/FP32 tiles fold their float values into a float accumulator (the
    // same metric, without FP64 operations per cell)
    using MA = typename std::conditional<TIER == TIER_FP64, MonAcc, MonAccF>::type;
    MA mon;
    const bool mon_on = a.monitor_now != 0;
    if (mon_on) mon_reset(a, mon);
    for (int u = threadIdx.x; u < T * T; u += kThreads) {
        const int i = u % T, j = u / T;
        const int o = (j + 1) * E + (i + 1);
        const int64_t g = (int64_t)(y0 + j) * a.nx + x0 + i;
        const CT cc = SC::at(smc, 0, j + 2, i + SC::O);
        CT cn;
        double s2ref = 0.0;
        CT s2f = 0;
        if (REF) {
            const double lapm = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(mu[o - 1], mu[o + 1]), mu[o - E]), mu[o + E]),
                                                    __dmul_rn(4.0, mu[o])), ph.dxdy);
            const double phi = __dmul_rn(cube_rn((double)cc),
                                         __dadd_rn(__dsub_rn(10.0, __dmul_rn(15.0, cc)), __dmul_rn(6.0, __dmul_rn(cc, cc))));
            double sum = 0.0;
            for (int p = 0; p < np; ++p)
                for (int q = p + 1; q < np; ++q)
                    sum = __dadd_rn(sum, __dmul_rn(__dmul_rn(SE::at(sme, p, j + 1, i + SE::O), SE::at(sme, q, j + 1, i + SE::O)), 2.0));
            const double mob = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(ph.dvol, phi), __dmul_rn(ph.dvap, __dsub_rn(1.0, phi))),
                                                   __dmul_rn(__dmul_rn(ph.dsur, cc), __dsub_rn(1.0, cc))),
                                         __dmul_rn(ph.dgrb, sum));
            double v = __dadd_rn(cc, __dmul_rn(__dmul_rn(ph.dt, mob), lapm));
            if (v >= 1) v = 1;
            else if (v < 0) v = 0;
            cn = v;
            double e0 = SE::at(sme, 0, j + 1, i + SE::O);
            s2ref = __dmul_rn(e0, e0);
            for (int k = 1; k < np; ++k) {
                const double e = SE::at(sme, k, j + 1, i + SE::O);
                s2ref = __dadd_rn(s2ref, __dmul_rn(e, e));
            }
        } else {
            cn = sint_c_new<CT, MT>(cc, mu + o, E, &SE::at(sme, 0, j + 1, i + SE::O), SE::FIELD, np, ph, s2f);
        }
        store_tier<TIER>(a, g, cn);
        if (mon_on && a.mfield <= 0)
            mon_add<T>(a, mon, 0, tile, j, i, g, (CT)round_to_tier<TIER>(cn), cc,
                       snap_prefetch<T>(a, 0, tile, j, i, g));
        for (int k = 0; k < np; ++k) {
            const CT *Ep = &SE::at(sme, k, j + 1, i + SE::O);
            const CT e = Ep[0];
            CT en;
            if (REF) {
                const double lap = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(__dadd_rn(Ep[-1], Ep[1]), Ep[-SE::P]), Ep[SE::P]),
                                                       __dmul_rn(4.0, e)), ph.dxdy);
                const double cnd = cn;
                const double dfd = __dmul_rn(ph.B, __dadd_rn(__dadd_rn(
                    __dmul_rn(__dmul_rn(-12.0, __dmul_rn(e, e)), __dsub_rn(2.0, cnd)),
                    __dmul_rn(__dmul_rn(12.0, e), __dsub_rn(1.0, cnd))), __dmul_rn(__dmul_rn(12.0, e), s2ref)));
                double v = __dsub_rn(e, __dmul_rn(ph.dt * ph.coefl, __dsub_rn(dfd, __dmul_rn(0.5 * ph.coefk, lap))));
                if (v >= 1) v = 1;
                else if (v < 0) v = 0;
                en = v;
            } else {
                en = sint_eta_new<CT>(Ep, SE::P, cn, s2f, ph);
            }
            store_tier<TIER>(a, (int64_t)(k + 1) * a.n + g, en);
        }
    }
    if (mon_on) {
        metric = mon_finish(a, mon, red, metric);
        if (threadIdx.x == 0) a.metric[tile] = metric;
    }
}

// ---- FP64 tiles in row bands ----------------------------------------------
// An FP64 tile of a non-monitor step (non-reference order) is split into
// T / kBandRows row bands, one CTA each: 4x the parallelism on the
// latency-bound FP64 arithmetic, and ~50 KB of shared memory instead of the
// whole tile's ~176 KB, so half/FP32 CTAs share the SM.  A band stages its
// rows of c (2-cell halo) and of every eta (1-cell halo) in double, forms mu on
// its rows + a 1-cell ring, then c' and every eta' -- the whole-tile path's
// per-cell arithmetic (sint_mu, sint_c_new, sint_eta_new), so the same bits.

template <int T> struct SintBand {
    static constexpr int BR = kBandRows, NB = T / BR;
    static constexpr int W1 = T + 2, H1 = BR + 2, FE = W1 * H1;  // etas
    static constexpr int W2 = T + 4, H2 = BR + 4;                // c
    static constexpr int WM = T + 2, HM = BR + 2;                // mu
    static size_t smem(int np) { return sizeof(double) * ((size_t)np * FE + W2 * H2 + WM * HM); }
};

template <int T>
__global__ void __launch_bounds__(kThreads) sint_step_f64_band_kernel(StepArgs a)
{
    using B = SintBand<T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ uint8_t ntier[9];
    // launched programmatically after the previous step's last grid: wait
    // for it, then release the step's half/FP32 launch (FP64 launch first)
    pdl_wait();
    pdl_trigger();
    const int item = blockIdx.x / B::NB, band = blockIdx.x % B::NB;
    if (item >= a.count[TIER_FP64]) return;
    const int tile = a.list[item];
    const int np = a.nf - 1;
    double *sme = reinterpret_cast<double *>(smraw);  // [np][H1][W1]
    double *smc = sme + np * B::FE;                   // [H2][W2]
    double *mu = smc + B::W2 * B::H2;                 // [HM][WM]
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int x0 = tx * T, y0 = ty * T, ly0 = band * B::BR;
    load_neighbour_tiers(a, tx, ty, ntier);
    __syncthreads();
    stage_band<double, T, 2>(a, smc, ntier, tx, ty, ly0 - 2, B::H2, 0, 1);
    stage_band<double, T, 1>(a, sme, ntier, tx, ty, ly0 - 1, B::H1, 1, np);
    __syncthreads();
    const Phys &ph = a.ph;
    // mu on the band + ring; with zero flux an out-of-domain ring cell takes
    // the mu of the cell it mirrors, which lies in the same band
    for (int u = threadIdx.x; u < B::WM * B::HM; u += kThreads) {
        int ly = ly0 - 1 + u / B::WM, lx = u % B::WM - 1;
        if (a.bc != 0) {
            lx = bc_map(x0 + lx, a.nx, 1) - x0;
            ly = bc_map(y0 + ly, a.ny, 1) - y0;
        }
        const double *C = smc + (ly - (ly0 - 2)) * B::W2 + lx + 2;
        const double *E = sme + (ly - (ly0 - 1)) * B::W1 + lx + 1;
        mu[u] = sint_mu<double, double>(C, B::W2, E, B::FE, np, ph);
    }
    __syncthreads();
    for (int u = threadIdx.x; u < B::BR * T; u += kThreads) {
        const int jb = u / T, i = u % T;
        const int64_t g = (int64_t)(y0 + ly0 + jb) * a.nx + x0 + i;
        const double cc = smc[(jb + 2) * B::W2 + i + 2];
        const double *E = sme + (jb + 1) * B::W1 + i + 1;
        double s2f;
        const double cn = sint_c_new<double, double>(cc, mu + (jb + 1) * B::WM + i + 1, B::WM, E, B::FE, np, ph, s2f);
        store_tier<TIER_FP64>(a, g, cn);
        for (int k = 0; k < np; ++k)
            store_tier<TIER_FP64>(a, (int64_t)(k + 1) * a.n + g, sint_eta_new<double>(E + k * B::FE, B::W1, cn, s2f, ph));
    }
}

// The tiles of one tier (list / count built by the classification).
// Launched programmatically after the previous step's last grid: its CTAs
// wait for that grid, then release the step's half/FP32 launch, which runs
// alongside (FP64 launch first).
template <int T, int TIER, bool REF, bool MU64>
__global__ void __launch_bounds__(kThreads) sint_step_kernel(StepArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    pdl_wait();
    pdl_trigger();
    if ((int)blockIdx.x >= a.count[TIER]) return;
    sint_tile<T, TIER, REF, MU64>(a, smraw, red, ntier, a.list[blockIdx.x]);
}

// The half and FP32 tiles of a step in one launch (one CTA per tile; FP64
// tiles, whose double staging needs more shared memory, are left to the FP64
// launch).  Separate half and FP32 launches would each cover only part of
// the grid and run one after the other.  After the step's FP64 launch it is
// launched to run alongside it (disjoint tiles and output stores; both read
// the previous step's state only); its last CTA waits for the FP64 grid
// before it exits, so this grid completes after both.
template <int T, bool MU64>
__global__ void __launch_bounds__(kThreads) sint_step_lo_kernel(StepArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    const int tile = blockIdx.x;
    const int tier = a.tier_out[tile];
    if (tier == TIER_FP32) sint_tile<T, TIER_FP32, false, MU64>(a, smraw, red, ntier, tile);
    else if (tier == TIER_HALF) sint_tile<T, TIER_HALF, false, MU64>(a, smraw, red, ntier, tile);
    if (blockIdx.x == gridDim.x - 1) pdl_wait();
}

template <int T, int TIER, bool MU64> static size_t sint_smem(int nf)
{
    using CT = typename std::conditional<TIER == TIER_FP64, double, float>::type;
    using MT = typename std::conditional<MU64, double, CT>::type;
    return sizeof(MT) * (T + 2) * (T + 2) + sizeof(CT) * ((size_t)Stage<CT, T, 2>::FIELD
                                                          + (size_t)(nf - 1) * Stage<CT, T, 1>::FIELD);
}

template <int T, int TIER, bool REF, bool MU64>
static cudaError_t sint_launch_t(const StepArgs &a, int grid, cudaStream_t s, bool pdl)
{
    return launch_kernel(sint_step_kernel<T, TIER, REF, MU64>, grid, sint_smem<T, TIER, MU64>(a.nf), s, pdl, a);
}

size_t sint_smem_bytes(int tile, int tier, int nf, bool mu64)
{
    if (tile == 32) {
        if (tier == TIER_FP64) return sint_smem<32, TIER_FP64, true>(nf);
        return mu64 ? sint_smem<32, TIER_FP32, true>(nf) : sint_smem<32, TIER_FP32, false>(nf);
    }
    if (tier == TIER_FP64) return sint_smem<16, TIER_FP64, true>(nf);
    return mu64 ? sint_smem<16, TIER_FP32, true>(nf) : sint_smem<16, TIER_FP32, false>(nf);
}

cudaError_t sint_launch(int tile, int tier, bool ref, bool mu64, const StepArgs &a, int grid, cudaStream_t s,
                        bool pdl)
{
    if (tier == TIER_FP64 && !ref && !a.monitor_now) {  // row bands (the monitor needs whole tiles)
        const int np = a.nf - 1;
        if (tile == 32) return launch_kernel(sint_step_f64_band_kernel<32>, grid * SintBand<32>::NB,
                                             SintBand<32>::smem(np), s, pdl, a);
        return launch_kernel(sint_step_f64_band_kernel<16>, grid * SintBand<16>::NB, SintBand<16>::smem(np), s,
                             pdl, a);
    }
#define AMPS_SINT(TT)                                                                              \
    switch (tier) {                                                                                \
    case TIER_HALF:                                                                                \
        return mu64 ? sint_launch_t<TT, TIER_HALF, false, true>(a, grid, s, pdl)                        \
                    : sint_launch_t<TT, TIER_HALF, false, false>(a, grid, s, pdl);                      \
    case TIER_FP32:                                                                                \
        return mu64 ? sint_launch_t<TT, TIER_FP32, false, true>(a, grid, s, pdl)                        \
                    : sint_launch_t<TT, TIER_FP32, false, false>(a, grid, s, pdl);                      \
    default:                                                                                       \
        return ref ? sint_launch_t<TT, TIER_FP64, true, true>(a, grid, s, pdl)                          \
                   : sint_launch_t<TT, TIER_FP64, false, true>(a, grid, s, pdl);                        \
    }
    if (tile == 32) { AMPS_SINT(32) }
    AMPS_SINT(16)
#undef AMPS_SINT
}

cudaError_t sint_launch_lo(int tile, bool mu64, const StepArgs &a, int grid, cudaStream_t s, bool after64)
{
#define AMPS_SLO(TT, MM) \
    return launch_kernel(sint_step_lo_kernel<TT, MM>, grid, sint_smem<TT, TIER_FP32, MM>(a.nf), s, after64, a)
    if (tile == 32) {
        if (mu64) AMPS_SLO(32, true);
        AMPS_SLO(32, false);
    }
    if (mu64) AMPS_SLO(16, true);
    AMPS_SLO(16, false);
#undef AMPS_SLO
}

cudaError_t sint_prepare_lo(int tile, bool mu64)
{
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (tile == 32)
        return mu64 ? cudaFuncSetAttribute(sint_step_lo_kernel<32, true>, attr, kMaxDynSmem)
                    : cudaFuncSetAttribute(sint_step_lo_kernel<32, false>, attr, kMaxDynSmem);
    return mu64 ? cudaFuncSetAttribute(sint_step_lo_kernel<16, true>, attr, kMaxDynSmem)
                : cudaFuncSetAttribute(sint_step_lo_kernel<16, false>, attr, kMaxDynSmem);
}

cudaError_t sint_prepare(int tile, int tier, bool ref, bool mu64)
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (tier == TIER_FP64 && !ref) {
        const cudaError_t e = tile == 32 ? cudaFuncSetAttribute(sint_step_f64_band_kernel<32>, attr, lim)
                                         : cudaFuncSetAttribute(sint_step_f64_band_kernel<16>, attr, lim);
        if (e != cudaSuccess) return e;
    }
#define AMPS_SP(TT)                                                                                      \
    switch (tier) {                                                                                      \
    case TIER_HALF:                                                                                      \
        return mu64 ? cudaFuncSetAttribute(sint_step_kernel<TT, TIER_HALF, false, true>, attr, lim)      \
                    : cudaFuncSetAttribute(sint_step_kernel<TT, TIER_HALF, false, false>, attr, lim);    \
    case TIER_FP32:                                                                                      \
        return mu64 ? cudaFuncSetAttribute(sint_step_kernel<TT, TIER_FP32, false, true>, attr, lim)      \
                    : cudaFuncSetAttribute(sint_step_kernel<TT, TIER_FP32, false, false>, attr, lim);    \
    default:                                                                                             \
        return ref ? cudaFuncSetAttribute(sint_step_kernel<TT, TIER_FP64, true, true>, attr, lim)        \
                   : cudaFuncSetAttribute(sint_step_kernel<TT, TIER_FP64, false, true>, attr, lim);      \
    }
    if (tile == 32) { AMPS_SP(32) }
    AMPS_SP(16)
#undef AMPS_SP
}

}  // namespace amps
