// k_kobayashi.cu -- fused Kobayashi anisotropic-dendrite step (phi, T).
//
// The reference splits a step into two kernels and seven full-size
// intermediate arrays (snowflake/function.h:5-35 kernel1_pure writes lap phi,
// lap T, phi_x, phi_y, eps, eps'; :36-60 kernel2_pure reads them at the 4
// neighbours).  Here one CTA per tile stages phi and T with a 2-cell halo,
// computes phi_x, phi_y, eps, eps' on the tile plus a 1-cell ring in shared
// memory (phase A), then the update on the tile (phase B).  Nothing but phi
// and T touches HBM.
#include "../../include/amps.h"
#include "amps_internal.cuh"
#include "amps_kernels.h"
#include <type_traits>

namespace amps {

// Seeded uniform noise in [0, 1) of (step a, cell b): SplitMix64's mixing
// function applied three times, the top 53 bits scaled by 2^-53.
// noise_u01 split at its per-step key: noise_key(seed, a) is the part that
// depends on the step only (computed once per tile), noise_u01_k(key, b)
// the per-cell rest; noise_u01_k(noise_key(seed, a), b) == noise_u01(seed,
// a, b) bit for bit.  Float: the 53-bit integer rounded once to float and
// scaled by 2^-53 (exact), which is (float)noise_u01 -- without three FP64
// operations per cell.
__device__ __forceinline__ uint64_t noise_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t noise_key(uint64_t seed, uint64_t a) { return noise_mix(seed ^ noise_mix(a)); }
template <typename CT> __device__ __forceinline__ CT noise_u01_k(uint64_t key, uint64_t b);
template <> __device__ __forceinline__ double noise_u01_k<double>(uint64_t key, uint64_t b)
{
    return (double)(noise_mix(key + b) >> 11) * 0x1.0p-53;
}
template <> __device__ __forceinline__ float noise_u01_k<float>(uint64_t key, uint64_t b)
{
    return __ull2float_rn(noise_mix(key + b) >> 11) * 0x1.0p-53f;
}
__device__ __forceinline__ double noise_u01(uint64_t seed, uint64_t a, uint64_t b)
{
    return noise_u01_k<double>(noise_key(seed, a), b);
}

// x != 0 for a double parameter, by an integer test of its bits (no FP64 op)
__device__ __forceinline__ bool nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }

template <typename CT> __device__ __forceinline__ CT k_atan2(CT y, CT x) { return atan2(y, x); }
template <typename CT> __device__ __forceinline__ CT k_cos(CT v) { return cos(v); }
template <typename CT> __device__ __forceinline__ CT k_sin(CT v) { return sin(v); }
template <typename CT> __device__ __forceinline__ CT k_atan(CT v) { return atan(v); }

// ---- per-cell arithmetic (non-reference order).  (Splitting tiles into row
// bands around these -- 4x the CTAs -- measured no faster at 512^2, where
// the step is a fixed-latency critical path, and 25-30% slower at 1024^2 and
// 2048^2, where the bands' shared ring rows cost throughput.)

// cos(a*theta) and sin(a*theta) for theta = atan2(y, x) and an even
// integer a, without trigonometric functions: the a-th power of the unit
// vector (x + iy) / |(x, y)| (de Moivre's formula), by repeated squaring.
// (x, y) is first scaled by a power of two (exact) so that x^2 + y^2 can
// neither underflow nor overflow.  A zero gradient stands for theta = 0 --
// for an even a the same cos and sin as atan2's +-0 and +-pi there.
__device__ __forceinline__ void kob_rot(float x, float y, int a, float &ca, float &sa)
{
    float c = 1.f, s = 0.f;
    const float m = fmaxf(fabsf(x), fabsf(y));
    if (m > 0.f) {
        int ex;
        frexpf(m, &ex);
        x = ldexpf(x, -ex);
        y = ldexpf(y, -ex);
        const float ir = rsqrtf(fmaf(x, x, y * y));
        c = x * ir;
        s = y * ir;
    }
    float pr = 1.f, pi = 0.f;  // the product so far
    for (int n = a;;) {
        if (n & 1) {
            const float t = fmaf(pr, c, -pi * s);
            pi = fmaf(pr, s, pi * c);
            pr = t;
        }
        n >>= 1;
        if (!n) break;
        const float t = fmaf(c, c, -s * s);
        s = 2.f * c * s;
        c = t;
    }
    ca = pr;
    sa = pi;
}

// Phase A at one cell (snowflake/function.h:30-34): P at the cell's phi,
// row stride ps.  POLY (float tiles, an even integer anisotropy mode):
// cos and sin of aniso*(theta - theta0) by kob_rot and the angle-difference
// identities, the same quantities without atan2/cos/sin, whose long code
// bounds the instruction fetch of this latency-bound step.
template <typename CT, bool POLY = false>
__device__ __forceinline__ void kob_aniso(const CT *P, int ps, const Phys &ph, CT &phx, CT &phy, CT &e, CT &ed)
{
    const CT pe = P[1], pw = P[-1], pn = P[ps], pso = P[-ps];
    phx = (pe - pw) * kc<CT>(ph, KB_HX);
    phy = (pn - pso) * kc<CT>(ph, KB_HY);
    if constexpr (POLY && std::is_same<CT, float>::value) {
        float ca, sa;
        kob_rot(phx, phy, (int)ph.kf[KB_MODE], ca, sa);
        const float c0 = ph.kf[KB_C0], s0 = ph.kf[KB_S0];
        const float cosv = fmaf(ca, c0, sa * s0), sinv = fmaf(sa, c0, -ca * s0);
        e = kc<CT>(ph, KB_EPSB) * fmaf(kc<CT>(ph, KB_DELTA), cosv, 1.f);
        ed = kc<CT>(ph, KB_ED) * sinv;
    } else {
        const CT arg = kc<CT>(ph, KB_ANISO) * (k_atan2<CT>(phy, phx) - kc<CT>(ph, KB_THETA0));
        e = kc<CT>(ph, KB_EPSB) * fma(kc<CT>(ph, KB_DELTA), k_cos<CT>(arg), CT(1));
        ed = kc<CT>(ph, KB_ED) * k_sin<CT>(arg);
    }
}

// Phase B at one cell (snowflake/function.h:54-59): P, Tm at the cell's phi
// and T (row stride sp); the phase-A arrays at index o, row stride es.  pn
// comes back as the tile's tier stores it (rnd: the storage rounding), and
// the latent heat added to T is kappa times that stored change of phi, so
// that a half tile's T moves with the phi it keeps, as the reference's half2
// update does (snowflake/function.h:512-513 reads the new half phi).
template <typename CT, typename RND>
__device__ __forceinline__ void kob_update(const CT *P, const CT *Tm, int sp, const CT *px, const CT *py,
                                           const CT *ep, const CT *epd, int o, int es, const Phys &ph, uint64_t nkey,
                                           int64_t g, RND rnd, CT &pn, CT &tn)
{
    const CT p0 = P[0], t0 = Tm[0];
    const CT inv = kc<CT>(ph, KB_INV);
    const CT lp = ((P[-1] + P[1]) + (P[-2] + P[2]) + (P[-sp] + P[sp]) + (P[-2 * sp] + P[2 * sp])
                   - CT(8) * p0) * inv;
    const CT lt = ((Tm[-1] + Tm[1]) + (Tm[-2] + Tm[2]) + (Tm[-sp] + Tm[sp]) + (Tm[-2 * sp] + Tm[2 * sp])
                   - CT(8) * t0) * inv;
    const int on = o + es, os = o - es, oe = o + 1, ow = o - 1;
    const CT term1 = (ep[on] * epd[on] * px[on] - ep[os] * epd[os] * px[os]) * kc<CT>(ph, KB_HY);
    const CT term2 = -(ep[oe] * epd[oe] * py[oe] - ep[ow] * epd[ow] * py[ow]) * kc<CT>(ph, KB_HX);
    const CT m = kc<CT>(ph, KB_M) * k_atan<CT>(kc<CT>(ph, KB_GAMA) * (kc<CT>(ph, KB_TEQ) - t0));
    CT drive = p0 - CT(0.5) + m;
    if (nonzero(ph.noise))
        drive += kc<CT>(ph, KB_NOISE) * (noise_u01_k<CT>(nkey, (uint64_t)g) - CT(0.5));
    const CT inner = term1 + term2 + ep[o] * ep[o] * lp + p0 * (CT(1) - p0) * drive;
    pn = rnd(fma(kc<CT>(ph, KB_DTT), inner, p0));
    tn = fma(kc<CT>(ph, KB_KAPPA), pn - p0, fma(kc<CT>(ph, KB_DT), lt, t0));
}

// Threads per Kobayashi tile CTA.  A 512^2 grid is 256 tiles of 32^2, so
// at 256 threads a tile the step ran one partial wave at ~14 warps per SM,
// latency-bound; 512 threads a tile double the warps in flight (two cells a
// thread).  A 16^2 half/FP32 tile keeps one cell a thread (256): 512 would
// leave half of them idle in phase B and fit fewer CTAs on an SM.  A 16^2
// FP64 tile keeps 512, so that its phase A (FP64 atan2/cos/sin on the 18^2
// ring, the tier's critical path) takes one pass.
template <int T, int TIER> constexpr int kob_threads() { return T == 32 || TIER == TIER_FP64 ? 512 : 256; }

// TIER of kob_tile for the half/FP32 launch: half or FP32 at run time, one
// copy of the tile code (with its long inlined atan2/cos/sin/atan chain) for
// both instead of two; the same bits, 1% faster at 512^2.
constexpr int TIER_LO = -1;

// One tile of one step at tier TIER (smraw: the kernel's dynamic shared
// memory, kob_smem<T, TIER> bytes; red / ntier: its static scratch; NT
// threads).  MON = false compiles the monitor out (steps without it), SR =
// false the stochastic rounding of half tiles (runs without AMPS_HALF_SR);
// POLY: float tiles take kob_aniso's trigonometry-free form.
template <int T, int TIER, bool REF, int NT = kob_threads<T, TIER>(), bool MON = true, bool SR = true, bool POLY = false>
__device__ __forceinline__ void kob_tile(const StepArgs &a, unsigned char *smraw, double *red, uint8_t *ntier,
                                         int tile)
{
    using CT = typename std::conditional<TIER == TIER_FP64, double, float>::type;
    constexpr int R = 2;
    using S = Stage<CT, T, R>;
    constexpr int E = T + 2;  // phase-A region side (tile + 1-cell ring)
    CT *sm = reinterpret_cast<CT *>(smraw);
    CT *px = sm + 2 * S::FIELD, *py = px + E * E, *ep = py + E * E, *epd = ep + E * E;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int x0 = tx * T, y0 = ty * T;
    // the tile is stored at half (TIER_LO: read from the classification)
    const bool half = TIER == TIER_HALF || (TIER == TIER_LO && a.tier_out[tile] == TIER_HALF);
    load_neighbour_tiers(a, tx, ty, ntier);
    __syncthreads();
    stage_tile<CT, T, R, false, true, NT>(a, sm, ntier, tx, ty, 0, 2);
    __syncthreads();
    const Phys &ph = a.ph;

    // phase A: snowflake/function.h:30-34 on the tile + ring.  With zero-flux
    // boundaries a ring cell outside the domain takes the intermediates of
    // the cell it mirrors, as an index-mapped read of the full-size arrays does.
    for (int u = threadIdx.x; u < E * E; u += NT) {
        int i = u % E - 1, j = u / E - 1;
        if (a.bc != 0) {
            i = bc_map(x0 + i, a.nx, 1) - x0;
            j = bc_map(y0 + j, a.ny, 1) - y0;
        }
        const int r = j + R, cc = i + S::O;
        const CT pe = S::at(sm, 0, r, cc + 1), pw = S::at(sm, 0, r, cc - 1);
        const CT pn = S::at(sm, 0, r + 1, cc), ps = S::at(sm, 0, r - 1, cc);
        CT phx, phy, e, ed;
        if (REF) {
            phx = __ddiv_rn(__dsub_rn(pe, pw), 2.0 * ph.dx);
            phy = __ddiv_rn(__dsub_rn(pn, ps), 2.0 * ph.dy);
            const double th = atan2((double)phy, (double)phx);
            const double arg = __dmul_rn(ph.aniso, __dsub_rn(th, ph.theta0));
            e = __dmul_rn(ph.epsb, __dadd_rn(1.0, __dmul_rn(ph.delta, cos(arg))));
            ed = __dmul_rn(__dmul_rn(__dmul_rn(-ph.epsb, ph.aniso), ph.delta), sin(arg));
        } else {
            kob_aniso<CT, POLY>(&S::at(sm, 0, r, cc), S::P, ph, phx, phy, e, ed);
        }
        const int o = u;
        px[o] = phx; py[o] = phy; ep[o] = e; epd[o] = ed;
    }
    __syncthreads();

    // phase B: snowflake/function.h:54-59 on the tile
    const int64_t step = *a.step_base + a.step_off;
    const uint64_t nkey = noise_key(ph.seed, (uint64_t)step);  // the noise's per-step part
    double metric = 0.0;
    // half/FP32 tiles fold their float values into a float accumulator (the
    // same metric, without FP64 operations per cell)
    using MA = typename std::conditional<TIER == TIER_FP64, MonAcc, MonAccF>::type;
    MA mon, m2;  // phi's samples, T's (fed by the same pass)
    const bool mon_on = MON && a.monitor_now != 0;
    const bool mon_t = mon_on && (a.mfield < 0 || a.mfield == 1);
    if (mon_on) mon_reset(a, mon);
    if (mon_t) mon_reset(a, m2);
    const int mslot = 0;
    for (int u = threadIdx.x; u < T * T; u += NT) {
        const int i = u % T, j = u / T;
        const int r = j + R, cc = i + S::O;
        const int o = (j + 1) * E + (i + 1);
        const CT p0 = S::at(sm, 0, r, cc), t0 = S::at(sm, 1, r, cc);
        const CT *P = &S::at(sm, 0, r, cc), *Tm = &S::at(sm, 1, r, cc);
        const int64_t g = (int64_t)(y0 + j) * a.nx + x0 + i;
        CT pn, tn;
        if (REF) {
            const double d = ph.dxdy;
            // lap: snowflake/function.h:27-28, each term divided separately, left to right
            double lp = __ddiv_rn(P[-1], d);
            lp = __dadd_rn(lp, __ddiv_rn(P[-2], d));
            lp = __dadd_rn(lp, __ddiv_rn(P[1], d));
            lp = __dadd_rn(lp, __ddiv_rn(P[2], d));
            lp = __dadd_rn(lp, __ddiv_rn(P[-S::P], d));
            lp = __dadd_rn(lp, __ddiv_rn(P[-2 * S::P], d));
            lp = __dadd_rn(lp, __ddiv_rn(P[S::P], d));
            lp = __dadd_rn(lp, __ddiv_rn(P[2 * S::P], d));
            lp = __dsub_rn(lp, __ddiv_rn(__dmul_rn(8.0, p0), d));
            double lt = __ddiv_rn(Tm[-1], d);
            lt = __dadd_rn(lt, __ddiv_rn(Tm[-2], d));
            lt = __dadd_rn(lt, __ddiv_rn(Tm[1], d));
            lt = __dadd_rn(lt, __ddiv_rn(Tm[2], d));
            lt = __dadd_rn(lt, __ddiv_rn(Tm[-S::P], d));
            lt = __dadd_rn(lt, __ddiv_rn(Tm[-2 * S::P], d));
            lt = __dadd_rn(lt, __ddiv_rn(Tm[S::P], d));
            lt = __dadd_rn(lt, __ddiv_rn(Tm[2 * S::P], d));
            lt = __dsub_rn(lt, __ddiv_rn(__dmul_rn(8.0, t0), d));
            const int on = o + E, os = o - E, oe = o + 1, ow = o - 1;
            const double term1 = __ddiv_rn(__dsub_rn(__dmul_rn(__dmul_rn(ep[on], epd[on]), px[on]),
                                                     __dmul_rn(__dmul_rn(ep[os], epd[os]), px[os])), 2.0 * ph.dy);
            const double term2 = -__ddiv_rn(__dsub_rn(__dmul_rn(__dmul_rn(ep[oe], epd[oe]), py[oe]),
                                                      __dmul_rn(__dmul_rn(ep[ow], epd[ow]), py[ow])), 2.0 * ph.dx);
            const double m = __dmul_rn(ph.alpha / ph.pi, atan(__dmul_rn(ph.gama, __dsub_rn(ph.teq, t0))));
            double drive = __dadd_rn(__dsub_rn(p0, 0.5), m);
            if (ph.noise != 0.0)
                drive = __dadd_rn(drive, __dmul_rn(ph.noise, __dsub_rn(noise_u01(ph.seed, (uint64_t)step, (uint64_t)g), 0.5)));
            const double inner = __dadd_rn(__dadd_rn(__dadd_rn(term1, term2), __dmul_rn(__dmul_rn(ep[o], ep[o]), lp)),
                                           __dmul_rn(__dmul_rn(p0, __dsub_rn(1.0, p0)), drive));
            pn = __dadd_rn(p0, __dmul_rn(ph.dt / ph.tau, inner));
            tn = __dadd_rn(__dadd_rn(t0, __dmul_rn(ph.dt, lt)), __dmul_rn(ph.kappa, __dsub_rn(pn, p0)));
        } else {
            // storage rounding: to nearest, or (half tiles, AMPS_HALF_SR) stochastic
            const bool sr = SR && half && a.half_arith == AMPS_HALF_SR;
            auto rnd = [&](CT v) -> CT {
                if (half && sr) return (CT)__half2float(half_sr((float)v, sr_bits(ph.seed, step, g)));
                if (TIER == TIER_LO) return half ? (CT)__half2float(__float2half_rn((float)v)) : v;
                return round_to_tier<TIER == TIER_LO ? TIER_FP32 : TIER>(v);
            };
            kob_update<CT>(P, Tm, S::P, px, py, ep, epd, o, E, ph, nkey, g, rnd, pn, tn);
            if (half && sr)
                tn = (CT)__half2float(half_sr((float)tn, sr_bits(ph.seed, step, (uint64_t)(a.n + g))));
        }
        // pn is stored as it stands (kob_update returns it rounded to storage)
        if constexpr (TIER == TIER_LO) {
            if (half) {
                store_tier<TIER_HALF>(a, g, pn);
                store_tier<TIER_HALF>(a, a.n + g, tn);
            } else {
                store_tier<TIER_FP32>(a, g, pn);
                store_tier<TIER_FP32>(a, a.n + g, tn);
            }
        } else {
            store_tier<TIER>(a, g, pn);
            store_tier<TIER>(a, a.n + g, tn);
        }
        if (mon_on && (a.mfield <= 0))
            mon_add<T>(a, mon, mslot, tile, j, i, g, pn, p0, snap_prefetch<T>(a, mslot, tile, j, i, g));
        if (mon_t) {
            // the second monitored field (T) at its stored value
            CT tv;
            if constexpr (TIER == TIER_LO) tv = half ? (CT)__half2float(__float2half_rn((float)tn)) : tn;
            else tv = round_to_tier<TIER>(tn);
            const int slot = a.mfield < 0 ? 1 : 0;
            mon_add<T>(a, m2, slot, tile, j, i, g, tv, t0, snap_prefetch<T>(a, slot, tile, j, i, g));
        }
    }
    if (mon_on) {
        metric = mon_finish<NT>(a, mon, red, metric);
        if (mon_t) {
            __syncthreads();  // red is reused
            metric = mon_finish<NT>(a, m2, red, metric);
        }
        if (threadIdx.x == 0) a.metric[tile] = metric;
    }
}

// The tiles of one tier (list / count built by the classification).
// Launched programmatically after the previous step's last grid (kob_launch):
// its CTAs wait for that grid to complete, its writes visible, and only then
// release the step's half/FP32 launch, which runs alongside (FP64 launch
// first) -- so no grid of this step reads before the previous one has
// written, and the launch itself overlaps the previous step.
template <int T, int TIER, bool REF, bool POLY>
__global__ void __launch_bounds__(kob_threads<T, TIER>()) kob_step_kernel(StepArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kob_threads<T, TIER>() / 32];
    __shared__ uint8_t ntier[9];
    pdl_wait();
    pdl_trigger();
    if ((int)blockIdx.x >= a.count[TIER]) return;
    kob_tile<T, TIER, REF, kob_threads<T, TIER>(), true, true, POLY>(a, smraw, red, ntier, a.list[blockIdx.x]);
}

// The half and FP32 tiles of a step in one launch (one CTA per tile; FP64
// tiles are left to the FP64 launch).  Per-tier launches would each cover
// only part of the grid -- at 512^2 with 32^2 tiles less than one wave apiece
// -- and run one after the other.  After the step's FP64 launch it is
// launched to run alongside it (disjoint tiles and output stores; both read
// the previous step's state only); its last CTA waits for the FP64 grid
// before it exits, so this grid completes after both.
template <int T, bool MON, bool SR, bool POLY>
__global__ void __launch_bounds__(kob_threads<T, TIER_LO>()) kob_step_lo_kernel(StepArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kob_threads<T, TIER_LO>() / 32];
    __shared__ uint8_t ntier[9];
    const int tile = blockIdx.x;
    const int tier = a.tier_out[tile];
    if (tier != TIER_FP64)
        kob_tile<T, TIER_LO, false, kob_threads<T, TIER_LO>(), MON, SR, POLY>(a, smraw, red, ntier, tile);
    if (blockIdx.x == gridDim.x - 1) pdl_wait();
}

template <int T, int TIER> static size_t kob_smem()
{
    using CT = typename std::conditional<TIER == TIER_FP64, double, float>::type;
    return (2 * (size_t)Stage<CT, T, 2>::FIELD + 4 * (size_t)(T + 2) * (T + 2)) * sizeof(CT);
}

template <int T, int TIER, bool REF, bool POLY>
static cudaError_t kob_launch_t(const StepArgs &a, int grid, cudaStream_t s, bool pdl)
{
    return launch_kernel_nt(kob_step_kernel<T, TIER, REF, POLY>, grid, kob_threads<T, TIER>(), kob_smem<T, TIER>(), s,
                            pdl, a);
}

size_t kob_smem_bytes(int tile, int tier)
{
    if (tile == 32) return tier == TIER_FP64 ? kob_smem<32, TIER_FP64>() : kob_smem<32, TIER_FP32>();
    return tier == TIER_FP64 ? kob_smem<16, TIER_FP64>() : kob_smem<16, TIER_FP32>();
}

// float tiles take the trigonometry-free anisotropy where the mode allows it
static bool kob_poly(const StepArgs &a) { return a.ph.kf[KB_MODE] != 0.f; }

template <int T>
static cudaError_t kob_launch_tt(int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s, bool pdl)
{
    const bool poly = kob_poly(a);
    switch (tier) {
    case TIER_HALF:
        return poly ? kob_launch_t<T, TIER_HALF, false, true>(a, grid, s, pdl)
                    : kob_launch_t<T, TIER_HALF, false, false>(a, grid, s, pdl);
    case TIER_FP32:
        return poly ? kob_launch_t<T, TIER_FP32, false, true>(a, grid, s, pdl)
                    : kob_launch_t<T, TIER_FP32, false, false>(a, grid, s, pdl);
    default:
        return ref ? kob_launch_t<T, TIER_FP64, true, false>(a, grid, s, pdl)
                   : kob_launch_t<T, TIER_FP64, false, false>(a, grid, s, pdl);
    }
}

cudaError_t kob_launch(int tile, int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s, bool pdl)
{
    return tile == 32 ? kob_launch_tt<32>(tier, ref, a, grid, s, pdl) : kob_launch_tt<16>(tier, ref, a, grid, s, pdl);
}

// the monitor steps take the variant with the monitor compiled in, runs
// with stochastic rounding the one with it; the others a kernel without
// that code (the step is instruction-fetch bound)
template <int T, bool POLY>
static cudaError_t kob_launch_lo_p(const StepArgs &a, int grid, cudaStream_t s, bool after64)
{
    const size_t smem = kob_smem<T, TIER_FP32>();
    constexpr int nt = kob_threads<T, TIER_LO>();
    const bool mon = a.monitor_now != 0, sr = a.half_arith == AMPS_HALF_SR;
    if (sr)
        return mon ? launch_kernel_nt(kob_step_lo_kernel<T, true, true, POLY>, grid, nt, smem, s, after64, a)
                   : launch_kernel_nt(kob_step_lo_kernel<T, false, true, POLY>, grid, nt, smem, s, after64, a);
    return mon ? launch_kernel_nt(kob_step_lo_kernel<T, true, false, POLY>, grid, nt, smem, s, after64, a)
               : launch_kernel_nt(kob_step_lo_kernel<T, false, false, POLY>, grid, nt, smem, s, after64, a);
}

cudaError_t kob_launch_lo(int tile, const StepArgs &a, int grid, cudaStream_t s, bool after64)
{
    const bool poly = kob_poly(a);
    if (tile == 32)
        return poly ? kob_launch_lo_p<32, true>(a, grid, s, after64) : kob_launch_lo_p<32, false>(a, grid, s, after64);
    return poly ? kob_launch_lo_p<16, true>(a, grid, s, after64) : kob_launch_lo_p<16, false>(a, grid, s, after64);
}

template <int T, bool POLY> static cudaError_t kob_prepare_lo_p()
{
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(kob_step_lo_kernel<T, true, true, POLY>, attr, kMaxDynSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kob_step_lo_kernel<T, false, true, POLY>, attr, kMaxDynSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kob_step_lo_kernel<T, true, false, POLY>, attr, kMaxDynSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kob_step_lo_kernel<T, false, false, POLY>, attr, kMaxDynSmem);
    return e;
}

template <int T> static cudaError_t kob_prepare_lo_t()
{
    cudaError_t e = kob_prepare_lo_p<T, false>();
    return e == cudaSuccess ? kob_prepare_lo_p<T, true>() : e;
}

cudaError_t kob_prepare_lo(int tile) { return tile == 32 ? kob_prepare_lo_t<32>() : kob_prepare_lo_t<16>(); }

template <int T> static cudaError_t kob_prepare_t(int tier, bool ref)
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e;
    switch (tier) {
    case TIER_HALF:
        e = cudaFuncSetAttribute(kob_step_kernel<T, TIER_HALF, false, false>, attr, lim);
        return e == cudaSuccess ? cudaFuncSetAttribute(kob_step_kernel<T, TIER_HALF, false, true>, attr, lim) : e;
    case TIER_FP32:
        e = cudaFuncSetAttribute(kob_step_kernel<T, TIER_FP32, false, false>, attr, lim);
        return e == cudaSuccess ? cudaFuncSetAttribute(kob_step_kernel<T, TIER_FP32, false, true>, attr, lim) : e;
    default:
        return ref ? cudaFuncSetAttribute(kob_step_kernel<T, TIER_FP64, true, false>, attr, lim)
                   : cudaFuncSetAttribute(kob_step_kernel<T, TIER_FP64, false, false>, attr, lim);
    }
}

cudaError_t kob_prepare(int tile, int tier, bool ref)
{
    return tile == 32 ? kob_prepare_t<32>(tier, ref) : kob_prepare_t<16>(tier, ref);
}

}  // namespace amps
