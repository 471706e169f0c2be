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
#include "amps_kernels.h"
#include "gg_tile.cuh"

#include <string.h>

namespace amps {

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
    if (gg_partial_tile(a, T, tx, ty)) {  // a ragged grid's edge tile: its wrapped halo
        patch_ragged<double, T>(a, sm, tx, ty);
        __syncthreads();
    }
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
    const int64_t gbase = (int64_t)(ty * T + r0) * a.px + tx * T + col;
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
            ((double *)a.out[TIER_FP64])[(int64_t)f * a.n + gbase + (int64_t)j * a.px] = out;
        }
    }
}

// ---- multi-step kernel ---------------------------------------------------------
// The interior steps of a period (no tier change, no monitor) in one launch.
// Every step launch of the fused kernel pays a start-up and a drain: its
// first wave of CTAs all stage at once and its last CTAs finish alone, about
// 2.4 us of a 13.8 us all-FP32 1024^2 Q=8 step (608 tiles take 9.0 us, 1216
// take 15.6 us).  Here one grid holds a CTA for every (step, tile) item; a
// CTA takes the next item in step-major, slow-first order from a counter
// (not its block index), and an item of step s starts as soon as the 3x3
// tiles of its neighbourhood have finished step s-1 -- the only data it
// reads, and the only readers of the buffer it overwrites -- so the next
// step's tiles run while the last ones of this step still compute.
//
// Progress needs no co-residency: a CTA claims an item only once it runs,
// so every earlier item belongs to a CTA that runs or has finished, and an
// item waits only on earlier ones (the dynamic-index rule of single-pass
// scans).  Each wait is bounded: past ~1 s it sets the device error flag
// (bit 1), which every other wait sees and gives up on, and the CTAs return.
// Visibility: the producing CTA's threads finish their stores, a CTA
// barrier, then one thread's device-scope release store of the tile's
// counter; each of the consumer's nine polling threads sees its counter and
// issues a device-scope acquire fence, and a CTA barrier precedes every
// thread's loads.
// Loads of step data avoid the read-only path (NC = false), which is not
// kept coherent with writes made during the launch.

// Threads 0..8, one tile each of the 3x3 neighbourhood of `tile` (after the
// boundary map): wait until it has completed `need` steps, then an acquire
// fence; false if the wait gave up or another did.  The nine waits run side
// by side (one L2 round trip when they are already met).
__device__ bool flow_wait(const StepArgs &a, const int *done, int tile, int need)
{
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    int x = tx + (int)threadIdx.x % 3 - 1, y = ty + (int)threadIdx.x / 3 - 1;
    if (a.bc == 0) {
        x = x < 0 ? a.ntx - 1 : (x >= a.ntx ? 0 : x);
        y = y < 0 ? a.nty - 1 : (y >= a.nty ? 0 : y);
    } else {
        x = x < 0 ? 0 : (x >= a.ntx ? a.ntx - 1 : x);
        y = y < 0 ? 0 : (y >= a.nty ? a.nty - 1 : y);
    }
    volatile const int *vd = done + y * a.ntx + x;
    volatile const int *vflag = a.flags;
    for (int it = 0; *vd < need; ++it) {
        if ((*vflag & 2) || it >= (1 << 24)) {
            atomicOr(a.flags, 2);
            return false;
        }
        if (it > 32) __nanosleep(64);
    }
    // acquire: the counter seen above, then the CTA barrier, order every
    // thread's loads after the producer's stores
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    return true;
}

// One CTA per (step, tile) item; a0: the arguments of even steps (counted
// from the launch's first), a1: of odd ones.
template <bool REF>
__global__ void __launch_bounds__(kThreads, 4) gg_flow_kernel(StepArgs a0, StepArgs a1, FlowArgs fl)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    __shared__ int item_s;
    float *sm = reinterpret_cast<float *>(smraw);
    const int ntiles = a0.ntx * a0.nty;
    if (threadIdx.x == 0) item_s = atomicAdd(fl.queue, 1);
    __syncthreads();
    const int item = item_s, step = item / ntiles;
    const int tile = a0.order ? a0.order[item % ntiles] : item % ntiles;
    if (step > 0) {
        const bool ok = threadIdx.x >= 9 || flow_wait(a0, fl.done, tile, step);
        if (!__syncthreads_and(ok)) return;
    }
    if (step & 1) gg_tile_step<32, REF, 0, 0, false>(a1, sm, ntier, red, tile);
    else gg_tile_step<32, REF, 0, 0, false>(a0, sm, ntier, red, tile);
    __syncthreads();
    if (threadIdx.x == 0) {
        // release: the CTA's stores (ordered before by the barrier), then the counter
        asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(fl.done + tile), "r"(step + 1) : "memory");
    }
}

size_t gg_flow_smem_bytes(int nf) { return gg_smem_bytes(32, -1, nf); }

cudaError_t gg_prepare_flow(bool ref)
{
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    return ref ? cudaFuncSetAttribute(gg_flow_kernel<true>, attr, kMaxDynSmem)
               : cudaFuncSetAttribute(gg_flow_kernel<false>, attr, kMaxDynSmem);
}

cudaError_t gg_launch_flow(bool ref, const StepArgs &a0, const StepArgs &a1, const FlowArgs &fl, cudaStream_t s)
{
    const int grid = fl.nsteps * a0.ntx * a0.nty;
    const size_t smem = gg_flow_smem_bytes(a0.nf);
    if (ref) gg_flow_kernel<true><<<grid, kThreads, smem, s>>>(a0, a1, fl);
    else gg_flow_kernel<false><<<grid, kThreads, smem, s>>>(a0, a1, fl);
    return cudaGetLastError();
}

// tier: TIER_FP64 selects the all-FP64 staged kernel; anything else the fused one.
size_t gg_smem_bytes(int tile, int tier, int nf)
{
    if (tier == TIER_FP64)
        return (size_t)nf * (tile == 32 ? Stage<double, 32, 1>::FIELD : Stage<double, 16, 1>::FIELD) * sizeof(double);
    // 32^2: + the sum-of-squares tile of gg_tile_lo_rows; + 128 bytes to align
    // the staging for tensor copies (gg_step_kernel)
    if (tile == 32) return ((size_t)nf * Stage<float, 32, 1>::FIELD + 32 * 32) * sizeof(float) + 128;
    return (size_t)nf * Stage<float, 16, 1>::FIELD * sizeof(float) + 128;
}

template <typename K>
static cudaError_t launch_pdl(K kernel, int grid, size_t smem, cudaStream_t s, const StepArgs &a, const CUtensorMap &tm)
{
    return launch_kernel(kernel, grid, smem, s, true, a, tm);
}

cudaError_t gg_launch(int tile, int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s, const CUtensorMap *tmp)
{
    CUtensorMap none;
    memset(&none, 0, sizeof none);
    const CUtensorMap &tm = tmp ? *tmp : none;
    const size_t smem = gg_smem_bytes(tile, tier, a.nf);
#define AMPS_GGL(K, TT)                                                         \
    do {                                                                        \
        if (ref) K<TT, true><<<grid, kThreads, smem, s>>>(a);                   \
        else K<TT, false><<<grid, kThreads, smem, s>>>(a);                      \
    } while (0)
#define AMPS_GGK(TT, MK)                                                                              \
    do {                                                                                              \
        if (ref) return launch_pdl(gg_step_kernel<TT, true, MK>, grid, smem, s, a, tm);               \
        return launch_pdl(gg_step_kernel<TT, false, MK>, grid, smem, s, a, tm);                       \
    } while (0)
#define AMPS_GGM(TT)                                                                                  \
    do {                                                                                              \
        switch (a.monitor_now ? a.monitor_kind : 0) {                                                 \
        case 0: AMPS_GGK(TT, 0);                                                                      \
        case 1: AMPS_GGK(TT, 1);                                                                      \
        case 2: AMPS_GGK(TT, 2);                                                                      \
        default: AMPS_GGK(TT, 3);                                                                     \
        }                                                                                             \
    } while (0)
    if (tier == TIER_FP64) {
        if (tile == 32) AMPS_GGL(gg_step_f64_kernel, 32);
        else AMPS_GGL(gg_step_f64_kernel, 16);
    } else if (a.nx % tile || a.ny % tile) {
        return gg_launch_ragged(tile, ref, a, grid, smem, s, tm);  // partial edge tiles (k_gg_ragged.cu)
    } else if (a.half_arith != 0) {
        return gg_launch_half(tile, ref, a, grid, smem, s, tm);  // binary16 half tiles (k_gg_half.cu)
    } else {
        if (tile == 32) AMPS_GGM(32);
        else AMPS_GGM(16);
    }
#undef AMPS_GGL
#undef AMPS_GGM
#undef AMPS_GGK
    return cudaGetLastError();
}

cudaError_t gg_prepare(int tile, int tier, bool ref, int half_arith, bool ragged)
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (tier == TIER_FP64) {
        if (tile == 32) return ref ? cudaFuncSetAttribute(gg_step_f64_kernel<32, true>, attr, lim)
                                   : cudaFuncSetAttribute(gg_step_f64_kernel<32, false>, attr, lim);
        return ref ? cudaFuncSetAttribute(gg_step_f64_kernel<16, true>, attr, lim)
                   : cudaFuncSetAttribute(gg_step_f64_kernel<16, false>, attr, lim);
    }
    if (half_arith != 0) return gg_prepare_half(tile, ref, half_arith);
    if (ragged) return gg_prepare_ragged(tile, ref);
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

}  // namespace amps
