// k_gg_ensemble.cu -- the ensemble's grain-growth step: many independent runs
// (members of any size, ragged or not, and any field count) advanced by one
// launch per group of members.  A CTA is one (member, tile) work item and
// runs the single-run fused step's per-tile code (gg_tile_step), so every
// member gets exactly its single-run results.  The group's step arguments
// are a by-value kernel parameter: the tile code reads its member's fields
// through the constant cache at a uniform offset, as the single-run kernel
// reads its own, and keeps that kernel's 64 registers (four CTAs an SM).
#include "amps_kernels.h"
#include "gg_tile.cuh"

namespace amps {

template <int T, bool REF, bool MON>
__global__ void __launch_bounds__(kThreads, 4) gg_ens_kernel(const __grid_constant__ EnsLaunch L)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    __shared__ __align__(8) uint64_t bar;
    // 128-byte aligned staging (gg_smem_bytes adds the slack), as tensor copies need
    float *sm = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smraw) + 127) & ~uintptr_t(127));
    // this CTA's member: the last whose first work item is at or before it
    const int b = (int)blockIdx.x;
    int lo = 0, hi = L.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const StepArgs &a = L.m[lo];
    gg_tile_step<T, REF, MON ? -1 : 0, 0, true, true>(a, sm, ntier, red, b - L.first[lo], a.tmap, &bar);
}

// ---- split tiles ---------------------------------------------------------------
// The two CTAs of a cluster advance one 32x32 tile of a member with
// 2 * kPairFields fields, kPairFields each (cluster rank r: fields
// [r * kPairFields, (r + 1) * kPairFields)).  The staging is half the whole
// tile's, so twice the CTAs share an SM (four, as for eight fields).  Each
// CTA forms the sum of squares over every field itself, in field order, from
// both stagings -- its own, and its peer's through distributed shared
// memory -- so every cell gets the whole-tile kernel's value to the bit.
// Non-monitor steps only (the monitor steps run whole tiles).
//
// Barriers: the two CTAs read the same tier, so both take the FP64 path
// (which uses no cluster barrier) or both take the staged path, where every
// thread of both CTAs runs both cluster barrier phases; a staging copy that
// gave up still passes them and skips the compute.
template <bool REF>
__device__ __forceinline__ void gg_tile_pair(const StepArgs &a, float *sm, uint8_t *ntier, double *red, int tile,
                                             uint32_t rank, uint64_t *bar)
{
    constexpr int T = 32, PH = kPairFields;
    using S = Stage<float, T, 1>;
    const int f0 = (int)rank * PH;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    load_neighbour_tiers(a, tx, ty, ntier);
    const bool spec = a.in[TIER_FP32] != nullptr;
    const CUtensorMap *tm = a.tmap8;
    const bool bulk = spec && tm != nullptr && tx >= 1 && ty >= 1 && tx <= a.ntx - 2 && ty <= a.nty - 2;
    if (bulk) {
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
            mbar_arrive_expect_tx(bar, (uint32_t)(S::FIELD * PH * sizeof(float)));
            tma_load_3d(sm, tm, tx * T - S::O, ty * T - 1, f0, bar);
        }
    } else if (spec) {
        stage_tile_async32<T, 1, false>(a, sm, tx, ty, PH, f0);
    }
    // the copies have landed (false: a bounded wait on the tensor copy gave
    // up -- flagged; thread 0 waits once more for it)
    auto spec_done = [&]() -> bool {
        if (!bulk) {
            cp_async_wait_all();
            return true;
        }
        const bool got = mbar_wait_bounded(bar, 0);
        if (__syncthreads_or(!got)) {
            if (threadIdx.x == 0) {
                atomicOr(a.flags, 2);
                if (!got) mbar_wait_bounded(bar, 0);
            }
            return false;
        }
        return true;
    };
    const int tier = a.tier_out[tile];
    __syncthreads();
    if (tier == TIER_FP64) {
        if (gg_partial_tile(a, T, tx, ty)) gg_tile_fp64_partial<T, REF, PH>(a, ntier, tile, tx, ty, red, f0);
        else gg_tile_fp64<T, REF, false, PH>(a, ntier, tile, tx, ty, red, f0);
        if (spec) spec_done();
        return;
    }
    const bool all32 = all_fp32(ntier);
    bool ok = true;
    if (spec) {
        ok = spec_done();
        if (ok && !all32) stage_tile<float, T, 1, true, true>(a, sm, ntier, tx, ty, f0, PH);
    } else if (all32) {
        stage_tile_async32<T, 1>(a, sm, tx, ty, PH, f0);
    } else {
        stage_tile<float, T, 1, false, true>(a, sm, ntier, tx, ty, f0, PH);
    }
    __syncthreads();
    if (ok && gg_partial_tile(a, T, tx, ty)) {  // a ragged grid's edge tile: its wrapped halo
        patch_ragged<float, T>(a, sm, tx, ty, f0, PH);
        __syncthreads();
    }
    cluster_arrive();  // both stagings complete, visible to the peer
    cluster_wait();
    float *ss = sm + PH * S::FIELD;  // gg_smem_bytes(32, -1, PH) reserves it
    {
        constexpr int GPR = 8;
        const int row = threadIdx.x / GPR, c = (threadIdx.x % GPR) * 4;
        const float *own = &S::at(sm, 0, row + 1, S::O + c);
        const uint32_t peer = cluster_map(own, rank ^ 1u);
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        auto add = [&](const float4 q) {
            acc.x = fmaf(q.x, q.x, acc.x);
            acc.y = fmaf(q.y, q.y, acc.y);
            acc.z = fmaf(q.z, q.z, acc.z);
            acc.w = fmaf(q.w, q.w, acc.w);
        };
        // fields 0 .. 2*PH-1 in order: rank 0's staging holds the first half
        if (rank == 0) {
#pragma unroll
            for (int f = 0; f < PH; ++f) add(*reinterpret_cast<const float4 *>(own + f * S::FIELD));
#pragma unroll
            for (int f = 0; f < PH; ++f) add(ld_cluster_f4(peer + (uint32_t)(f * S::FIELD * sizeof(float))));
        } else {
#pragma unroll
            for (int f = 0; f < PH; ++f) add(ld_cluster_f4(peer + (uint32_t)(f * S::FIELD * sizeof(float))));
#pragma unroll
            for (int f = 0; f < PH; ++f) add(*reinterpret_cast<const float4 *>(own + f * S::FIELD));
        }
        *reinterpret_cast<float4 *>(ss + row * T + c) = acc;
    }
    cluster_arrive();  // done reading the peer's staging
    __syncthreads();
    if (ok) {
        if (tier == TIER_FP32) gg_tile_lo_rows<TIER_FP32, 8, 0, PH>(a, sm, ss, tile, tx, ty, red, f0);
        else gg_tile_lo_rows<TIER_HALF, 8, 0, PH>(a, sm, ss, tile, tx, ty, red, f0);
    }
    cluster_wait();  // the peer is done reading this staging before the CTA exits
}

template <bool REF>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 4)
    gg_ens_pair_kernel(const __grid_constant__ EnsLaunch L)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ double red[kThreads / 32];
    __shared__ uint8_t ntier[9];
    __shared__ __align__(8) uint64_t bar;
    float *sm = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smraw) + 127) & ~uintptr_t(127));
    uint32_t rank;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    // this cluster's work item, and its member as in gg_ens_kernel
    const int b = (int)(blockIdx.x >> 1);
    int lo = 0, hi = L.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    gg_tile_pair<REF>(L.m[lo], sm, ntier, red, b - L.first[lo], rank, &bar);
}

cudaError_t gg_prepare_ens_pair(size_t smem)
{
    return cudaFuncSetAttribute(gg_ens_pair_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t gg_launch_ens_pair(const EnsLaunch &L, size_t smem, cudaStream_t s)
{
    const unsigned grid = 2u * (unsigned)L.first[L.count];
    if (grid == 0) return cudaSuccess;
    gg_ens_pair_kernel<false><<<grid, kThreads, smem, s>>>(L);
    return cudaGetLastError();
}

// staging for a group's member with the most fields
size_t gg_ens_smem_bytes(int tile, int max_nf) { return gg_smem_bytes(tile, -1, max_nf); }

#define AMPS_GGE_DISPATCH(MACRO) \
    do {                         \
        if (tile == 32) {        \
            if (ref) MACRO(32, true);  \
            else MACRO(32, false);     \
        } else {                 \
            if (ref) MACRO(16, true);  \
            else MACRO(16, false);     \
        }                        \
    } while (0)

cudaError_t gg_prepare_ens(int tile, bool ref, size_t max_smem)
{
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaSuccess;
#define AMPS_GGE(TT, RR)                                                                            \
    do {                                                                                            \
        e = cudaFuncSetAttribute(gg_ens_kernel<TT, RR, false>, attr, (int)max_smem);                \
        if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_ens_kernel<TT, RR, true>, attr, (int)max_smem); \
    } while (0)
    AMPS_GGE_DISPATCH(AMPS_GGE);
#undef AMPS_GGE
    return e;
}

cudaError_t gg_ens_occupancy(int tile, bool ref, size_t smem, int *blocks_per_sm)
{
    cudaError_t e = cudaSuccess;
#define AMPS_GGO(TT, RR) \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gg_ens_kernel<TT, RR, false>, kThreads, smem)
    AMPS_GGE_DISPATCH(AMPS_GGO);
#undef AMPS_GGO
    return e;
}

cudaError_t gg_launch_ens(int tile, bool ref, bool monitor, const EnsLaunch &L, size_t smem, cudaStream_t s)
{
    const unsigned grid = (unsigned)L.first[L.count];
    if (grid == 0) return cudaSuccess;
#define AMPS_GGL(TT, RR)                                                          \
    do {                                                                          \
        if (monitor) gg_ens_kernel<TT, RR, true><<<grid, kThreads, smem, s>>>(L); \
        else gg_ens_kernel<TT, RR, false><<<grid, kThreads, smem, s>>>(L);        \
    } while (0)
    AMPS_GGE_DISPATCH(AMPS_GGL);
#undef AMPS_GGL
    return cudaGetLastError();
}

#undef AMPS_GGE_DISPATCH

}  // namespace amps
