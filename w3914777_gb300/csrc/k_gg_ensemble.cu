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
