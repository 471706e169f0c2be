// k_gg_ragged.cu -- the fused grain-growth step for ragged grids (a side that
// is not a multiple of the tile): the same per-tile code (gg_tile.cuh) with
// its partial-edge-tile handling compiled in -- the staged halo's wrapped
// column/row re-read at the owner tiles' tiers, FP64 edge tiles' owner-tier
// loads, cells past the domain kept out of the monitor.  Apart from
// k_graingrowth.cu, so that the whole-tile kernels carry none of it and the
// two compile in parallel.
#include "amps_kernels.h"
#include "gg_tile.cuh"

namespace amps {

template <int T, bool REF>
static cudaError_t launch_mk(const StepArgs &a, int grid, size_t smem, cudaStream_t s, const CUtensorMap &tm)
{
    switch (a.monitor_now ? a.monitor_kind : 0) {
    case 0: return launch_kernel(gg_step_kernel<T, REF, 0, 0, true>, grid, smem, s, true, a, tm);
    case 1: return launch_kernel(gg_step_kernel<T, REF, 1, 0, true>, grid, smem, s, true, a, tm);
    case 2: return launch_kernel(gg_step_kernel<T, REF, 2, 0, true>, grid, smem, s, true, a, tm);
    default: return launch_kernel(gg_step_kernel<T, REF, 3, 0, true>, grid, smem, s, true, a, tm);
    }
}

cudaError_t gg_launch_ragged(int tile, bool ref, const StepArgs &a, int grid, size_t smem, cudaStream_t s,
                             const CUtensorMap &tm)
{
    if (tile == 32) return ref ? launch_mk<32, true>(a, grid, smem, s, tm) : launch_mk<32, false>(a, grid, smem, s, tm);
    return ref ? launch_mk<16, true>(a, grid, smem, s, tm) : launch_mk<16, false>(a, grid, smem, s, tm);
}

template <int T, bool REF>
static cudaError_t prepare_mk()
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 0, 0, true>, attr, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 1, 0, true>, attr, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 2, 0, true>, attr, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 3, 0, true>, attr, lim);
    return e;
}

cudaError_t gg_prepare_ragged(int tile, bool ref)
{
    if (tile == 32) return ref ? prepare_mk<32, true>() : prepare_mk<32, false>();
    return ref ? prepare_mk<16, true>() : prepare_mk<16, false>();
}

}  // namespace amps
