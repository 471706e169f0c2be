// k_gg_half.cu -- the fused grain-growth step whose half tiles compute in
// binary16 (amps_params.half_arith: AMPS_HALF_REF, the reference's
// expression order with every operation rounded; AMPS_HALF_HFMA2, packed
// fused multiply-adds).  The per-tile code is gg_tile.cuh's; this file only
// instantiates and launches it, apart from k_graingrowth.cu so that the two
// compile in parallel.
#include "amps_kernels.h"
#include "gg_tile.cuh"

namespace amps {

template <int T, bool REF, int HA>
static cudaError_t launch_mk(const StepArgs &a, int grid, size_t smem, cudaStream_t s, const CUtensorMap &tm)
{
    switch (a.monitor_now ? a.monitor_kind : 0) {
    case 0: return launch_kernel(gg_step_kernel<T, REF, 0, HA>, grid, smem, s, true, a, tm);
    case 1: return launch_kernel(gg_step_kernel<T, REF, 1, HA>, grid, smem, s, true, a, tm);
    case 2: return launch_kernel(gg_step_kernel<T, REF, 2, HA>, grid, smem, s, true, a, tm);
    default: return launch_kernel(gg_step_kernel<T, REF, 3, HA>, grid, smem, s, true, a, tm);
    }
}

template <int T, int HA>
static cudaError_t launch_ref(bool ref, const StepArgs &a, int grid, size_t smem, cudaStream_t s, const CUtensorMap &tm)
{
    return ref ? launch_mk<T, true, HA>(a, grid, smem, s, tm) : launch_mk<T, false, HA>(a, grid, smem, s, tm);
}

cudaError_t gg_launch_half(int tile, bool ref, const StepArgs &a, int grid, size_t smem, cudaStream_t s,
                           const CUtensorMap &tm)
{
    if (a.half_arith == 1)
        return tile == 32 ? launch_ref<32, 1>(ref, a, grid, smem, s, tm) : launch_ref<16, 1>(ref, a, grid, smem, s, tm);
    if (a.half_arith == 2)
        return tile == 32 ? launch_ref<32, 2>(ref, a, grid, smem, s, tm) : launch_ref<16, 2>(ref, a, grid, smem, s, tm);
    return cudaErrorInvalidValue;
}

template <int T, bool REF, int HA>
static cudaError_t prepare_mk()
{
    const int lim = kMaxDynSmem;
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 0, HA>, attr, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 1, HA>, attr, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 2, HA>, attr, lim);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gg_step_kernel<T, REF, 3, HA>, attr, lim);
    return e;
}

template <int HA>
static cudaError_t prepare_ha(int tile, bool ref)
{
    if (tile == 32) return ref ? prepare_mk<32, true, HA>() : prepare_mk<32, false, HA>();
    return ref ? prepare_mk<16, true, HA>() : prepare_mk<16, false, HA>();
}

cudaError_t gg_prepare_half(int tile, bool ref, int half_arith)
{
    if (half_arith == 1) return prepare_ha<1>(tile, ref);
    if (half_arith == 2) return prepare_ha<2>(tile, ref);
    return cudaErrorInvalidValue;
}

}  // namespace amps
