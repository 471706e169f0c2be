// amps_kernels.h -- host-side launchers of the libamps kernels.
#pragma once
#include "amps_internal.cuh"

namespace amps {

// tm (nullable): tensor map of the step's FP32 input, used when a.tma_stage.
cudaError_t gg_launch(int tile, int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s,
                      const CUtensorMap *tm = nullptr);
// pdl: launched programmatically after the stream's previous grid (the kernel waits for it first)
cudaError_t kob_launch(int tile, int tier, bool ref, const StepArgs &a, int grid, cudaStream_t s, bool pdl = false);
cudaError_t sint_launch(int tile, int tier, bool ref, bool mu64, const StepArgs &a, int grid, cudaStream_t s,
                        bool pdl = false);
size_t gg_smem_bytes(int tile, int tier, int nf);
// Kobayashi / sintering: the half and FP32 tiles of a step in one launch
// (grid = all tiles; FP64 tiles are skipped, left to the FP64 tier launch).
// after64: this step's FP64 launch directly precedes (run alongside it)
cudaError_t kob_launch_lo(int tile, const StepArgs &a, int grid, cudaStream_t s, bool after64);
cudaError_t sint_launch_lo(int tile, bool mu64, const StepArgs &a, int grid, cudaStream_t s, bool after64);
cudaError_t kob_prepare_lo(int tile);
cudaError_t sint_prepare_lo(int tile, bool mu64);
// Raise the dynamic shared-memory limit of the kernel a launch would use
// (must run before any graph capture).
// ragged: a side is not a multiple of the tile (the partial-edge-tile kernels).
cudaError_t gg_prepare(int tile, int tier, bool ref, int half_arith, bool ragged = false);
// The fused step with binary16 arithmetic on half tiles (half_arith 1 or 2;
// k_gg_half.cu), called by gg_launch / gg_prepare.
cudaError_t gg_launch_half(int tile, bool ref, const StepArgs &a, int grid, size_t smem, cudaStream_t s,
                           const CUtensorMap &tm);
cudaError_t gg_prepare_half(int tile, bool ref, int half_arith);
// The fused step for ragged grids (a side not a multiple of the tile: partial
// edge tiles; k_gg_ragged.cu), called by gg_launch / gg_prepare.
cudaError_t gg_launch_ragged(int tile, bool ref, const StepArgs &a, int grid, size_t smem, cudaStream_t s,
                             const CUtensorMap &tm);
cudaError_t gg_prepare_ragged(int tile, bool ref);
cudaError_t kob_prepare(int tile, int tier, bool ref);
cudaError_t sint_prepare(int tile, int tier, bool ref, bool mu64);
// Sintering in the reference's own mixed arithmetic (half_arith = AMPS_HALF_REF):
// mu of every cell at its owner's tier into mu[n], then c' and every eta'.
cudaError_t sint_ref_launch(int tile, const StepArgs &a, double *mu, int grid, cudaStream_t s);
// Multi-step grain-growth kernel (32x32 tiles, the fused step's arithmetic):
// `nsteps` consecutive steps without a tier change or a monitor in one
// launch, a CTA per (step, tile); a0 the arguments of the first (and every
// even) step, a1 of the odd ones; done[ntiles] and *queue zero at launch.
struct FlowArgs {
    int *done;
    int *queue;
    int nsteps;
};
size_t gg_flow_smem_bytes(int nf);
cudaError_t gg_prepare_flow(bool ref);
cudaError_t gg_launch_flow(bool ref, const StepArgs &a0, const StepArgs &a1, const FlowArgs &fl, cudaStream_t s);
// Persistent TMA-pipelined grain-growth step (32x32 tiles, FP32 neighbourhoods by tensor copy).
constexpr int kTmaMaxFields = 16;
size_t gg_tma_smem_bytes(int nf);
cudaError_t gg_prepare_tma(bool ref, int nf, int *blocks_per_sm);
cudaError_t gg_launch_tma(bool ref, const CUtensorMap &tm, const StepArgs &a, int grid, cudaStream_t s);
// Ensemble step: one launch per group of members, one CTA per (member, tile)
// work item; the group's step arguments travel by value in the kernel's
// parameter space (up to kEnsCap members), read through the constant cache.
constexpr int kEnsCap = 40;
struct EnsLaunch {
    int count;               // members in this launch
    int first[kEnsCap + 1];  // first CTA of each member; first[count] = the grid
    StepArgs m[kEnsCap];
};
static_assert(sizeof(EnsLaunch) <= 32764, "kernel parameter space");
size_t gg_ens_smem_bytes(int tile, int max_nf);
// sets the kernels' dynamic shared-memory limit to max_smem
cudaError_t gg_prepare_ens(int tile, bool ref, size_t max_smem);
cudaError_t gg_ens_occupancy(int tile, bool ref, size_t smem, int *blocks_per_sm);
cudaError_t gg_launch_ens(int tile, bool ref, bool monitor, const EnsLaunch &L, size_t smem, cudaStream_t s);
// Split tiles (32^2, the library's order, non-monitor steps): every member of
// L has 2 * kPairFields fields, and each tile runs as a two-CTA cluster of
// kPairFields fields each (grid: two CTAs per work item of L.first).
cudaError_t gg_prepare_ens_pair(size_t smem);
cudaError_t gg_launch_ens_pair(const EnsLaunch &L, size_t smem, cudaStream_t s);
size_t kob_smem_bytes(int tile, int tier);
size_t sint_smem_bytes(int tile, int tier, int nf, bool mu64);

// Geometry + storage view used by the utility kernels.
struct Grid {
    void *store[3];           // one parity, per tier
    const uint8_t *tier;      // tier of every tile
    int nx, ny, ntx, nty, tile, nf;
    int64_t n;                // cells of the domain (nx * ny): the row-major arrays these kernels exchange
    int px;                   // storage row pitch (ntx * tile)
    int64_t fs;               // storage field stride (px * nty * tile)
};

// Row-major [nf][ny][nx] double/float <-> tiered storage (pitch px, field stride fs).
cudaError_t scatter_fields(const Grid &g, const void *src, int src_f32, cudaStream_t s);
cudaError_t gather_fields(const Grid &g, void *dst, int dst_f32, int f0, int nfs, cudaStream_t s);
// Monitor at time 0 (or after a set_field): metric and temporal snapshot from the state.
// diff != 0 (kind 2): metric = max |state - snap| over the samples instead of the range.
cudaError_t monitor_state(const Grid &g, int kind, int samples, int mfield, double *metric, double *snap,
                          int write_snap, int *flags, cudaStream_t s, int diff = 0);
// get_type (snowflake/tools.h:212-230) on the device, three tiers, plus
// ordered per-tier tile lists, stats and the decision log.
struct ClassifyArgs {
    const double *metric;
    uint8_t *tier_prev, *tier_cur;
    int *lists, *counts;
    int ntx, nty;
    double thr_lo, thr_hi;
    int high_tier, use_mid;
    unsigned long long *stats;  // [0..2] tile-steps, [3] evals, [4] promotions, [5] demotions
    uint8_t *log;
    int *log_n;
    int max_log;
    int64_t *step_base;
    int advance;                // steps to add to *step_base (one period, or 0)
    int stat_steps;             // steps the current counts ran for (tile-step stats)
    int *order;                 // optional: launch order of the fused grain-growth step
    int bc;                     // boundary map of the tile neighbourhood (for order)
    // optional tier schedule: the k-th classification takes its tier map from
    // sched[min(k, sched_n - 1)] instead of the metric (*sched_i = k, advanced here)
    const uint8_t *sched;
    int sched_n;
    int *sched_i;
};
cudaError_t classify(const ClassifyArgs &c, cudaStream_t s);
// Ensembles: classify (or do the period bookkeeping of) count members whose
// arguments are the device array cs[count], one launch for all.
cudaError_t classify_batch(const ClassifyArgs *cs, int count, cudaStream_t s);
cudaError_t advance_batch(const ClassifyArgs *cs, int count, cudaStream_t s);
// Rebuild lists/counts from tier_cur without reclassifying (static tier maps).
cudaError_t build_lists(const uint8_t *tier, int ntiles, int *lists, int *counts, cudaStream_t s);
// The reference's temporal snapshot (amps_params.ref_snapshot), after a
// classification: on the 4x4 lattice, tiles now at half keep their previous
// snapshot in the lattice columns of the tile's second half; keep := snap.
cudaError_t snap_ref_fixup(double *snap, double *keep, const uint8_t *tier, int ntiles, int nmon, cudaStream_t s);
// Bookkeeping at the end of a period when no classification runs.
cudaError_t advance_period(int64_t *step_base, int advance, int stat_steps, const int *counts,
                           unsigned long long *stats, cudaStream_t s);
// FP64 reductions over one field (block partials, then one ordered pass).
cudaError_t reduce_field(const Grid &g, int field, int kind, double *partials, double *out, cudaStream_t s);
cudaError_t compare_field(const Grid &g, int field, const double *other, double *partials, double *out2,
                          cudaStream_t s);

// Diagnostics on row-major FP64 fields (k_diag.cu).  acc/box/lab/parent are
// device scratch: acc >= max(3, 2*q*q) counters, box 4 ints, lab and parent
// n ints each; flags bit 2: a union-find walk hit its cap.
cudaError_t diag_interface(const double *f, int nx, int ny, int bc, double level, unsigned long long *acc, int *box,
                           cudaStream_t s);
cudaError_t diag_grains(const double *fields, int e0, int q, int nx, int ny, int bc, double thr, const double *conc,
                        double clevel, int *lab, int *parent, unsigned long long *acc, int *flags, cudaStream_t s);
cudaError_t diag_boundaries(const double *fields, int e0, int q, int nx, int ny, int bc, const double *conc,
                            double clevel, int *lab, unsigned long long *acc, cudaStream_t s);
// out = {max |a-b|, rms, mean |a-b|}; partials: 3*np doubles
cudaError_t diag_compare3(const double *a, const double *b, int64_t n, double *partials, int np, double *out,
                          cudaStream_t s);

}  // namespace amps
