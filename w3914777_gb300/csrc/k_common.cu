// k_common.cu -- utility kernels of libamps: tiered state <-> row-major
// arrays, the monitor on a resting state, tile classification with ordered
// per-tier work lists, and deterministic FP64 reductions.
#include "../../include/amps.h"
#include "amps_kernels.h"

namespace amps {

// ---------------------------------------------------------------- state ----
__device__ __forceinline__ int tier_of(const Grid &g, int x, int y)
{
    return g.tier[(y / g.tile) * g.ntx + x / g.tile];
}

// storage index of domain cell (x, y) of field f
__device__ __forceinline__ int64_t store_index(const Grid &g, int f, int x, int y)
{
    return (int64_t)f * g.fs + (int64_t)y * g.px + x;
}

__global__ void scatter_kernel(Grid g, const void *src, int src_f32)
{
    const int64_t total = (int64_t)g.nf * g.n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = k % g.n;
        const int x = (int)(c % g.nx), y = (int)(c / g.nx);
        const double v = src_f32 ? (double)((const float *)src)[k] : ((const double *)src)[k];
        const int t = tier_of(g, x, y);
        const int64_t q = store_index(g, (int)(k / g.n), x, y);
        if (t == TIER_FP64) ((double *)g.store[2])[q] = v;
        else if (t == TIER_FP32) ((float *)g.store[1])[q] = (float)v;
        else ((__half *)g.store[0])[q] = __float2half_rn((float)v);
    }
}

// c: index of the cell in the row-major domain array
__device__ __forceinline__ double read_cell(const Grid &g, int f, int64_t c)
{
    const int x = (int)(c % g.nx), y = (int)(c / g.nx);
    const int t = tier_of(g, x, y);
    const int64_t k = store_index(g, f, x, y);
    if (t == TIER_FP64) return ((const double *)g.store[2])[k];
    if (t == TIER_FP32) return (double)((const float *)g.store[1])[k];
    return (double)__half2float(((const __half *)g.store[0])[k]);
}

__global__ void gather_kernel(Grid g, void *dst, int dst_f32, int f0, int nfs)
{
    const int64_t total = (int64_t)nfs * g.n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const double v = read_cell(g, f0 + (int)(k / g.n), k % g.n);
        if (dst_f32) ((float *)dst)[k] = (float)v;
        else ((double *)dst)[k] = v;
    }
}

static int grid_for(int64_t total)
{
    int64_t b = (total + 255) / 256;
    return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

cudaError_t scatter_fields(const Grid &g, const void *src, int src_f32, cudaStream_t s)
{
    scatter_kernel<<<grid_for((int64_t)g.nf * g.n), 256, 0, s>>>(g, src, src_f32);
    return cudaGetLastError();
}

cudaError_t gather_fields(const Grid &g, void *dst, int dst_f32, int f0, int nfs, cudaStream_t s)
{
    gather_kernel<<<grid_for((int64_t)nfs * g.n), 256, 0, s>>>(g, dst, dst_f32, f0, nfs);
    return cudaGetLastError();
}

// ------------------------------------------------------ resting monitor ----
// One CTA per tile: the spatial metric of the current state, and/or the
// temporal snapshot (same lattice and slots as the fused epilogues).
// diff: the temporal metric against snap (max |state - snap|, the fused
// temporal monitor's reduction) in place of the range.
__global__ void monitor_state_kernel(Grid g, int kind, int samples, int mfield, double *metric, double *snap,
                                     int write_snap, int *flags, int diff)
{
    __shared__ double red[8];
    const int tile = blockIdx.x;
    const int T = g.tile;
    const int tx = tile % g.ntx, ty = tile / g.ntx;
    double result = 0.0;
    for (int f = 0; f < g.nf; ++f) {
        if (mfield >= 0 && f != mfield) continue;
        const int slot = mfield < 0 ? f : 0;
        double mn = samples ? INFINITY : 1.0, mx = samples && !diff ? -INFINITY : 0.0;
        int bad = 0;
        for (int u = threadIdx.x; u < T * T; u += blockDim.x) {
            const int i = u % T, j = u / T;
            // a ragged grid's edge tile: only its cells inside the domain
            if (tx * T + i >= g.nx || ty * T + j >= g.ny) continue;
            const int64_t c = (int64_t)(ty * T + j) * g.nx + tx * T + i;
            const int64_t sc = (int64_t)(ty * T + j) * g.px + tx * T + i;  // snapshot slot: storage layout
            const double v = read_cell(g, f, c);
            if (!(v == v) || isinf(v)) bad = 1;
            int si = 0;
            if (!samples) {
                int ir = -1, ic = -1;
                for (int k = 0; k < 4; ++k) {
                    const int p = kind == 1 ? (k * (T - 1) * 2 + 3) / 6 : T / 8 + k * (T / 4);
                    if (j == p) ir = k;
                    if (i == p) ic = k;
                }
                si = (ir < 0 || ic < 0) ? -1 : ir * 4 + ic;
            }
            if (si < 0) continue;
            if (diff) {
                const double r = samples ? snap[(int64_t)slot * g.fs + sc]
                                         : snap[((int64_t)slot * g.ntx * g.nty + tile) * 16 + si];
                mx = fmax(mx, fabs(r - v));
                continue;
            }
            mn = fmin(mn, v);
            mx = fmax(mx, v);
            if (write_snap) {
                if (samples) snap[(int64_t)slot * g.fs + sc] = v;
                else snap[((int64_t)slot * g.ntx * g.nty + tile) * 16 + si] = v;
            }
        }
        const double bmx = block_max(mx, red);
        const double bmn = block_min(mn, red);
        result = fmax(result, diff ? bmx : bmx - bmn);
        if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flags, 1);
    }
    if (threadIdx.x == 0 && metric) metric[tile] = result;
}

cudaError_t monitor_state(const Grid &g, int kind, int samples, int mfield, double *metric, double *snap,
                          int write_snap, int *flags, cudaStream_t s, int diff)
{
    monitor_state_kernel<<<g.ntx * g.nty, kThreads, 0, s>>>(g, kind, samples, mfield, metric, snap, write_snap,
                                                          flags, diff);
    return cudaGetLastError();
}

// ------------------------------------------------------------ classify ----
// Inclusive scan of 64-bit packed counters over a 1024-thread block.
__device__ __forceinline__ unsigned long long block_scan(unsigned long long v, unsigned long long *ws)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) ws[w] = v;
    __syncthreads();
    if (w == 0) {
        unsigned long long t = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += u;
        }
        ws[lane] = t;
    }
    __syncthreads();
    const unsigned long long r = v + (w > 0 ? ws[w - 1] : 0ull);
    __syncthreads();
    return r;
}

// Inclusive scan of two 64-bit packed counters at once (the barriers of one
// scan); *ta, *tb: the block's totals.
__device__ __forceinline__ void block_scan2(unsigned long long &a, unsigned long long &b, unsigned long long *ws,
                                            unsigned long long *ta, unsigned long long *tb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long ua = __shfl_up_sync(0xffffffffu, a, o);
        const unsigned long long ub = __shfl_up_sync(0xffffffffu, b, o);
        if (lane >= o) {
            a += ua;
            b += ub;
        }
    }
    if (lane == 31) {
        ws[w] = a;
        ws[32 + w] = b;
    }
    __syncthreads();
    if (w == 0) {
        unsigned long long sa = lane < nw ? ws[lane] : 0ull, sb = lane < nw ? ws[32 + lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long ua = __shfl_up_sync(0xffffffffu, sa, o);
            const unsigned long long ub = __shfl_up_sync(0xffffffffu, sb, o);
            if (lane >= o) {
                sa += ua;
                sb += ub;
            }
        }
        ws[lane] = sa;
        ws[32 + lane] = sb;
    }
    __syncthreads();
    if (w > 0) {
        a += ws[w - 1];
        b += ws[32 + w - 1];
    }
    *ta = ws[nw - 1];
    *tb = ws[32 + nw - 1];
    __syncthreads();
}

// Ordered compaction of the tiles of each tier (tier maps are small: one
// 1024-thread CTA loops over them).
__device__ void lists_from_tiers(const uint8_t *tier, int ntiles, int *lists, int *counts, unsigned long long *ws)
{
    __shared__ unsigned long long base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int t0 = 0; t0 < ntiles; t0 += blockDim.x) {
        const int t = t0 + threadIdx.x;
        const int k = t < ntiles ? tier[t] : -1;
        const unsigned long long mine = k >= 0 ? (1ull << (21 * k)) : 0ull;
        const unsigned long long inc = block_scan(mine, ws);
        const unsigned long long b = base;
        if (k >= 0) {
            const unsigned long long excl = b + inc - mine;
            const int rank = (int)((excl >> (21 * k)) & AMPS_MAX_TILES);
            lists[k * ntiles + rank] = t;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) base = b + inc;
        __syncthreads();
    }
    if (threadIdx.x < 3) counts[threadIdx.x] = (int)((base >> (21 * threadIdx.x)) & AMPS_MAX_TILES);
}

// Launch order of the fused grain-growth step: first the tiles that take
// its slow paths -- FP64 or half tiles, and FP32 tiles with a neighbour
// (after the boundary map) at another tier, which stage their neighbourhood
// with conversions -- then the all-FP32 neighbourhoods, each group in tile
// order.  Slow tiles then run in the first wave, where their extra time is
// absorbed, instead of straggling at the end of the step.  Scheduling only:
// every tile is computed by exactly one CTA either way.
__device__ void order_slow_first(const ClassifyArgs &c, const uint8_t *tier, unsigned long long *ws)
{
    __shared__ unsigned long long base;
    __shared__ int nslow;
    const int ntiles = c.ntx * c.nty;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();  // also: this block's tier_cur writes are visible to it
    for (int pass = 0; pass < 2; ++pass) {
        for (int t0 = 0; t0 < ntiles; t0 += blockDim.x) {
            const int t = t0 + threadIdx.x;
            bool slow = false;
            if (t < ntiles) {
                const int x = t % c.ntx, y = t / c.ntx;
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        int yy = y + dy, xx = x + dx;
                        if (c.bc == 0) {
                            yy = yy < 0 ? yy + c.nty : (yy >= c.nty ? yy - c.nty : yy);
                            xx = xx < 0 ? xx + c.ntx : (xx >= c.ntx ? xx - c.ntx : xx);
                        } else {
                            yy = yy < 0 ? 0 : (yy >= c.nty ? c.nty - 1 : yy);
                            xx = xx < 0 ? 0 : (xx >= c.ntx ? c.ntx - 1 : xx);
                        }
                        slow |= tier[yy * c.ntx + xx] != TIER_FP32;
                    }
            }
            // pass 0 places the slow tiles, pass 1 (after nslow of them) the others
            const bool mine = t < ntiles && slow == (pass == 0);
            const unsigned long long inc = block_scan((unsigned long long)mine, ws);
            const unsigned long long b = base;
            if (mine) c.order[(pass ? nslow : 0) + (int)(b + inc - 1)] = t;
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) base = b + inc;
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (pass == 0) nslow = (int)base;
            base = 0;
        }
        __syncthreads();
    }
}

// lists_from_tiers and order_slow_first in one pass, for maps of at most one
// tile per thread: one scan of two packed counters -- the tier ranks, and
// the slow (low 32 bits) / all-FP32 (high 32 bits) ranks of the launch
// order.  Same lists, counts and order as the two routines.
__device__ void lists_and_order(const ClassifyArgs &c, const uint8_t *tier, unsigned long long *ws)
{
    const int ntiles = c.ntx * c.nty;
    const int t = threadIdx.x;
    int k = -1;
    bool slow = false;
    if (t < ntiles) {
        k = tier[t];
        const int x = t % c.ntx, y = t / c.ntx;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int yy = y + dy, xx = x + dx;
                if (c.bc == 0) {
                    yy = yy < 0 ? yy + c.nty : (yy >= c.nty ? yy - c.nty : yy);
                    xx = xx < 0 ? xx + c.ntx : (xx >= c.ntx ? xx - c.ntx : xx);
                } else {
                    yy = yy < 0 ? 0 : (yy >= c.nty ? c.nty - 1 : yy);
                    xx = xx < 0 ? 0 : (xx >= c.ntx ? c.ntx - 1 : xx);
                }
                slow |= tier[yy * c.ntx + xx] != TIER_FP32;
            }
    }
    const unsigned long long ma = k >= 0 ? (1ull << (21 * k)) : 0ull;
    const unsigned long long mb = k >= 0 ? (slow ? 1ull : (1ull << 32)) : 0ull;
    unsigned long long a = ma, b = mb, ta, tb;
    block_scan2(a, b, ws, &ta, &tb);
    if (k >= 0) {
        const unsigned long long ea = a - ma, eb = b - mb;
        c.lists[k * ntiles + (int)((ea >> (21 * k)) & AMPS_MAX_TILES)] = t;
        c.order[slow ? (int)(eb & 0xFFFFFFFFull) : (int)(tb & 0xFFFFFFFFull) + (int)(eb >> 32)] = t;
    }
    if (t < 3) c.counts[t] = (int)((ta >> (21 * t)) & AMPS_MAX_TILES);
}

// Tier maps of up to this many tiles are also kept in the classifying CTA's
// shared memory, so that the lists, the launch order and the log read them
// there instead of from global memory.
constexpr int kClassifyShared = 8192;

__device__ void classify_body(const ClassifyArgs &c)
{
    __shared__ unsigned long long ws[64];
    __shared__ int prom, dem;
    __shared__ uint8_t s_tier[kClassifyShared];
    const int ntiles = c.ntx * c.nty;
    const bool in_smem = ntiles <= kClassifyShared;
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) c.stats[k] += (unsigned long long)c.counts[k] * (unsigned long long)c.stat_steps;
        c.stats[3] += 1;
        *c.step_base += c.advance;
        prom = 0;
        dem = 0;
    }
    __syncthreads();
    int np = 0, nd = 0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        const int x = t % c.ntx, y = t / c.ntx;
        double m = c.metric[t];
        if (y < c.nty - 1) m = fmax(m, c.metric[t + c.ntx]);
        if (y > 0) m = fmax(m, c.metric[t - c.ntx]);
        if (x < c.ntx - 1) m = fmax(m, c.metric[t + 1]);
        if (x > 0) m = fmax(m, c.metric[t - 1]);
        // NaN metric (a NaN in the tile) promotes: fmax drops NaN, so test the tile's own
        const bool nan = !(c.metric[t] == c.metric[t]);
        int nt;
        if (nan || m >= c.thr_hi) nt = c.high_tier;
        else if (c.use_mid && m >= c.thr_lo) nt = TIER_FP32;
        else nt = TIER_HALF;
        if (c.sched) nt = c.sched[(int64_t)min(*c.sched_i, c.sched_n - 1) * ntiles + t];
        const int old = c.tier_cur[t];
        c.tier_prev[t] = (uint8_t)old;
        c.tier_cur[t] = (uint8_t)nt;
        if (in_smem) s_tier[t] = (uint8_t)nt;
        np += nt > old;
        nd += nt < old;
    }
    atomicAdd(&prom, np);
    atomicAdd(&dem, nd);
    __syncthreads();
    const uint8_t *tier = in_smem ? s_tier : c.tier_cur;
    if (c.order && ntiles <= (int)blockDim.x) {
        lists_and_order(c, tier, ws);
    } else {
        lists_from_tiers(tier, ntiles, c.lists, c.counts, ws);
        if (c.order) order_slow_first(c, tier, ws);
    }
    if (threadIdx.x == 0) {
        c.stats[4] += prom;
        c.stats[5] += dem;
        if (c.sched) *c.sched_i += 1;  // every thread read it before the barriers above
    }
    if (c.log && c.max_log > 0) {
        const int n = *c.log_n;
        __syncthreads();
        if (n < c.max_log) {
            for (int t = threadIdx.x; t < ntiles; t += blockDim.x) c.log[(int64_t)n * ntiles + t] = tier[t];
            if (threadIdx.x == 0) *c.log_n = n + 1;
        }
    }
}

// Launched with programmatic dependent launch after the period's last step:
// its launch overlaps that step's tail, and the next step's launch overlaps
// it; it waits for the step (and its writes) before reading the metric.
__global__ void __launch_bounds__(1024) classify_kernel(ClassifyArgs c)
{
    pdl_trigger();
    pdl_wait();
    classify_body(c);
}

// One CTA per ensemble member; member b's arguments are cs[b].
__global__ void __launch_bounds__(1024) classify_batch_kernel(const ClassifyArgs *cs) { classify_body(cs[blockIdx.x]); }

cudaError_t classify(const ClassifyArgs &c, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(1024);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, classify_kernel, c);
}

cudaError_t classify_batch(const ClassifyArgs *cs, int count, cudaStream_t s)
{
    classify_batch_kernel<<<count, 1024, 0, s>>>(cs);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(1024) build_lists_kernel(const uint8_t *tier, int ntiles, int *lists, int *counts)
{
    __shared__ unsigned long long ws[32];
    lists_from_tiers(tier, ntiles, lists, counts, ws);
}

// graingrowth/function.h:38-39,68-73 (and snowflake/function.h:69-70,106-113):
// at every 10th step the update kernel copies the monitored field into the
// snapshot, but a low tile's second 8-column block returns before the copy,
// so its samples in columns 10 and 14 keep the value of the last step at
// which the tile was high.  Here the monitor step's epilogue has written the
// whole lattice (the state the classification just judged); this puts the
// earlier values back where the reference keeps them.  keep holds the
// snapshot as it stood after the previous classification.
__global__ void snap_ref_kernel(double *snap, double *keep, const uint8_t *tier, int ntiles, int total)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int si = i % 16, t = (i / 16) % ntiles;
    if (tier[t] == TIER_HALF && (si % 4) >= 2) snap[i] = keep[i];
    keep[i] = snap[i];
}

cudaError_t snap_ref_fixup(double *snap, double *keep, const uint8_t *tier, int ntiles, int nmon, cudaStream_t s)
{
    const int total = nmon * ntiles * 16;
    snap_ref_kernel<<<(total + 255) / 256, 256, 0, s>>>(snap, keep, tier, ntiles, total);
    return cudaGetLastError();
}

cudaError_t build_lists(const uint8_t *tier, int ntiles, int *lists, int *counts, cudaStream_t s)
{
    build_lists_kernel<<<1, 1024, 0, s>>>(tier, ntiles, lists, counts);
    return cudaGetLastError();
}

__global__ void advance_kernel(int64_t *step_base, int advance, int stat_steps, const int *counts,
                               unsigned long long *stats)
{
    for (int k = 0; k < 3; ++k) stats[k] += (unsigned long long)counts[k] * (unsigned long long)stat_steps;
    *step_base += advance;
}

cudaError_t advance_period(int64_t *step_base, int advance, int stat_steps, const int *counts,
                           unsigned long long *stats, cudaStream_t s)
{
    advance_kernel<<<1, 1, 0, s>>>(step_base, advance, stat_steps, counts, stats);
    return cudaGetLastError();
}

// Period bookkeeping of every ensemble member without a classification
// (one thread per member; advance and stat_steps from each member's args).
__global__ void advance_batch_kernel(const ClassifyArgs *cs, int count)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    const ClassifyArgs &c = cs[b];
    for (int k = 0; k < 3; ++k) c.stats[k] += (unsigned long long)c.counts[k] * (unsigned long long)c.stat_steps;
    *c.step_base += c.advance;
}

cudaError_t advance_batch(const ClassifyArgs *cs, int count, cudaStream_t s)
{
    advance_batch_kernel<<<(count + 127) / 128, 128, 0, s>>>(cs, count);
    return cudaGetLastError();
}

// ---------------------------------------------------------- reductions ----
constexpr int kRedBlocks = 1024;

__global__ void reduce_partial_kernel(Grid g, int field, int kind, double *partials)
{
    __shared__ double red[8];
    double acc = kind == 1 ? INFINITY : (kind == 2 ? -INFINITY : 0.0);
    // contiguous chunk per block, fixed order inside: deterministic
    const int64_t chunk = (g.n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(g.n, lo + chunk);
    for (int64_t c = lo + threadIdx.x; c < hi; c += blockDim.x) {
        const double v = read_cell(g, field, c);
        if (kind == 0) acc += v;
        else if (kind == 1) acc = fmin(acc, v);
        else if (kind == 2) acc = fmax(acc, v);
        else acc += v * v;
    }
    // fixed-shape tree: warp shuffles then warps in order
    if (kind == 1) acc = block_min(acc, red);
    else if (kind == 2) acc = block_max(acc, red);
    else {
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        acc = 0.0;
        for (int w = 0; w < 8; ++w) acc += red[w];
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void reduce_final_kernel(const double *partials, int np, int kind, double *out)
{
    if (threadIdx.x != 0) return;
    double acc = kind == 1 ? INFINITY : (kind == 2 ? -INFINITY : 0.0);
    for (int k = 0; k < np; ++k) {
        if (kind == 1) acc = fmin(acc, partials[k]);
        else if (kind == 2) acc = fmax(acc, partials[k]);
        else acc += partials[k];
    }
    *out = acc;
}

cudaError_t reduce_field(const Grid &g, int field, int kind, double *partials, double *out, cudaStream_t s)
{
    reduce_partial_kernel<<<kRedBlocks, kThreads, 0, s>>>(g, field, kind, partials);
    reduce_final_kernel<<<1, 32, 0, s>>>(partials, kRedBlocks, kind, out);
    return cudaGetLastError();
}

__global__ void compare_partial_kernel(Grid g, int field, const double *other, double *partials)
{
    __shared__ double red[8];
    double mx = 0.0, ss = 0.0;
    const int64_t chunk = (g.n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(g.n, lo + chunk);
    for (int64_t c = lo + threadIdx.x; c < hi; c += blockDim.x) {
        const double d = read_cell(g, field, c) - other[c];
        mx = (fabs(d) > mx || !(d == d)) ? fabs(d) : mx;
        ss += d * d;
    }
    mx = block_max(mx, red);
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        partials[2 * blockIdx.x] = mx;
        partials[2 * blockIdx.x + 1] = t;
    }
}

__global__ void compare_final_kernel(const double *partials, int np, int64_t n, double *out2)
{
    if (threadIdx.x != 0) return;
    double mx = 0.0, ss = 0.0;
    for (int k = 0; k < np; ++k) {
        mx = fmax(mx, partials[2 * k]);
        ss += partials[2 * k + 1];
    }
    out2[0] = mx;
    out2[1] = sqrt(ss / (double)n);
}

cudaError_t compare_field(const Grid &g, int field, const double *other, double *partials, double *out2,
                          cudaStream_t s)
{
    compare_partial_kernel<<<kRedBlocks, kThreads, 0, s>>>(g, field, other, partials);
    compare_final_kernel<<<1, 32, 0, s>>>(partials, kRedBlocks, g.n, out2);
    return cudaGetLastError();
}

}  // namespace amps
