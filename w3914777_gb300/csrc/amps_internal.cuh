// amps_internal.cuh -- shared types and device helpers of libamps.
//
// Data layout in HBM.  Every field has one row-major [ny][nx] array per tier
// in use (half, float, double) and per ping-pong parity; field f of tier t
// lives at store[t][parity] + f*n.  A tile (tile x tile cells) is valid in
// exactly one tier at a time, recorded in a uint8 tier map.  A step reads
// every tile at its input tier (tier_in) and writes it at its output tier
// (tier_out), so promotion/demotion costs nothing beyond the step itself: the
// conversion happens in registers while the tile is staged.
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace amps {

constexpr int kThreads = 256;  // threads per tile CTA
constexpr int kMaxFields = 33; // Q <= 32 order parameters / N <= 32 particles + c
// dynamic shared memory a tile CTA may use (the 227 KB opt-in less room for static shared memory)
constexpr int kMaxDynSmem = 226 * 1024;

enum { TIER_HALF = 0, TIER_FP32 = 1, TIER_FP64 = 2 };

// Model constants (double; each kernel rounds them to its compute type).
struct Phys {
    double dx, dy, dt, dxdy, inv_dxdy;
    // Kobayashi
    double tau, epsb, kappa, delta, aniso, alpha, gama, teq, theta0, pi, noise;
    // grain growth
    double mobil, grcoef, gamma;
    // sintering
    double coefm, coefk, coefl, dvol, dvap, dsur, dgrb, A, B;
    uint64_t seed;
    // grain growth's FP32-tile constants, rounded once on the host (on GB300
    // a handful of FP64 conversions per thread and tile cost ~18% of a step):
    // (float)(dt*L), (float)(2*gamma), (float)kappa, (float)(1/dxdy)
    float gg_dtm, gg_g2, gg_kap, gg_inv;
    // grain growth's binary16 constants (half_arith != 0; enum GgHalf): each
    // double constant rounded to float, then to half, as the reference's
    // __float2half2_rn(double) calls do (graingrowth/end2end_mix.cu:59-67)
    unsigned short gg_h[8];
    // sintering's binary16 constants (half_arith = AMPS_HALF_REF; enum SintHalf),
    // rounded double -> float -> half as sintering/tools.h's
    // lowprecision2highprecision(double) rounds them
    unsigned short sn_h[12];
    // Kobayashi and sintering constants of the non-reference-order tiles,
    // derived on the host in double (kd) and rounded to float (kf), the same
    // values the tiles would derive per thread (index: enum KConst)
    double kd[24];
    float kf[24];
};

enum KConst {
    // Kobayashi: 0.5/dx, 0.5/dy, aniso, theta0, epsb, delta, -epsb*aniso*delta,
    // alpha/pi, gama, teq, noise, dt/tau, kappa, dt, 1/dxdy; the anisotropy
    // mode when it is an even integer 2..16 (else 0), cos and sin of
    // aniso*theta0
    KB_HX, KB_HY, KB_ANISO, KB_THETA0, KB_EPSB, KB_DELTA, KB_ED, KB_M, KB_GAMA, KB_TEQ, KB_NOISE, KB_DTT,
    KB_KAPPA, KB_DT, KB_INV, KB_MODE, KB_C0, KB_S0,
    // sintering: 1/dxdy, B, 2A, 0.5*coefm, dvol, dvap, dsur, dgrb, dt, 12B, dt*coefl, 0.5*coefk
    SN_INV = 0, SN_B, SN_A2, SN_HCM, SN_DVOL, SN_DVAP, SN_DSUR, SN_DGRB, SN_DT, SN_B12, SN_DTL, SN_HCK,
    KCONST_MAX = 24
};

// Indices of Phys::gg_h: dt, L, kappa, dx*dy, gamma (the reference's
// AMPS_HALF_REF expressions) and dt*L, kappa/(dx*dy), 2*gamma (the HFMA2 form).
enum GgHalf { GH_DT, GH_MOB, GH_KAP, GH_DXDY, GH_GAM, GH_DTM, GH_KINV, GH_G2 };
// Indices of Phys::sn_h: coefm, coefk, coefl, dvol, dvap, dsur, dgrb, dx*dy, dt, 2A, B.
enum SintHalf { SH_COEFM, SH_COEFK, SH_COEFL, SH_DVOL, SH_DVAP, SH_DSUR, SH_DGRB, SH_DXDY, SH_DT, SH_A2, SH_B };

// Constant i of Phys::kd / Phys::kf at the tile's compute type.
template <typename CT> __device__ __forceinline__ CT kc(const Phys &ph, int i);
template <> __device__ __forceinline__ double kc<double>(const Phys &ph, int i) { return ph.kd[i]; }
template <> __device__ __forceinline__ float kc<float>(const Phys &ph, int i) { return ph.kf[i]; }

// Arguments of one tier launch of a fused step kernel.
struct StepArgs {
    const void *in[3];        // input parity, per tier (nullptr when the tier is unused)
    void *out[3];             // output parity, per tier
    const uint8_t *tier_in;   // tier of every tile's input data
    const uint8_t *tier_out;  // tier every tile is computed and stored in
    const int *list;          // tiles whose tier_out == this launch's tier
    const int *count;         // count[tier]
    const int *order;         // fused grain-growth step: tile of each CTA (nullptr: blockIdx.x)
    int nx, ny, ntx, nty, nf, bc, stencil;
    int px;                   // row pitch of the storage: ntx * tile (== nx unless the grid is ragged)
    int64_t n;                // field stride of the storage: px * nty * tile (== nx * ny unless ragged)
    // monitor (active when monitor_now != 0)
    int monitor_now, monitor_kind, samples, mfield, mu_lap_fp64, cadence;
    int half_arith;           // grain growth: AMPS_HALF_FP32 / _REF / _HFMA2 (half tiles' arithmetic)
    int tma_stage;            // grain growth: the launch carries a tensor map of the FP32 input (bulk staging)
    const CUtensorMap *tmap;  // ensemble steps: the member's tensor map of its FP32 input in global memory (or null)
    const CUtensorMap *tmap8; // ensemble split tiles: the same input with boxes of kPairFields fields (or null)
    double *metric;           // [ntiles]
    double *snap;             // temporal snapshot: [nmon][ntiles][16] or [nmon][n]
    int *flags;               // bit 0: NaN/Inf seen; bit 1: a bounded device wait gave up
    const int64_t *step_base; // step index of the first step of the current period
    int step_off;             // this step's offset within the period
    Phys ph;
};

// ---- TMA / mbarrier (inline PTX) -------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's generic-proxy shared-memory accesses before later async-proxy (TMA) writes
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// ---- thread-block clusters (the two CTAs of a split tile) --------------------
// Every thread of both CTAs executes each barrier phase (aligned forms).
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
// The address of this CTA's shared-memory location p in the shared memory of cluster CTA `rank`.
__device__ __forceinline__ uint32_t cluster_map(const void *p, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ float4 ld_cluster_f4(uint32_t addr)
{
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr)
                 : "memory");
    return v;
}

// 3-D tiled tensor load of one box into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on one phase of an mbarrier: false when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (int it = 0; it < (1 << 20); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}

// ---- launches ----------------------------------------------------------------
// Launch `kernel` on `s`; pdl: with programmatic stream serialization, so it
// may begin once every CTA of the previous kernel on the stream has started
// (that kernel executes griddepcontrol.launch_dependents).  A kernel launched
// this way reads nothing the previous one writes before its own
// griddepcontrol.wait.
template <typename K, typename... Args>
inline cudaError_t launch_kernel_nt(K kernel, int grid, int threads, size_t smem, cudaStream_t s, bool pdl,
                                   Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename K, typename... Args>
inline cudaError_t launch_kernel(K kernel, int grid, size_t smem, cudaStream_t s, bool pdl, Args... args)
{
    return launch_kernel_nt(kernel, grid, kThreads, smem, s, pdl, args...);
}

// x is +0 (bit pattern 0): an integer test, no floating-point instruction
__device__ __forceinline__ bool pos_zero(double x) { return __double_as_longlong(x) == 0; }
__device__ __forceinline__ bool pos_zero(float x) { return __float_as_uint(x) == 0u; }

// x^3 correctly rounded (to nearest), from error-free products (Dekker's
// exact product through a fused multiply-add: x*x = p + pe exactly, p*x = hi
// + he exactly, so x^3 = hi + he + pe*x with pe*x far below hi's last bit).
// The reference's pow(x, 3) is a library call whose last bit depends on the
// platform's pow; the reference-order sintering kernels take this cube so
// that their FP64 tiles can be pinned bit for bit against the reference's
// kernels built for the CPU with the same cube.  Each operation is rounded
// on its own, in the order written here (the CPU build runs the same five).
__device__ __forceinline__ double cube_rn(double x)
{
    const double p = __dmul_rn(x, x), pe = __fma_rn(x, x, -p);
    const double hi = __dmul_rn(p, x), he = __fma_rn(p, x, -hi);
    return __dadd_rn(hi, __dadd_rn(he, __dmul_rn(pe, x)));
}

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---- boundary mapping ------------------------------------------------------
// Periodic wrap (snowflake/function.h:13-18) or mirror (zero flux) about the
// domain face: -1 -> 0, -2 -> 1, n -> n-1, n+1 -> n-2.
__device__ __forceinline__ int bc_map(int i, int n, int bc)
{
    if (bc == 0) return i < 0 ? i + n : (i >= n ? i - n : i);
    return i < 0 ? -i - 1 : (i >= n ? 2 * n - i - 1 : i);
}

// ---- typed loads / stores ----------------------------------------------------
template <typename CT> __device__ __forceinline__ CT load_tier(const StepArgs &a, int tier, int64_t idx)
{
    if (tier == TIER_FP64) return (CT)((const double *)a.in[2])[idx];
    if (tier == TIER_FP32) return (CT)((const float *)a.in[1])[idx];
    return (CT)__half2float(((const __half *)a.in[0])[idx]);
}

// Load of step input: NC through the read-only (non-coherent) path, for
// kernels in which the data cannot change; otherwise from L2 (.cg), for a
// kernel that also writes what it reads (the persistent multi-step kernel).
template <bool NC, typename V> __device__ __forceinline__ V ldro(const V *p) { return NC ? __ldg(p) : __ldcg(p); }

// 8 consecutive cells from a tier array, 16-byte aligned (idx % 8 == 0).
template <typename CT, bool NC = true>
__device__ __forceinline__ void load8_tier(const StepArgs &a, int tier, int64_t idx, CT v[8])
{
    if (tier == TIER_FP64) {
        const double2 *p = (const double2 *)((const double *)a.in[2] + idx);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double2 d = ldro<NC>(p + k);
            v[2 * k] = (CT)d.x;
            v[2 * k + 1] = (CT)d.y;
        }
    } else if (tier == TIER_FP32) {
        const float4 *p = (const float4 *)((const float *)a.in[1] + idx);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float4 f = ldro<NC>(p + k);
            v[4 * k] = (CT)f.x; v[4 * k + 1] = (CT)f.y; v[4 * k + 2] = (CT)f.z; v[4 * k + 3] = (CT)f.w;
        }
    } else {
        uint4 u = ldro<NC>((const uint4 *)((const __half *)a.in[0] + idx));
        const __half2 *h = (const __half2 *)&u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float2 f = __half22float2(h[k]);
            v[2 * k] = (CT)f.x;
            v[2 * k + 1] = (CT)f.y;
        }
    }
}

// Storage rounding of a computed value (what the next step will read back).
template <int TIER, typename CT> __device__ __forceinline__ CT round_to_tier(CT v)
{
    if (TIER == TIER_HALF) return (CT)__half2float(__float2half_rn((float)v));
    if (TIER == TIER_FP32) return (CT)(float)v;
    return v;
}

// Stochastic rounding of a float to binary16 (half_arith = AMPS_HALF_SR):
// the binary16 neighbours lo <= v <= hi, hi with probability
// (v - lo) / (hi - lo) for the 24-bit uniform r24.  Unbiased, so a change
// below half an ulp accumulates in expectation instead of rounding away at
// every step (Croci & Giles, "Effects of round-to-nearest and stochastic
// rounding in the numerical solution of the heat equation in low
// precision", 2020).  NaN stays NaN; exact values are kept.
__device__ __forceinline__ __half half_sr(float v, uint32_t r24)
{
    const __half lo = __float2half_rd(v), hi = __float2half_ru(v);
    const float flo = __half2float(lo), fhi = __half2float(hi);
    return (float)r24 * 0x1.0p-24f * (fhi - flo) < v - flo ? hi : lo;
}

// 24 uniform bits for the stochastic rounding of cell `cell` at step `step`
// (a SplitMix64 finaliser; a stream of its own, apart from the seeded noise).
__device__ __forceinline__ uint32_t sr_bits(uint64_t seed, uint64_t step, uint64_t cell)
{
    auto mix = [](uint64_t z) {
        z += 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    return (uint32_t)(mix(mix(~seed ^ mix(step)) + cell) >> 40);
}

template <int TIER, typename CT> __device__ __forceinline__ void store_tier(const StepArgs &a, int64_t idx, CT v)
{
    if (TIER == TIER_FP64) ((double *)a.out[2])[idx] = (double)v;
    else if (TIER == TIER_FP32) ((float *)a.out[1])[idx] = (float)v;
    else ((__half *)a.out[0])[idx] = __float2half_rn((float)v);
}

// ---- staged halo tile in shared memory ----------------------------------------
// Field f occupies rows 0..T+2R-1 of pitch P = T + 2*O, the interior starting
// at column O (16-byte aligned), the halo at O-R..O-1 and O+T..O+T+R-1.
// Fields per CTA of a split grain-growth tile (ensemble members with twice
// as many fields run a non-monitor step's tile as a two-CTA cluster).
constexpr int kPairFields = 8;

template <typename CT, int T, int R> struct Stage {
    static constexpr int O = 16 / sizeof(CT) >= R ? 16 / sizeof(CT) : R;
    static constexpr int P = T + 2 * O;
    static constexpr int ROWS = T + 2 * R;
    static constexpr int FIELD = ROWS * P;
    __device__ static CT &at(CT *sm, int f, int r, int c) { return sm[f * FIELD + r * P + c]; }
};

// Tiers of the 3x3 tile neighbourhood of (tx, ty) after the boundary mapping
// (periodic: wrap; zero flux: the mirrored halo of an edge tile lies in the
// tile itself).  Filled by threads 0..8; the caller synchronises.
__device__ __forceinline__ void load_neighbour_tiers(const StepArgs &a, int tx, int ty, uint8_t *nt)
{
    if (threadIdx.x < 9) {
        const int dy = (int)threadIdx.x / 3 - 1, dx = (int)threadIdx.x % 3 - 1;
        int yy = ty + dy, xx = tx + dx;
        if (a.bc == 0) {
            yy = yy < 0 ? yy + a.nty : (yy >= a.nty ? yy - a.nty : yy);
            xx = xx < 0 ? xx + a.ntx : (xx >= a.ntx ? xx - a.ntx : xx);
        } else {
            yy = yy < 0 ? 0 : (yy >= a.nty ? a.nty - 1 : yy);
            xx = xx < 0 ? 0 : (xx >= a.ntx ? a.ntx - 1 : xx);
        }
        nt[threadIdx.x] = a.tier_in[yy * a.ntx + xx];
    }
}

// Stage fields [f0, f0+nfs) of tile (tx, ty) with an R-cell halo, every cell
// read at its owner tile's input tier (nt: load_neighbour_tiers) and
// converted to CT.  Each thread owns fixed slots of the field's footprint --
// an interior 8-cell row segment (16-byte vector loads) or one halo cell --
// whose coordinates, tier and offsets are computed once; the field loop then
// only adds the field stride, issuing a batch of loads before any store.
// SKIP32: the FP32-owned slots already hold their values (copied by this
// same thread: stage_tile_async32 gives every thread the same slots); only
// the others are loaded and converted.
template <typename CT, int T, int R, bool SKIP32 = false, bool NC = true, int NT = kThreads>
__device__ __forceinline__ void stage_tile(const StepArgs &a, CT *sm, const uint8_t *nt, int tx, int ty, int f0,
                                           int nfs)
{
    using S = Stage<CT, T, R>;
    constexpr int SEG = T / 8;
    constexpr int UI = S::ROWS * SEG;    // interior 8-cell segments per field
    constexpr int UH = S::ROWS * 2 * R;  // halo cells per field
    constexpr int U = UI + UH;
    constexpr int SLOTS = (U + NT - 1) / NT;
    constexpr int B0 = (sizeof(CT) == 8 ? 2 : 4) / SLOTS;
    constexpr int B = B0 < 1 ? 1 : B0;   // fields per batch
    const int x0 = tx * T, y0 = ty * T;
    int kind[SLOTS], tier[SLOTS], soff[SLOTS];
    int64_t goff[SLOTS];
#pragma unroll
    for (int q = 0; q < SLOTS; ++q) {
        const int u = threadIdx.x + q * NT;
        kind[q] = 0; tier[q] = 0; soff[q] = 0; goff[q] = 0;
        if (u < UI) {
            const int sg = u % SEG, r = u / SEG;
            const int gy = bc_map(y0 - R + r, a.ny, a.bc);
            kind[q] = 1;
            tier[q] = nt[(r < R ? 0 : (r < T + R ? 3 : 6)) + 1];
            goff[q] = (int64_t)gy * a.px + x0 + 8 * sg;
            soff[q] = r * S::P + S::O + 8 * sg;
        } else if (u < U) {
            const int h = u - UI, k = h % (2 * R), r = h / (2 * R);
            const int gy = bc_map(y0 - R + r, a.ny, a.bc);
            const int lx = k < R ? x0 - R + k : x0 + T + (k - R);
            const int gx = bc_map(lx, a.nx, a.bc);
            kind[q] = 2;
            tier[q] = nt[(r < R ? 0 : (r < T + R ? 3 : 6)) + (k < R ? 0 : 2)];
            goff[q] = (int64_t)gy * a.px + gx;
            soff[q] = r * S::P + (k < R ? S::O - R + k : S::O + T + (k - R));
        }
        if (SKIP32 && tier[q] == TIER_FP32) kind[q] = 0;
    }
    // half-owned slots first: raw halves take half the registers of
    // converted values, so HB fields (all 8 when a thread has one slot) go
    // in one round trip -- 16-byte loads of 8 cells, 2-byte loads of halo
    // cells -- and are converted on the way to shared memory
    constexpr int HB0 = 8 / SLOTS;
    constexpr int HB = HB0 < 1 ? 1 : HB0;
    bool anyh = false;
#pragma unroll
    for (int q = 0; q < SLOTS; ++q) anyh |= kind[q] != 0 && tier[q] == TIER_HALF;
    if (anyh) {
        const __half *hs = (const __half *)a.in[TIER_HALF];
        for (int fb = 0; fb < nfs; fb += HB) {
            uint4 raw[SLOTS][HB];
#pragma unroll
            for (int q = 0; q < SLOTS; ++q)
#pragma unroll
                for (int b = 0; b < HB; ++b) {
                    raw[q][b] = make_uint4(0u, 0u, 0u, 0u);
                    if (kind[q] != 0 && tier[q] == TIER_HALF && fb + b < nfs) {
                        const __half *src = hs + (int64_t)(f0 + fb + b) * a.n + goff[q];
                        if (kind[q] == 1) raw[q][b] = ldro<NC>(reinterpret_cast<const uint4 *>(src));
                        else raw[q][b].x = ldro<NC>(reinterpret_cast<const unsigned short *>(src));
                    }
                }
#pragma unroll
            for (int q = 0; q < SLOTS; ++q)
#pragma unroll
                for (int b = 0; b < HB; ++b) {
                    if (kind[q] == 0 || tier[q] != TIER_HALF || fb + b >= nfs) continue;
                    CT *dst = sm + (fb + b) * S::FIELD + soff[q];
                    if (kind[q] == 2) {
                        dst[0] = (CT)__half2float(__ushort_as_half((unsigned short)raw[q][b].x));
                        continue;
                    }
                    const __half2 *h2 = reinterpret_cast<const __half2 *>(&raw[q][b]);
                    float c[8];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const float2 f = __half22float2(h2[k]);
                        c[2 * k] = f.x;
                        c[2 * k + 1] = f.y;
                    }
                    if (sizeof(CT) == 4) {
                        float4 *d4 = reinterpret_cast<float4 *>(dst);
                        d4[0] = make_float4(c[0], c[1], c[2], c[3]);
                        d4[1] = make_float4(c[4], c[5], c[6], c[7]);
                    } else {
                        double2 *d2 = reinterpret_cast<double2 *>(dst);
#pragma unroll
                        for (int k = 0; k < 4; ++k) d2[k] = make_double2((double)c[2 * k], (double)c[2 * k + 1]);
                    }
                }
        }
#pragma unroll
        for (int q = 0; q < SLOTS; ++q)
            if (tier[q] == TIER_HALF) kind[q] = 0;
    }
    for (int fb = 0; fb < nfs; fb += B) {
        CT v[SLOTS][B][8];
#pragma unroll
        for (int q = 0; q < SLOTS; ++q)
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int f = fb + b;
                if (f < nfs) {
                    const int64_t idx = (int64_t)(f0 + f) * a.n + goff[q];
                    if (kind[q] == 1) load8_tier<CT, NC>(a, tier[q], idx, v[q][b]);
                    else if (kind[q] == 2) v[q][b][0] = load_tier<CT>(a, tier[q], idx);
                }
            }
#pragma unroll
        for (int q = 0; q < SLOTS; ++q)
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int f = fb + b;
                if (f < nfs) {
                    CT *dst = sm + f * S::FIELD + soff[q];
                    if (kind[q] == 1) {  // 16-byte aligned: O, P and FIELD are multiples of 16 bytes
                        if (sizeof(CT) == 4) {
                            float4 *d4 = reinterpret_cast<float4 *>(dst);
                            d4[0] = make_float4((float)v[q][b][0], (float)v[q][b][1], (float)v[q][b][2], (float)v[q][b][3]);
                            d4[1] = make_float4((float)v[q][b][4], (float)v[q][b][5], (float)v[q][b][6], (float)v[q][b][7]);
                        } else {
                            double2 *d2 = reinterpret_cast<double2 *>(dst);
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                d2[k] = make_double2((double)v[q][b][2 * k], (double)v[q][b][2 * k + 1]);
                        }
                    } else if (kind[q] == 2) {
                        dst[0] = v[q][b][0];
                    }
                }
            }
    }
}

// Rows per CTA of the band kernels (a tile of a non-monitor step split into
// T / kBandRows row bands, one CTA each).
constexpr int kBandRows = 8;

// Rows [ly0, ly0 + H) x columns [-R, T + R) (tile-local) of fields
// [f0, f0 + nfs) of tile (tx, ty), each cell read at its owner tile's input
// tier (nt: load_neighbour_tiers) and converted to CT, into dst[f][H][T + 2R]
// (a row band of a tile, for the band kernels).
template <typename CT, int T, int R>
__device__ __forceinline__ void stage_band(const StepArgs &a, CT *dst, const uint8_t *nt, int tx, int ty, int ly0,
                                           int H, int f0, int nfs)
{
    constexpr int W = T + 2 * R;
    const int x0 = tx * T, y0 = ty * T;
    for (int u = threadIdx.x; u < H * W; u += kThreads) {
        const int ly = ly0 + u / W, lx = u % W - R;
        const int tier = nt[(ly < 0 ? 0 : (ly < T ? 3 : 6)) + (lx < 0 ? 0 : (lx < T ? 1 : 2))];
        const int64_t off = (int64_t)bc_map(y0 + ly, a.ny, a.bc) * a.px + bc_map(x0 + lx, a.nx, a.bc);
#pragma unroll 4
        for (int f = 0; f < nfs; ++f) dst[f * H * W + u] = load_tier<CT>(a, tier, (int64_t)(f0 + f) * a.n + off);
    }
}

// Stage fields [f0, f0 + nfs) of a tile whose whole 3x3 neighbourhood holds FP32
// input (no conversion) with an R-cell halo, by asynchronous global->shared
// copies: 16-byte copies for the interior 8-cell row segments (L2 only, the
// values are read once from global memory) and 4-byte copies for the halo
// cells, every field in flight at once, no register round trip.  Same slot
// layout and the same floats as stage_tile; the caller synchronises after
// the final wait issued here (WAIT = false: committed, not waited for --
// cp_async_wait_all before the shared memory is read or reused).
template <int T, int R, bool WAIT = true>
__device__ __forceinline__ void stage_tile_async32(const StepArgs &a, float *sm, int tx, int ty, int nfs, int f0 = 0)
{
    using S = Stage<float, T, R>;
    constexpr int SEG = T / 8;
    constexpr int UI = S::ROWS * SEG;
    constexpr int UH = S::ROWS * 2 * R;
    const float *src = (const float *)a.in[TIER_FP32];
    const int x0 = tx * T, y0 = ty * T;
    for (int u = threadIdx.x; u < UI + UH; u += kThreads) {
        int64_t goff;
        int soff;
        bool seg;
        if (u < UI) {
            const int sg = u % SEG, r = u / SEG;
            goff = (int64_t)bc_map(y0 - R + r, a.ny, a.bc) * a.px + x0 + 8 * sg;
            soff = r * S::P + S::O + 8 * sg;
            seg = true;
        } else {
            const int h = u - UI, k = h % (2 * R), r = h / (2 * R);
            const int lx = k < R ? x0 - R + k : x0 + T + (k - R);
            goff = (int64_t)bc_map(y0 - R + r, a.ny, a.bc) * a.px + bc_map(lx, a.nx, a.bc);
            soff = r * S::P + (k < R ? S::O - R + k : S::O + T + (k - R));
            seg = false;
        }
        for (int f = 0; f < nfs; ++f) {
            const float *g = src + (int64_t)(f0 + f) * a.n + goff;
            const uint32_t d = smem_u32(sm + f * S::FIELD + soff);
            if (seg) {
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(g) : "memory");
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16), "l"(g + 4) : "memory");
            } else {
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(g) : "memory");
            }
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    if (WAIT) asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Wait for this thread's committed asynchronous copies (stage_tile_async32<..., false>).
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// ---- block reductions (warp shuffle + one shared slot per warp) ------------------
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// Max over the block of NT threads; every thread gets the result.  red: >=
// NT/32 doubles of shared memory.
template <int NT = kThreads>
__device__ __forceinline__ double block_max(double v, double *red)
{
    v = warp_max(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = red[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) r = fmax(r, red[w]);
    return r;
}
template <int NT = kThreads>
__device__ __forceinline__ double block_min(double v, double *red)
{
    v = warp_min(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = red[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) r = fmin(r, red[w]);
    return r;
}

// Is (row, col) of a tile on the monitor's sample lattice?  kind 1: spatial
// {0,5,10,15} (snowflake/tools.h:185), kind 2: temporal {2,6,10,14}
// (snowflake/tools.h:203), scaled to the tile; samples==1: every cell.
template <int T> __device__ __forceinline__ int sample_index(int kind, int samples, int row, int col)
{
    if (samples) return 0;
    int ir = -1, ic = -1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int p = kind == 1 ? (k * (T - 1) * 2 + 3) / 6 : T / 8 + k * (T / 4);
        if (row == p) ir = k;
        if (col == p) ic = k;
    }
    return (ir < 0 || ic < 0) ? -1 : ir * 4 + ic;
}

// Address of the temporal-monitor snapshot of one cell (si: lattice index).
template <int T>
__device__ __forceinline__ double *snap_ptr(const StepArgs &a, int mslot, int tile, int64_t gidx, int si)
{
    return a.samples ? a.snap + (int64_t)mslot * a.n + gidx
                     : a.snap + ((int64_t)mslot * a.ntx * a.nty + tile) * 16 + si;
}

// Snapshot value of one cell for kind 2 (0 elsewhere), read before the cell is computed.
template <int T>
__device__ __forceinline__ double snap_prefetch(const StepArgs &a, int mslot, int tile, int row, int col,
                                                int64_t gidx)
{
    if (a.monitor_kind != 2) return 0.0;
    const int si = sample_index<T>(2, a.samples, row, col);
    return si < 0 ? 0.0 : *snap_ptr<T>(a, mslot, tile, gidx, si);
}

// Per-tile monitor accumulator for one field, reduced at the end of the field.
struct MonAcc {
    double mn, mx, dmax;
    float dmaxf;  // kind 3: the largest |(float)v - (float)old|, scaled by the cadence once per tile
    int bad;
};

// Fold one computed (storage-rounded) value into the accumulator.  kind 1:
// spatial range; kind 2: change since the snapshot of the previous monitor
// step (the snapshot is updated here); kind 3: this step's change `v - old`
// scaled by the cadence (no snapshot).  `snapv` is the snapshot value the
// caller prefetched for kind 2.
template <int T>
__device__ __forceinline__ void mon_add(const StepArgs &a, MonAcc &m, int mslot, int tile, int row, int col,
                                        int64_t gidx, double v, double old, double snapv)
{
    // NaN or infinite: the exponent field all ones (integer test, off the FP64 pipe)
    if ((__double2hiint(v) & 0x7ff00000) == 0x7ff00000) m.bad = 1;
    const int si = sample_index<T>(a.monitor_kind == 1 ? 1 : 2, a.samples, row, col);
    if (si < 0) return;
    if (a.monitor_kind == 1) {
        m.mn = fmin(m.mn, v);
        m.mx = fmax(m.mx, v);
    } else if (a.monitor_kind == 2) {
        m.dmax = fmax(m.dmax, fabs(snapv - v));
        *snap_ptr<T>(a, mslot, tile, gidx, si) = v;
    } else {
        // max_i (x_i * cadence) = (max_i x_i) * cadence: rounding is monotone
        m.dmaxf = fmaxf(m.dmaxf, fabsf((float)v - (float)old));
    }
}

// Float accumulator for half/FP32 tiles: the values are floats, so min/max
// are exact in float and the range is taken in double once per tile; the
// rate monitor is defined in FP32 arithmetic; the temporal (snapshot)
// difference stays in double.  Keeps per-cell work off the FP64 pipe.
struct MonAccF {
    float mn, mx, dmaxf;
    double dmax;
    int bad;
    float chk;  // NaN-propagating max of |v| (mon_add_k): non-finite iff a value was
};

__device__ __forceinline__ void mon_reset(const StepArgs &a, MonAccF &m)
{
    m.mn = a.samples ? INFINITY : 1.0f;
    m.mx = a.samples ? -INFINITY : 0.0f;
    m.dmaxf = 0.f;
    m.dmax = 0.0;
    m.bad = 0;
    m.chk = 0.f;
}

__device__ __forceinline__ float fmax_nan(float x, float y)
{
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
    return r;
}

// Kind 2 (temporal) step of the float accumulator, out of line: its FP64
// would otherwise be predicated into every cell of the other kinds.
template <int T>
__device__ __noinline__ void mon_add_tem(const StepArgs &a, MonAccF &m, int mslot, int tile, int64_t gidx, int si,
                                         float v, double snapv)
{
    m.dmax = fmax(m.dmax, fabs(snapv - (double)v));
    *snap_ptr<T>(a, mslot, tile, gidx, si) = (double)v;
}

template <int T>
__device__ __forceinline__ void mon_add(const StepArgs &a, MonAccF &m, int mslot, int tile, int row, int col,
                                        int64_t gidx, float v, float old, double snapv)
{
    if (!(v == v) || isinf(v)) m.bad = 1;
    const int si = sample_index<T>(a.monitor_kind == 1 ? 1 : 2, a.samples, row, col);
    if (si < 0) return;
    if (a.monitor_kind == 1) {
        m.mn = fminf(m.mn, v);
        m.mx = fmaxf(m.mx, v);
    } else if (a.monitor_kind == 2) {
        mon_add_tem<T>(a, m, mslot, tile, gidx, si, v, snapv);
    } else {
        m.dmaxf = fmaxf(m.dmaxf, fabsf(v - old));
    }
}

__device__ __forceinline__ float warp_maxf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int NT = kThreads>
__device__ __forceinline__ float block_maxf(float v, float *red)
{
    v = warp_maxf(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = red[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) r = fmaxf(r, red[w]);
    return r;
}

template <int NT = kThreads>
__device__ __forceinline__ double mon_finish(const StepArgs &a, MonAccF &m, double *red, double metric)
{
    float *redf = reinterpret_cast<float *>(red);
    double v;
    if (a.monitor_kind == 1) {
        const float mx = block_maxf<NT>(m.mx, redf);
        const float mn = -block_maxf<NT>(-m.mn, redf);
        v = (double)mx - (double)mn;
    } else if (a.monitor_kind == 2) {
        v = block_max<NT>(m.dmax, red);
    } else {
        v = (double)block_maxf<NT>(m.dmaxf, redf) * a.cadence;
    }
    if (__syncthreads_or(m.bad) && threadIdx.x == 0) atomicOr(a.flags, 1);
    return fmax(metric, v);
}

// mon_add for a monitor kind fixed at compile time (2: temporal, 3: rate),
// so that no other kind's code -- above all kind 2's FP64 -- is predicated
// into every cell of the others.  Same metric and flag as mon_add.
template <int T, int KIND>
__device__ __forceinline__ void mon_add_k(const StepArgs &a, MonAccF &m, int mslot, int tile, int row, int col,
                                          int64_t gidx, float v, float old)
{
    static_assert(KIND == 2 || KIND == 3, "temporal or rate monitor");
    if constexpr (KIND == 3) {
        // NaN-propagating: a NaN or infinite value (or a step of more than
        // FLT_MAX) leaves dmaxf non-finite, which mon_finish_k flags
        m.dmaxf = fmax_nan(m.dmaxf, fabsf(v - old));
    } else {
        m.chk = fmax_nan(m.chk, fabsf(v));
        const int si = sample_index<T>(2, a.samples, row, col);
        if (si < 0) return;
        double *sp = snap_ptr<T>(a, mslot, tile, gidx, si);
        m.dmax = fmax(m.dmax, fabs(*sp - (double)v));
        *sp = (double)v;
    }
}

// Tile metric of mon_add_k's accumulator (valid in thread 0) and the NaN/Inf flag.
template <int KIND>
__device__ __forceinline__ double mon_finish_k(const StepArgs &a, MonAccF &m, double *red)
{
    double v;
    const float chk = KIND == 3 ? m.dmaxf : m.chk;
    if constexpr (KIND == 3) {
        // the reduction drops a thread's NaN (flagged below) as fmaxf would per cell
        const float mx = block_maxf(m.dmaxf, reinterpret_cast<float *>(red));
        v = threadIdx.x == 0 ? fmax(0.0, (double)mx * a.cadence) : 0.0;
    } else {
        v = fmax(0.0, block_max(m.dmax, red));
    }
    if (__syncthreads_or(!(chk <= 3.402823466e38f)) && threadIdx.x == 0) atomicOr(a.flags, 1);
    return v;
}

__device__ __forceinline__ void mon_reset(const StepArgs &a, MonAcc &m)
{
    // the reference's lattice monitor starts from min=1, max=0 (snowflake/tools.h:184)
    m.mn = a.samples ? INFINITY : 1.0;
    m.mx = a.samples ? -INFINITY : 0.0;
    m.dmax = 0.0;
    m.dmaxf = 0.f;
    m.bad = 0;
}

// Reduce one field's accumulator over the block of NT threads and fold into the tile metric.
template <int NT = kThreads>
__device__ __forceinline__ double mon_finish(const StepArgs &a, MonAcc &m, double *red, double metric)
{
    double v;
    if (a.monitor_kind == 1) {
        const double mx = block_max<NT>(m.mx, red);
        const double mn = block_min<NT>(m.mn, red);
        v = mx - mn;
    } else if (a.monitor_kind == 2) {
        v = block_max<NT>(m.dmax, red);
    } else {
        v = (double)block_maxf<NT>(m.dmaxf, reinterpret_cast<float *>(red)) * a.cadence;
    }
    if (__syncthreads_or(m.bad) && threadIdx.x == 0) atomicOr(a.flags, 1);
    return fmax(metric, v);
}

}  // namespace amps
