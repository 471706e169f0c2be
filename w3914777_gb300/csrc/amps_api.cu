// amps_api.cu -- handle, time loop and state transfer of the C ABI.
//
// The time loop issues, per step, one fused update kernel per tier in use
// (each over a device-side list of the tiles at that tier), and at the end of
// every monitor period one classification kernel (get_type) that rebuilds the
// tier map and the per-tier lists.  Whole periods are captured once into a
// CUDA graph and replayed; the kernels read every step-varying quantity (tier
// map, lists, counts, step index) from device memory, so one graph serves
// every period.
#include "../../include/amps.h"
#include "amps_kernels.h"

#include <cudaTypedefs.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

using namespace amps;

struct amps_handle {
    amps_params p;
    int nf = 0, T = 0, ntx = 0, nty = 0, ntiles = 0;
    int64_t n = 0;   // cells of the domain (nx * ny): host and gathered arrays
    // storage of one field: whole tiles, row pitch px = ntx * T, nty * T rows
    // (ns = px * nty * T; px == nx and ns == n unless the grid is ragged)
    int px = 0;
    int64_t ns = 0;
    bool ragged = false;
    bool used[3] = {false, false, false};
    bool mixed = false, use_mid = false;
    void *store[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    int parity = 0;
    bool transition = false;  // next step reads tiles at tier_prev
    // every tile is at FP64 until the next classification (the first period
    // of a temporal / rate monitor): grain growth takes the staged FP64 kernel
    // when it is prepared (stage64: its FP64 staging fits in shared memory)
    bool all_fp64 = false, stage64 = false;
    uint8_t *d_tier_prev = nullptr, *d_tier_cur = nullptr;
    int *d_lists = nullptr, *d_counts = nullptr;
    int *d_order = nullptr;  // launch order of the fused grain-growth step (adaptive runs)
    double *d_metric = nullptr, *d_snap = nullptr;
    int nmon = 0;
    // ref_snapshot (grain growth, Kobayashi; temporal monitor on the lattice):
    // the snapshot as it stood after the last classification
    double *d_snap_keep = nullptr;
    // tier schedule (amps_set_tier_schedule): sched_n maps of ntiles bytes,
    // the next one to use at *d_sched_i
    uint8_t *d_sched = nullptr;
    int sched_n = 0;
    int *d_sched_i = nullptr;
    // on-demand monitor (amps_measure_tiles): its own snapshot and metric
    double *d_msnap = nullptr, *d_mmetric = nullptr;
    bool msnap_valid = false;
    unsigned long long *d_stats = nullptr;
    int *d_flags = nullptr;
    uint8_t *d_log = nullptr;
    int *d_log_n = nullptr;
    int64_t *d_step_base = nullptr;
    double *d_stage = nullptr, *d_partials = nullptr, *d_out = nullptr;
    double *h_pinned = nullptr;  // nf*n doubles, page-locked
    cudaStream_t own = nullptr, stream = nullptr;
    // private stream on which a handle working on the default stream (which
    // cannot be captured) captures its period graphs; replayed on the default stream
    cudaStream_t cap = nullptr;

    int64_t step = 0;
    int64_t launches = 0;  // kernels enqueued by the run loop (graph replays add their graph's count)
    bool graphs = true;
    std::map<int, cudaGraphExec_t> graph;  // key: parity | transition<<1 | all_fp64<<2
    std::map<int, int64_t> graph_launches;  // kernels in each period graph
    std::string err;
    // kernel timing
    bool profiling = false;
    struct Ev { int tier; cudaEvent_t a, b; int n; };  // n launches between a and b
    std::vector<Ev> evs;
    std::vector<cudaEvent_t> ev_stash;  // created ahead of a captured profiled period
    // grain growth: persistent multi-step kernel for the interior steps of a
    // period (d_flow: per-tile step counters, then the item counter)
    bool use_flow = false;
    int *d_flow = nullptr;
    // grain growth: persistent TMA kernel over the FP32 ping-pong buffers
    bool use_tma = false;
    bool tma_stage = false;  // tm[] encoded: the fused step stages interior tiles by tensor copy
    double *d_mu = nullptr;  // sintering, AMPS_HALF_REF: the chemical potential of every cell
    int tma_grid = 0;
    alignas(64) CUtensorMap tm[2];
    // diagnostics scratch (allocated on first use): lab, parent (n ints each),
    // one FP64 field, counters, bounding box
    char *d_diag = nullptr;
    double prof_ms[4] = {0, 0, 0, 0};
    int64_t prof_launches[4] = {0, 0, 0, 0};
    unsigned long long prof_stats0[3] = {0, 0, 0};
};

static std::string g_create_err;

#define FAIL(h, code, ...)                                         \
    do {                                                           \
        char _b[512];                                              \
        snprintf(_b, sizeof _b, __VA_ARGS__);                      \
        (h)->err = _b;                                             \
        return (code);                                             \
    } while (0)
#define CK(h, call)                                                                              \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

extern "C" const char *amps_status_string(int s)
{
    switch (s) {
    case AMPS_OK: return "ok";
    case AMPS_ERR_INVALID: return "invalid argument";
    case AMPS_ERR_CUDA: return "CUDA error";
    case AMPS_ERR_ALLOC: return "allocation failed";
    case AMPS_ERR_TIMEOUT: return "device wait timed out";
    case AMPS_ERR_NUMERIC: return "NaN or Inf in the state";
    case AMPS_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

extern "C" const char *amps_last_error(const amps_handle *h)
{
    return h ? h->err.c_str() : g_create_err.c_str();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// [nf][ny][nx] float array (nx: the storage's row pitch, ny: its rows) ->
// box {40 columns, 34 rows, nf fields}: a 32x32 tile with a 1-cell halo and
// its columns padded to 16-byte boundaries.
// boxf: fields per box (0: all nf)
static bool encode_field_map(CUtensorMap *tm, void *base, int nx, int ny, int nf, int boxf = 0)
{
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nf};
    const cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    const cuuint32_t box[3] = {40, 34, (cuuint32_t)(boxf > 0 ? boxf : nf)};
    const cuuint32_t es[3] = {1, 1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

static size_t tier_size(int t) { return t == TIER_FP64 ? 8 : (t == TIER_FP32 ? 4 : 2); }

static Phys make_phys(const amps_params &p)
{
    Phys ph;
    memset(&ph, 0, sizeof ph);
    ph.dx = p.dx; ph.dy = p.dy; ph.dt = p.dt;
    ph.dxdy = p.dx * p.dy;
    ph.inv_dxdy = 1.0 / ph.dxdy;
    ph.tau = p.tau; ph.epsb = p.epsb; ph.kappa = p.kappa; ph.delta = p.delta; ph.aniso = p.aniso;
    ph.alpha = p.alpha; ph.gama = p.gama; ph.teq = p.teq; ph.theta0 = p.theta0; ph.pi = p.pi; ph.noise = p.noise;
    ph.mobil = p.mobil; ph.grcoef = p.grcoef; ph.gamma = p.gamma;
    ph.coefm = p.coefm; ph.coefk = p.coefk; ph.coefl = p.coefl; ph.dvol = p.dvol; ph.dvap = p.dvap;
    ph.dsur = p.dsur; ph.dgrb = p.dgrb; ph.A = p.A; ph.B = p.B;
    ph.seed = p.seed;
    ph.gg_dtm = (float)(ph.dt * ph.mobil);
    ph.gg_g2 = (float)(2.0 * ph.gamma);
    ph.gg_kap = (float)ph.grcoef;
    ph.gg_inv = (float)ph.inv_dxdy;
    {
        const double gh[8] = {ph.dt, ph.mobil, ph.grcoef, ph.dxdy, ph.gamma, ph.dt * ph.mobil,
                              ph.grcoef * ph.inv_dxdy, 2.0 * ph.gamma};
        for (int i = 0; i < 8; ++i) ph.gg_h[i] = __half_as_ushort(__float2half_rn((float)gh[i]));
        const double sh[11] = {ph.coefm, ph.coefk, ph.coefl, ph.dvol, ph.dvap, ph.dsur, ph.dgrb, ph.dxdy, ph.dt,
                               2.0 * ph.A, ph.B};
        for (int i = 0; i < 11; ++i) ph.sn_h[i] = __half_as_ushort(__float2half_rn((float)sh[i]));
    }
    double *k = ph.kd;
    if (p.model == AMPS_KOBAYASHI) {
        k[KB_HX] = 0.5 / ph.dx; k[KB_HY] = 0.5 / ph.dy; k[KB_ANISO] = ph.aniso; k[KB_THETA0] = ph.theta0;
        k[KB_EPSB] = ph.epsb; k[KB_DELTA] = ph.delta; k[KB_ED] = -ph.epsb * ph.aniso * ph.delta;
        k[KB_M] = ph.alpha / ph.pi; k[KB_GAMA] = ph.gama; k[KB_TEQ] = ph.teq; k[KB_NOISE] = ph.noise;
        k[KB_DTT] = ph.dt / ph.tau; k[KB_KAPPA] = ph.kappa; k[KB_DT] = ph.dt; k[KB_INV] = ph.inv_dxdy;
        const bool even = ph.aniso >= 2 && ph.aniso <= 16 && ph.aniso == 2 * std::floor(ph.aniso / 2);
        k[KB_MODE] = even ? ph.aniso : 0;
        k[KB_C0] = std::cos(ph.aniso * ph.theta0); k[KB_S0] = std::sin(ph.aniso * ph.theta0);
    } else if (p.model == AMPS_SINTERING) {
        k[SN_INV] = ph.inv_dxdy; k[SN_B] = ph.B; k[SN_A2] = 2.0 * ph.A; k[SN_HCM] = 0.5 * ph.coefm;
        k[SN_DVOL] = ph.dvol; k[SN_DVAP] = ph.dvap; k[SN_DSUR] = ph.dsur; k[SN_DGRB] = ph.dgrb; k[SN_DT] = ph.dt;
        k[SN_B12] = 12.0 * ph.B; k[SN_DTL] = ph.dt * ph.coefl; k[SN_HCK] = 0.5 * ph.coefk;
    }
    for (int i = 0; i < KCONST_MAX; ++i) ph.kf[i] = (float)ph.kd[i];
    return ph;
}

static size_t kernel_smem(const amps_params &p, int tier, int nf, bool only64)
{
    if (p.model == AMPS_GRAINGROWTH) return gg_smem_bytes(p.tile, only64 ? TIER_FP64 : -1, nf);
    if (p.model == AMPS_KOBAYASHI) return kob_smem_bytes(p.tile, tier);
    return sint_smem_bytes(p.tile, tier, nf, p.mu_lap_fp64 || tier == TIER_FP64);
}

static void free_all(amps_handle *h)
{
    for (auto &e : h->evs) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    h->evs.clear();
    for (cudaEvent_t e : h->ev_stash) cudaEventDestroy(e);
    h->ev_stash.clear();
    for (auto &kv : h->graph) cudaGraphExecDestroy(kv.second);
    h->graph.clear();
    for (int t = 0; t < 3; ++t)
        for (int q = 0; q < 2; ++q)
            if (h->store[t][q]) cudaFree(h->store[t][q]);
    void *ps[] = {h->d_tier_prev, h->d_tier_cur, h->d_lists, h->d_order, h->d_counts, h->d_metric, h->d_snap, h->d_stats,
                  h->d_flags, h->d_log, h->d_log_n, h->d_step_base, h->d_stage, h->d_partials, h->d_out,
                  h->d_diag, h->d_sched, h->d_sched_i, h->d_msnap, h->d_mmetric, h->d_snap_keep, h->d_flow,
                  h->d_mu};
    for (void *q : ps)
        if (q) cudaFree(q);
    if (h->h_pinned) cudaFreeHost(h->h_pinned);
    if (h->own) cudaStreamDestroy(h->own);
    if (h->cap) cudaStreamDestroy(h->cap);
}

extern "C" int amps_create(const amps_params *p, amps_handle **out)
{
    char msg[256];
    if (!out) return AMPS_ERR_INVALID;
    *out = nullptr;
    if (amps_check_params(p, msg, sizeof msg) != AMPS_OK) {
        g_create_err = msg;
        return AMPS_ERR_INVALID;
    }
    amps_handle *h = new (std::nothrow) amps_handle();
    if (!h) return AMPS_ERR_ALLOC;
    h->p = *p;
    h->nf = amps_num_fields(p);
    h->T = p->tile;
    h->ntx = (p->nx + p->tile - 1) / p->tile;
    h->nty = (p->ny + p->tile - 1) / p->tile;
    h->ntiles = h->ntx * h->nty;
    h->n = (int64_t)p->nx * p->ny;
    h->px = h->ntx * p->tile;
    h->ns = (int64_t)h->px * h->nty * p->tile;
    h->ragged = h->ns != h->n;
    const int high = p->high_tier;
    h->mixed = p->mode == AMPS_END2END_MIX;
    h->use_mid = h->mixed && high == TIER_FP64 && p->thr_lo < p->thr_hi;
    switch (p->mode) {
    case AMPS_PUREHIGH: h->used[high] = true; break;
    case AMPS_PURELOW: h->used[TIER_HALF] = true; break;
    default:
        h->used[TIER_HALF] = h->used[high] = true;
        if (h->use_mid) h->used[TIER_FP32] = true;
    }
    for (int t = 0; t < 3; ++t)
        if (h->used[t] && kernel_smem(*p, t, h->nf, h->used[TIER_FP64] && !h->used[TIER_FP32] && !h->used[TIER_HALF])
                              > (size_t)kMaxDynSmem) {
            g_create_err = "tile staging exceeds 226 KB of shared memory: use tile=16 or fewer fields";
            delete h;
            return AMPS_ERR_UNSUPPORTED;
        }
    auto fail = [&](int code, const char *what) {
        g_create_err = std::string("allocation failed: ") + what;
        free_all(h);
        delete h;
        return code;
    };
#define ALLOC(ptr, bytes, what)                                              \
    if (cudaMalloc((void **)&(ptr), (bytes)) != cudaSuccess) return fail(AMPS_ERR_ALLOC, what);
    for (int t = 0; t < 3; ++t)
        if (h->used[t])
            for (int q = 0; q < 2; ++q) ALLOC(h->store[t][q], (size_t)h->nf * h->ns * tier_size(t), "field storage");
    ALLOC(h->d_tier_prev, h->ntiles, "tier map");
    ALLOC(h->d_tier_cur, h->ntiles, "tier map");
    ALLOC(h->d_lists, sizeof(int) * 3 * h->ntiles, "tile lists");
    ALLOC(h->d_order, sizeof(int) * h->ntiles, "launch order");
    ALLOC(h->d_counts, sizeof(int) * 4, "tile counts");
    ALLOC(h->d_metric, sizeof(double) * h->ntiles, "monitor metric");
    h->nmon = p->monitor_field < 0 ? h->nf : 1;
    const size_t snap = p->monitor_samples ? (size_t)h->nmon * h->ns : (size_t)h->nmon * h->ntiles * 16;
    ALLOC(h->d_snap, sizeof(double) * snap, "monitor snapshot");
    if (p->ref_snapshot && p->monitor == AMPS_MONITOR_TEM && !p->monitor_samples && p->model != AMPS_SINTERING &&
        h->mixed)
        ALLOC(h->d_snap_keep, sizeof(double) * snap, "reference snapshot");
    ALLOC(h->d_stats, sizeof(unsigned long long) * 8, "stats");
    ALLOC(h->d_flags, sizeof(int) * 4, "flags");
    ALLOC(h->d_log_n, sizeof(int), "log count");
    if (p->max_log > 0) ALLOC(h->d_log, (size_t)p->max_log * h->ntiles, "decision log");
    ALLOC(h->d_step_base, sizeof(int64_t), "step counter");
    if (p->model == AMPS_SINTERING && p->half_arith == AMPS_HALF_REF)
        ALLOC(h->d_mu, sizeof(double) * h->n, "chemical potential");
    ALLOC(h->d_stage, sizeof(double) * h->nf * h->n, "staging");
    ALLOC(h->d_partials, sizeof(double) * 2 * 1024, "partials");
    ALLOC(h->d_out, sizeof(double) * 4, "result");
    if (cudaMallocHost((void **)&h->h_pinned, sizeof(double) * h->nf * h->n) != cudaSuccess)
        return fail(AMPS_ERR_ALLOC, "pinned staging");
#undef ALLOC
    if (cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking) != cudaSuccess)
        return fail(AMPS_ERR_CUDA, "stream");

    h->stream = h->own;
    cudaMemsetAsync(h->d_stats, 0, sizeof(unsigned long long) * 8, h->stream);
    cudaMemsetAsync(h->d_flags, 0, sizeof(int) * 4, h->stream);
    cudaMemsetAsync(h->d_log_n, 0, sizeof(int), h->stream);
    cudaMemsetAsync(h->d_step_base, 0, sizeof(int64_t), h->stream);
    cudaMemsetAsync(h->d_metric, 0, sizeof(double) * h->ntiles, h->stream);
    cudaMemsetAsync(h->d_snap, 0, sizeof(double) * snap, h->stream);
    // zero state at the starting tier so that an un-initialised run is defined
    for (int t = 0; t < 3; ++t)
        if (h->used[t])
            for (int q = 0; q < 2; ++q) cudaMemsetAsync(h->store[t][q], 0, (size_t)h->nf * h->ns * tier_size(t), h->stream);
    for (int t = 0; t < 3; ++t) {
        if (!h->used[t]) continue;
        cudaError_t pe;
        if (p->model == AMPS_GRAINGROWTH) {
            const bool only64 = h->used[TIER_FP64] && !h->used[TIER_FP32] && !h->used[TIER_HALF];
            pe = gg_prepare(h->T, only64 ? TIER_FP64 : -1, p->ref_order != 0, p->half_arith, h->ragged);
        }
        else if (p->model == AMPS_KOBAYASHI) pe = kob_prepare(h->T, t, p->ref_order != 0);
        else pe = sint_prepare(h->T, t, p->ref_order != 0, p->mu_lap_fp64 != 0);
        if (pe == cudaSuccess && p->model != AMPS_GRAINGROWTH && t == TIER_FP32 && h->used[TIER_HALF])
            pe = p->model == AMPS_KOBAYASHI ? kob_prepare_lo(h->T) : sint_prepare_lo(h->T, p->mu_lap_fp64 != 0);
        if (pe != cudaSuccess) {
            g_create_err = std::string("kernel attributes: ") + cudaGetErrorString(pe);
            free_all(h);
            delete h;
            return AMPS_ERR_CUDA;
        }
    }
    // adaptive grain growth with an FP64 high tier: the staged FP64 kernel for
    // periods whose tiles are all FP64 (a refused attribute leaves the fused kernel)
    if (p->model == AMPS_GRAINGROWTH && h->mixed && high == TIER_FP64 &&
        kernel_smem(*p, TIER_FP64, h->nf, true) <= (size_t)kMaxDynSmem)
        h->stage64 = gg_prepare(h->T, TIER_FP64, p->ref_order != 0, 0) == cudaSuccess;
    cudaGetLastError();
    {
        // grain growth, 32x32 tiles, an FP32 tier: tensor maps of the two FP32
        // parities, so that the fused step fetches interior tiles' FP32
        // neighbourhoods by one bulk tensor copy each (AMPS_DISABLE_TMA_STAGE=1:
        // per-thread asynchronous copies only)
        const char *off = getenv("AMPS_DISABLE_TMA_STAGE");
        if (p->model == AMPS_GRAINGROWTH && p->tile == 32 && h->used[TIER_FP32] && !(off && off[0] == '1'))
            h->tma_stage = encode_field_map(&h->tm[0], h->store[TIER_FP32][0], h->px, h->nty * h->T, h->nf) &&
                           encode_field_map(&h->tm[1], h->store[TIER_FP32][1], h->px, h->nty * h->T, h->nf);
        cudaGetLastError();
    }
    {
        // persistent TMA kernel (opt-in, AMPS_ENABLE_TMA=1): grain growth, 32x32 tiles, an FP32 tier, few
        // enough fields for two buffers.  Measured slower than the 4-CTA/SM staged kernel on GB300 (two
        // double-buffered CTAs per SM leave 16 warps for a latency-bound compute phase), so not the default.
        const bool only64 = h->used[TIER_FP64] && !h->used[TIER_FP32] && !h->used[TIER_HALF];
        const char *on = getenv("AMPS_ENABLE_TMA");
        if (p->model == AMPS_GRAINGROWTH && p->tile == 32 && h->used[TIER_FP32] && !only64 && h->nf <= kTmaMaxFields &&
            p->half_arith == AMPS_HALF_FP32 && !h->ragged && on && on[0] == '1') {
            int bps = 0, dev = 0, sms = 0;
            if (encode_field_map(&h->tm[0], h->store[TIER_FP32][0], h->px, h->nty * h->T, h->nf) &&
                encode_field_map(&h->tm[1], h->store[TIER_FP32][1], h->px, h->nty * h->T, h->nf) &&
                gg_prepare_tma(p->ref_order != 0, h->nf, &bps) == cudaSuccess && bps > 0 &&
                cudaGetDevice(&dev) == cudaSuccess &&
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) {
                h->use_tma = true;
                h->tma_grid = bps * sms < h->ntiles ? bps * sms : h->ntiles;
            }
            cudaGetLastError();  // a refused attribute / encode leaves the generic kernel in charge
        }
    }
    {
        // multi-step kernel for the interior steps of a period (opt-in,
        // AMPS_ENABLE_FLOW=1; grain growth, 32x32 tiles, the fused step's
        // half/FP32 arithmetic).  Measured slower than one launch per step on
        // GB300 (1024^2 Q=8 all-FP32: 14.7 against 13.5 us a step; 4096^2:
        // 241 against 204): each CTA's claim, neighbour wait and release cost
        // more than the launch tail they remove.
        const bool only64 = h->used[TIER_FP64] && !h->used[TIER_FP32] && !h->used[TIER_HALF];
        const char *on = getenv("AMPS_ENABLE_FLOW");
        if (p->model == AMPS_GRAINGROWTH && p->tile == 32 && !only64 && p->half_arith == AMPS_HALF_FP32 &&
            !h->use_tma && !h->ragged && on && on[0] == '1' && gg_prepare_flow(p->ref_order != 0) == cudaSuccess &&
            cudaMalloc((void **)&h->d_flow, sizeof(int) * (h->ntiles + 1)) == cudaSuccess)
            h->use_flow = true;
        cudaGetLastError();  // a refused attribute or allocation leaves one launch per step
    }
    const int start = p->mode == AMPS_PURELOW ? TIER_HALF : high;
    cudaMemsetAsync(h->d_tier_cur, start, h->ntiles, h->stream);
    cudaMemsetAsync(h->d_tier_prev, start, h->ntiles, h->stream);
    build_lists(h->d_tier_cur, h->ntiles, h->d_lists, h->d_counts, h->stream);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        g_create_err = std::string("initialisation: ") + cudaGetErrorString(e);
        free_all(h);
        delete h;
        return AMPS_ERR_CUDA;
    }
    *out = h;
    return AMPS_OK;
}

extern "C" int amps_destroy(amps_handle *h)
{
    if (!h) return AMPS_ERR_INVALID;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return AMPS_OK;
}

extern "C" int amps_set_stream(amps_handle *h, void *stream)
{
    if (!h) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    h->stream = stream ? (cudaStream_t)stream : h->own;
    return AMPS_OK;
}

extern "C" int amps_synchronize(amps_handle *h)
{
    if (!h) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    int flag = 0;
    CK(h, cudaMemcpy(&flag, h->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag & 2) FAIL(h, AMPS_ERR_TIMEOUT, "a bounded device wait gave up (a tensor copy, or a multi-step "
                                            "kernel's wait on a neighbouring tile, did not complete)");
    if (flag & 1) FAIL(h, AMPS_ERR_NUMERIC, "NaN or Inf detected by the monitor");
    return AMPS_OK;
}

extern "C" int amps_set_graphs(amps_handle *h, int enable)
{
    if (!h) return AMPS_ERR_INVALID;
    h->graphs = enable != 0;
    return AMPS_OK;
}

// ------------------------------------------------------------------ state ----
static Grid grid_view(amps_handle *h, int parity, const uint8_t *tier)
{
    Grid g;
    for (int t = 0; t < 3; ++t) g.store[t] = h->store[t][parity];
    g.tier = tier;
    g.nx = h->p.nx; g.ny = h->p.ny; g.ntx = h->ntx; g.nty = h->nty; g.tile = h->T; g.nf = h->nf; g.n = h->n;
    g.px = h->px; g.fs = h->ns;
    return g;
}

static const uint8_t *live_tiers(amps_handle *h) { return h->transition ? h->d_tier_prev : h->d_tier_cur; }

// Tier map of the current period from the monitor on a resting state:
// Monitor1 classifies the state itself; Monitor2 starts all-high (the
// reference's warm start phi_old = (phi==0), snowflake/end2end_mix.cu:44-46).
static int reclassify_resting(amps_handle *h)
{
    const amps_params &p = h->p;
    Grid g = grid_view(h, h->parity, live_tiers(h));
    if (p.mode == AMPS_END2END_MIX) {
        if (p.monitor != AMPS_MONITOR_SPA) {
            if (p.monitor == AMPS_MONITOR_TEM)
                CK(h, monitor_state(g, 2, p.monitor_samples, p.monitor_field, nullptr, h->d_snap, 1, h->d_flags,
                                    h->stream));
            // every tile to the high tier for the first period
            h->all_fp64 = h->stage64 && h->sched_n == 0;
            std::vector<double> big(h->ntiles, 1e300);
            CK(h, cudaMemcpyAsync(h->d_metric, big.data(), sizeof(double) * h->ntiles, cudaMemcpyHostToDevice, h->stream));
            CK(h, cudaStreamSynchronize(h->stream));
        } else {
            h->all_fp64 = false;
            CK(h, monitor_state(g, 1, p.monitor_samples, p.monitor_field, h->d_metric, nullptr, 0, h->d_flags, h->stream));
        }
        ClassifyArgs c{};
        c.metric = h->d_metric; c.tier_prev = h->d_tier_prev; c.tier_cur = h->d_tier_cur;
        c.lists = h->d_lists; c.counts = h->d_counts; c.ntx = h->ntx; c.nty = h->nty;
        c.thr_lo = p.thr_lo; c.thr_hi = p.thr_hi; c.high_tier = p.high_tier; c.use_mid = h->use_mid;
        c.stats = h->d_stats; c.log = h->d_log; c.log_n = h->d_log_n; c.max_log = p.max_log;
        c.step_base = h->d_step_base; c.advance = 0; c.stat_steps = 0;
        c.order = h->d_order; c.bc = p.bc;
        if (h->sched_n) {
            // a schedule restarts with its first map at every new state
            CK(h, cudaMemsetAsync(h->d_sched_i, 0, sizeof(int), h->stream));
            c.sched = h->d_sched; c.sched_n = h->sched_n; c.sched_i = h->d_sched_i;
        }
        CK(h, classify(c, h->stream));
        if (h->d_snap_keep && !h->sched_n)
            CK(h, snap_ref_fixup(h->d_snap, h->d_snap_keep, h->d_tier_cur, h->ntiles, h->nmon, h->stream));
        h->transition = true;
    }
    return AMPS_OK;
}

// Static tier maps for the non-adaptive modes.
static int static_tiers(amps_handle *h)
{
    const amps_params &p = h->p;
    std::vector<uint8_t> m(h->ntiles, (uint8_t)(p.mode == AMPS_PURELOW ? TIER_HALF : p.high_tier));
    if (p.mode == AMPS_GRAM1 || p.mode == AMPS_GRAM2) {
        // snowflake/function.h:72-79: GRAM1 tiles below ratio*ntiles are low;
        // GRAM2 tiles whose index mod 100 is below 100*ratio are low
        for (int t = 0; t < h->ntiles; ++t) {
            const bool low = p.mode == AMPS_GRAM1 ? t < h->ntiles * p.gram_ratio : (t % 100) < 100 * p.gram_ratio;
            m[t] = low ? TIER_HALF : (uint8_t)p.high_tier;
        }
    }
    if (p.mode == AMPS_END2END_MIX) return AMPS_OK;
    CK(h, cudaMemcpyAsync(h->d_tier_cur, m.data(), h->ntiles, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->d_tier_prev, m.data(), h->ntiles, cudaMemcpyHostToDevice, h->stream));
    CK(h, build_lists(h->d_tier_cur, h->ntiles, h->d_lists, h->d_counts, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return AMPS_OK;
}

// Write the staged [nf][n] doubles (d_stage) as the current state.
static int commit_stage(amps_handle *h)
{
    if (h->p.mode == AMPS_END2END_MIX) {
        // resting state lives at the high tier until the monitor has looked at it
        CK(h, cudaMemsetAsync(h->d_tier_cur, h->p.high_tier, h->ntiles, h->stream));
        CK(h, cudaMemsetAsync(h->d_tier_prev, h->p.high_tier, h->ntiles, h->stream));
        h->transition = false;
        Grid g = grid_view(h, h->parity, h->d_tier_cur);
        CK(h, scatter_fields(g, h->d_stage, 0, h->stream));
        int r = reclassify_resting(h);
        if (r) return r;
    } else {
        int r = static_tiers(h);
        if (r) return r;
        h->transition = false;
        Grid g = grid_view(h, h->parity, h->d_tier_cur);
        CK(h, scatter_fields(g, h->d_stage, 0, h->stream));
    }
    return AMPS_OK;
}

extern "C" int amps_init(amps_handle *h, int kind)
{
    if (!h) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    std::vector<double *> f(h->nf);
    for (int k = 0; k < h->nf; ++k) f[k] = h->h_pinned + (int64_t)k * h->n;
    int r = amps_init_host(&h->p, kind, f.data());
    if (r) FAIL(h, r, "initial state: invalid kind %d or particle placement failed", kind);
    CK(h, cudaMemcpyAsync(h->d_stage, h->h_pinned, sizeof(double) * h->nf * h->n, cudaMemcpyHostToDevice, h->stream));
    h->step = 0;
    CK(h, cudaMemsetAsync(h->d_step_base, 0, sizeof(int64_t), h->stream));
    return commit_stage(h);
}

static int set_impl(amps_handle *h, int f0, int nfs, const void *src, int dtype, int on_device)
{
    if (!h || !src || (dtype != AMPS_F64 && dtype != AMPS_F32) || f0 < 0 || f0 + nfs > h->nf)
        return AMPS_ERR_INVALID;
    // every field must be in the stage: fetch the others first
    Grid live = grid_view(h, h->parity, live_tiers(h));
    if (nfs < h->nf) CK(h, gather_fields(live, h->d_stage, 0, 0, h->nf, h->stream));
    const size_t cnt = (size_t)nfs * h->n;
    double *dst = h->d_stage + (int64_t)f0 * h->n;
    if (dtype == AMPS_F64) {
        CK(h, cudaMemcpyAsync(dst, src, cnt * 8, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    } else {
        // float input (a set-up path, not the time loop): widened to double
        // on the host, through the pinned buffer
        CK(h, cudaStreamSynchronize(h->stream));
        if (on_device) {
            std::vector<float> tmp(cnt);
            CK(h, cudaMemcpy(tmp.data(), src, cnt * 4, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < cnt; ++i) h->h_pinned[i] = tmp[i];
        } else {
            for (size_t i = 0; i < cnt; ++i) h->h_pinned[i] = ((const float *)src)[i];
        }
        CK(h, cudaMemcpyAsync(dst, h->h_pinned, cnt * 8, cudaMemcpyHostToDevice, h->stream));
    }
    return commit_stage(h);
}

extern "C" int amps_set_field(amps_handle *h, int field, const void *src, int dtype, int on_device)
{
    return set_impl(h, field, 1, src, dtype, on_device);
}

extern "C" int amps_set_fields(amps_handle *h, const void *src, int dtype, int on_device)
{
    return set_impl(h, 0, h ? h->nf : 0, src, dtype, on_device);
}

static int get_impl(amps_handle *h, int f0, int nfs, void *dst, int dtype, int on_device)
{
    if (!h || !dst || (dtype != AMPS_F64 && dtype != AMPS_F32) || f0 < 0 || f0 + nfs > h->nf)
        return AMPS_ERR_INVALID;
    Grid g = grid_view(h, h->parity, live_tiers(h));
    const size_t bytes = (size_t)nfs * h->n * (dtype == AMPS_F64 ? 8 : 4);
    if (on_device) {
        CK(h, gather_fields(g, dst, dtype == AMPS_F32, f0, nfs, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    } else {
        CK(h, gather_fields(g, h->d_stage, dtype == AMPS_F32, f0, nfs, h->stream));
        CK(h, cudaMemcpyAsync(dst, h->d_stage, bytes, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    return AMPS_OK;
}

extern "C" int amps_get_field(amps_handle *h, int field, void *dst, int dtype, int on_device)
{
    return get_impl(h, field, 1, dst, dtype, on_device);
}

extern "C" int amps_get_fields(amps_handle *h, void *dst, int dtype, int on_device)
{
    return get_impl(h, 0, h ? h->nf : 0, dst, dtype, on_device);
}

// -------------------------------------------------------------- time loop ----
// Arguments of the step at offset step_off of a period, from parity
// `parity` (transition: this step reads tiles at their previous tier).
static StepArgs step_args(const amps_handle *h, int parity, bool transition, int step_off, bool monitor_now)
{
    const amps_params &p = h->p;
    StepArgs a;
    memset(&a, 0, sizeof a);
    for (int t = 0; t < 3; ++t) {
        a.in[t] = h->store[t][parity];
        a.out[t] = h->store[t][parity ^ 1];
    }
    a.tier_in = transition ? h->d_tier_prev : h->d_tier_cur;
    a.tier_out = h->d_tier_cur;
    a.count = h->d_counts;
    // adaptive runs: slow tiles first (the classification's launch order)
    a.order = p.model == AMPS_GRAINGROWTH && p.mode == AMPS_END2END_MIX ? h->d_order : nullptr;
    a.nx = p.nx; a.ny = p.ny; a.ntx = h->ntx; a.nty = h->nty; a.nf = h->nf; a.bc = p.bc; a.stencil = p.stencil;
    a.px = h->px;
    a.n = h->ns;
    a.monitor_now = monitor_now ? 1 : 0;
    a.monitor_kind = p.monitor;
    a.samples = p.monitor_samples;
    a.mfield = p.monitor_field;
    a.mu_lap_fp64 = p.mu_lap_fp64;
    a.cadence = p.cadence;
    a.half_arith = p.half_arith;
    a.tma_stage = h->tma_stage ? 1 : 0;
    a.metric = h->d_metric;
    a.snap = h->d_snap;
    a.flags = h->d_flags;
    a.step_base = h->d_step_base;
    a.step_off = step_off;
    a.ph = make_phys(p);
    return a;
}

// Records a profiling event on the handle's stream; while the stream is
// being captured the record becomes a graph node, so the pair around a
// kernel brackets it on the device with no host gap in between.
static cudaError_t prof_record(amps_handle *h, cudaEvent_t e)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (h->stream) cudaStreamIsCapturing(h->stream, &cs);
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(e, h->stream, cudaEventRecordExternal)
                                               : cudaEventRecord(e, h->stream);
}

// Event pair of one profiled launch (from the stash when there is one) and
// the record of its first event.
static int prof_begin(amps_handle *h, amps_handle::Ev &ev)
{
    for (cudaEvent_t *e : {&ev.a, &ev.b}) {
        if (!h->ev_stash.empty()) {
            *e = h->ev_stash.back();
            h->ev_stash.pop_back();
        } else if (cudaEventCreate(e) != cudaSuccess) {
            FAIL(h, AMPS_ERR_CUDA, "event create");
        }
    }
    CK(h, prof_record(h, ev.a));
    return AMPS_OK;
}

static int launch_step(amps_handle *h, int step_off, bool monitor_now)
{
    const amps_params &p = h->p;
    StepArgs a = step_args(h, h->parity, h->transition, step_off, monitor_now);
    const bool ref = p.ref_order != 0;
    if (p.model == AMPS_GRAINGROWTH) {
        // one fused launch covers every tier (profiled per chunk by enqueue_chunk)
        // all-FP64 runs and steps use the staged FP64 kernel, every other the fused one
        const bool only64 = (h->used[TIER_FP64] && !h->used[TIER_FP32] && !h->used[TIER_HALF]) ||
                            (h->all_fp64 && !monitor_now);
        cudaError_t e = h->use_tma ? gg_launch_tma(ref, h->tm[h->parity], a, h->tma_grid, h->stream)
                                   : gg_launch(h->T, only64 ? TIER_FP64 : -1, ref, a, h->ntiles, h->stream,
                                               h->tma_stage ? &h->tm[h->parity] : nullptr);
        if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "step kernel launch: %s", cudaGetErrorString(e));
        ++h->launches;
        h->parity ^= 1;
        h->transition = false;
        return AMPS_OK;
    }
    if (h->d_mu) {
        // sintering in the reference's own mixed arithmetic: the chemical
        // potential pass, then the update pass, every tier in each (index 3)
        amps_handle::Ev ev{3, nullptr, nullptr, 1};
        if (h->profiling) {
            const int r = prof_begin(h, ev);
            if (r) return r;
        }
        cudaError_t e = sint_ref_launch(h->T, a, h->d_mu, h->ntiles, h->stream);
        if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "step kernel launch: %s", cudaGetErrorString(e));
        h->launches += 2;
        if (h->profiling) {
            CK(h, prof_record(h, ev.b));
            h->evs.push_back(ev);
        }
        h->parity ^= 1;
        h->transition = false;
        return AMPS_OK;
    }
    // half + FP32 in use: one launch covers both (profiled as index 3)
    const bool lo_fused = h->used[TIER_HALF] && h->used[TIER_FP32];
    for (int t = 2; t >= 0; --t) {
        if (!h->used[t] || (lo_fused && t == TIER_HALF)) continue;
        const bool fused = lo_fused && t == TIER_FP32;
        cudaStream_t st = h->stream;
        a.list = h->d_lists + t * h->ntiles;
        cudaError_t e;
        amps_handle::Ev ev{fused ? 3 : t, nullptr, nullptr, 1};
        if (h->profiling) {
            const int r = prof_begin(h, ev);
            if (r) return r;
        }
        // the FP64 launch (t = 2) came just before: run alongside it
        const bool after64 = h->used[TIER_FP64] && !h->profiling;
        if (fused) e = p.model == AMPS_KOBAYASHI ? kob_launch_lo(h->T, a, h->ntiles, st, after64)
                                                 : sint_launch_lo(h->T, p.mu_lap_fp64 != 0, a, h->ntiles, st, after64);
        else if (p.model == AMPS_KOBAYASHI) e = kob_launch(h->T, t, ref, a, h->ntiles, st, !h->profiling);
        else e = sint_launch(h->T, t, ref, p.mu_lap_fp64 != 0, a, h->ntiles, st, !h->profiling);
        if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "step kernel launch: %s", cudaGetErrorString(e));
        ++h->launches;
        if (h->profiling) {
            CK(h, prof_record(h, ev.b));
            h->evs.push_back(ev);
        }
    }
    h->parity ^= 1;
    h->transition = false;
    return AMPS_OK;
}

static ClassifyArgs classify_args(const amps_handle *h, int advance, int stat_steps)
{
    const amps_params &p = h->p;
    ClassifyArgs c{};
    c.metric = h->d_metric; c.tier_prev = h->d_tier_prev; c.tier_cur = h->d_tier_cur;
    c.lists = h->d_lists; c.counts = h->d_counts; c.ntx = h->ntx; c.nty = h->nty;
    c.thr_lo = p.thr_lo; c.thr_hi = p.thr_hi; c.high_tier = p.high_tier; c.use_mid = h->use_mid;
    c.stats = h->d_stats; c.log = h->d_log; c.log_n = h->d_log_n; c.max_log = p.max_log;
    c.step_base = h->d_step_base; c.advance = advance; c.stat_steps = stat_steps;
    c.order = h->d_order; c.bc = p.bc;
    if (h->sched_n) { c.sched = h->d_sched; c.sched_n = h->sched_n; c.sched_i = h->d_sched_i; }
    return c;
}

// Steps [k0, k0+n) as one multi-step launch (no tier change and no monitor
// among them).
static int launch_flow(amps_handle *h, int k0, int n)
{
    CK(h, cudaMemsetAsync(h->d_flow, 0, sizeof(int) * (h->ntiles + 1), h->stream));
    const StepArgs a0 = step_args(h, h->parity, false, k0, false);
    const StepArgs a1 = step_args(h, h->parity ^ 1, false, k0 + 1, false);
    FlowArgs fl;
    fl.done = h->d_flow;
    fl.queue = h->d_flow + h->ntiles;
    fl.nsteps = n;
    const cudaError_t e = gg_launch_flow(h->p.ref_order != 0, a0, a1, fl, h->stream);
    if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "multi-step kernel launch: %s", cudaGetErrorString(e));
    ++h->launches;
    if (n & 1) h->parity ^= 1;
    return AMPS_OK;
}

// Steps [k0, k0+cnt) of a period, then the period's bookkeeping.
static int enqueue_chunk(amps_handle *h, int k0, int cnt)
{
    const amps_params &p = h->p;
    const bool period_end = k0 + cnt == p.cadence;
    // grain growth: one event pair spans the chunk's back-to-back step
    // launches (a pair around each ~20 us launch would time its launch
    // latency too, which consecutive launches otherwise overlap)
    const bool span = h->profiling && p.model == AMPS_GRAINGROWTH;
    amps_handle::Ev ev{3, nullptr, nullptr, cnt};
    if (span) {
        const int r = prof_begin(h, ev);
        if (r) return r;
    }
    for (int s = 0; s < cnt;) {
        // a tier schedule stands in for the monitor: no epilogue
        const bool mon = h->mixed && period_end && s == cnt - 1 && h->sched_n == 0;
        if (h->use_flow && !h->transition && !h->all_fp64 && !mon) {
            // the run of steps up to the monitor step (or the chunk's end)
            const int run = (h->mixed && period_end && h->sched_n == 0) ? cnt - 1 - s : cnt - s;
            if (run >= 2) {
                int r = launch_flow(h, k0 + s, run);
                if (r) return r;
                s += run;
                continue;
            }
        }
        int r = launch_step(h, k0 + s, mon);
        if (r) return r;
        ++s;
    }
    if (span) {
        CK(h, prof_record(h, ev.b));
        h->evs.push_back(ev);
    }
    if (h->mixed && period_end) {
        CK(h, classify(classify_args(h, p.cadence, cnt), h->stream));
        ++h->launches;
        if (h->d_snap_keep && !h->sched_n) {
            CK(h, snap_ref_fixup(h->d_snap, h->d_snap_keep, h->d_tier_cur, h->ntiles, h->nmon, h->stream));
            ++h->launches;
        }
        h->transition = true;
        h->all_fp64 = false;
    } else {
        CK(h, advance_period(h->d_step_base, period_end ? p.cadence : 0, cnt, h->d_counts, h->d_stats, h->stream));
        ++h->launches;
    }
    return AMPS_OK;
}

extern "C" int amps_run(amps_handle *h, int nsteps)
{
    if (!h || nsteps < 0) return AMPS_ERR_INVALID;
    const int cad = h->p.cadence;
    while (nsteps > 0) {
        const int k0 = (int)(h->step % cad);
        const int cnt = nsteps < cad - k0 ? nsteps : cad - k0;
        if (h->graphs && h->profiling && k0 == 0 && cnt == cad && h->stream != nullptr) {
            // a profiled period runs as a one-off graph with its event records
            // as nodes (the host enqueues eager launches and event records
            // slower than the GPU runs them, and would time its own gaps)
            while (h->ev_stash.size() < (size_t)6 * cad) {
                cudaEvent_t e;
                CK(h, cudaEventCreate(&e));
                h->ev_stash.push_back(e);
            }
            cudaGraph_t gr;
            CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            int r = enqueue_chunk(h, 0, cad);
            cudaError_t e = cudaStreamEndCapture(h->stream, &gr);
            if (r) return r;
            if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
            cudaGraphExec_t ex;
            e = cudaGraphInstantiate(&ex, gr, 0);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
            e = cudaGraphLaunch(ex, h->stream);
            cudaGraphExecDestroy(ex);  // freed once the launch completes
            if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
        } else if (h->graphs && !h->profiling && k0 == 0 && cnt == cad) {
            const int key = h->parity | (h->transition ? 2 : 0) | (h->all_fp64 ? 4 : 0);
            auto it = h->graph.find(key);
            if (it == h->graph.end()) {
                const int par0 = h->parity;
                const bool tr0 = h->transition, all0 = h->all_fp64;
                const int64_t n0 = h->launches;
                // the default stream cannot be captured: capture on a private
                // stream (the period's launches go to h->stream meanwhile)
                // and replay the graph on the default stream below
                cudaStream_t user = h->stream;
                if (!user && !h->cap) CK(h, cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
                if (!user) h->stream = h->cap;
                cudaGraph_t gr = nullptr;
                cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
                int r = e == cudaSuccess ? enqueue_chunk(h, 0, cad) : AMPS_OK;
                if (e == cudaSuccess) e = cudaStreamEndCapture(h->stream, &gr);
                h->stream = user;
                if (r) {
                    if (gr) cudaGraphDestroy(gr);
                    return r;
                }
                if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
                cudaGraphExec_t ex;
                e = cudaGraphInstantiate(&ex, gr, 0);
                cudaGraphDestroy(gr);
                if (e != cudaSuccess) FAIL(h, AMPS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
                it = h->graph.emplace(key, ex).first;
                h->graph_launches[key] = h->launches - n0;
                h->parity = par0;  // capture advanced the host-side state; replay does it for real
                h->transition = tr0;
                h->all_fp64 = all0;
                h->launches = n0;
            }
            CK(h, cudaGraphLaunch(it->second, h->stream));
            h->launches += h->graph_launches[key];
            // mirror the period's effect on the host-side state
            if (cad & 1) h->parity ^= 1;
            h->transition = h->mixed;
            if (h->mixed) h->all_fp64 = false;
        } else {
            int r = enqueue_chunk(h, k0, cnt);
            if (r) return r;
        }
        h->step += cnt;
        nsteps -= cnt;
    }
    return AMPS_OK;
}

// ------------------------------------------------------------- diagnostics ----
extern "C" int amps_get_tile_tiers(amps_handle *h, uint8_t *out)
{
    if (!h || !out) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaMemcpy(out, h->d_tier_cur, h->ntiles, cudaMemcpyDeviceToHost));
    return AMPS_OK;
}

extern "C" int amps_get_tile_types(amps_handle *h, uint8_t *out)
{
    const int r = amps_get_tile_tiers(h, out);
    if (r) return r;
    const int high = h->p.high_tier;
    for (int t = 0; t < h->ntiles; ++t) out[t] = out[t] == TIER_HALF ? 1 : (out[t] == high ? 2 : 3);
    return AMPS_OK;
}

extern "C" int amps_get_tile_metric(amps_handle *h, double *out)
{
    if (!h || !out) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaMemcpy(out, h->d_metric, sizeof(double) * h->ntiles, cudaMemcpyDeviceToHost));
    return AMPS_OK;
}

// The tiers a map may hold: those with storage in this handle's mode.
static int check_maps(amps_handle *h, const uint8_t *maps, int n_maps, const char *what)
{
    for (int64_t i = 0; i < (int64_t)n_maps * h->ntiles; ++i)
        if (maps[i] > TIER_FP64 || !h->used[maps[i]])
            FAIL(h, AMPS_ERR_INVALID, "%s: map %d tile %d: tier %d is not one of this mode's tiers", what,
                 (int)(i / h->ntiles), (int)(i % h->ntiles), (int)maps[i]);
    return AMPS_OK;
}

extern "C" int amps_set_tier_schedule(amps_handle *h, const uint8_t *maps, int n_maps)
{
    if (!h || n_maps < 0 || (n_maps > 0 && !maps)) return AMPS_ERR_INVALID;
    if (!h->mixed) FAIL(h, AMPS_ERR_INVALID, "amps_set_tier_schedule: only adaptive runs classify");
    int r = check_maps(h, maps, n_maps, "amps_set_tier_schedule");
    if (r) return r;
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->d_sched) cudaFree(h->d_sched);
    h->d_sched = nullptr;
    h->sched_n = 0;
    if (!h->d_sched_i) CK(h, cudaMalloc(&h->d_sched_i, sizeof(int)));
    if (n_maps) {
        const size_t bytes = (size_t)n_maps * h->ntiles;
        CK(h, cudaMalloc(&h->d_sched, bytes));
        CK(h, cudaMemcpyAsync(h->d_sched, maps, bytes, cudaMemcpyHostToDevice, h->stream));
    }
    CK(h, cudaMemsetAsync(h->d_sched_i, 0, sizeof(int), h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->sched_n = n_maps;
    // the captured periods hold the old classification arguments and monitor steps
    for (auto &kv : h->graph) cudaGraphExecDestroy(kv.second);
    h->graph.clear();
    return AMPS_OK;
}

extern "C" int amps_set_tile_tiers(amps_handle *h, const uint8_t *tiers)
{
    if (!h || !tiers) return AMPS_ERR_INVALID;
    if (h->mixed) FAIL(h, AMPS_ERR_INVALID, "amps_set_tile_tiers: adaptive runs take their tiers from the monitor");
    int r = check_maps(h, tiers, 1, "amps_set_tile_tiers");
    if (r) return r;
    // the state at its current tiers -> FP64 stage -> stored at the new tiers
    Grid live = grid_view(h, h->parity, live_tiers(h));
    CK(h, gather_fields(live, h->d_stage, 0, 0, h->nf, h->stream));
    CK(h, cudaMemcpyAsync(h->d_tier_cur, tiers, h->ntiles, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->d_tier_prev, tiers, h->ntiles, cudaMemcpyHostToDevice, h->stream));
    CK(h, build_lists(h->d_tier_cur, h->ntiles, h->d_lists, h->d_counts, h->stream));
    h->transition = false;
    Grid g = grid_view(h, h->parity, h->d_tier_cur);
    CK(h, scatter_fields(g, h->d_stage, 0, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return AMPS_OK;
}

extern "C" int amps_measure_tiles(amps_handle *h, int kind, double *out)
{
    if (!h || (kind != AMPS_MONITOR_SPA && kind != AMPS_MONITOR_TEM) || (kind == AMPS_MONITOR_SPA && !out))
        return AMPS_ERR_INVALID;
    const amps_params &p = h->p;
    if (kind == AMPS_MONITOR_TEM && out && !h->msnap_valid)
        FAIL(h, AMPS_ERR_INVALID, "amps_measure_tiles: no temporal reference stored yet (call with out == NULL)");
    CK(h, cudaStreamSynchronize(h->stream));
    if (!h->d_mmetric) CK(h, cudaMalloc(&h->d_mmetric, sizeof(double) * h->ntiles));
    if (kind == AMPS_MONITOR_TEM && !h->d_msnap) {
        const size_t snap = p.monitor_samples ? (size_t)h->nmon * h->ns : (size_t)h->nmon * h->ntiles * 16;
        CK(h, cudaMalloc(&h->d_msnap, sizeof(double) * snap));
    }
    Grid g = grid_view(h, h->parity, live_tiers(h));
    if (kind == AMPS_MONITOR_SPA) {
        CK(h, monitor_state(g, 1, p.monitor_samples, p.monitor_field, h->d_mmetric, nullptr, 0, h->d_flags, h->stream));
    } else if (!out) {
        CK(h, monitor_state(g, 2, p.monitor_samples, p.monitor_field, nullptr, h->d_msnap, 1, h->d_flags, h->stream));
        h->msnap_valid = true;
    } else {
        CK(h, monitor_state(g, 2, p.monitor_samples, p.monitor_field, h->d_mmetric, h->d_msnap, 0, h->d_flags,
                            h->stream, 1));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    if (out) CK(h, cudaMemcpy(out, h->d_mmetric, sizeof(double) * h->ntiles, cudaMemcpyDeviceToHost));
    return AMPS_OK;
}

extern "C" int amps_get_decision_log(amps_handle *h, uint8_t *out, int max_entries, int *n_out)
{
    if (!h || !n_out) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    int n = 0;
    CK(h, cudaMemcpy(&n, h->d_log_n, sizeof(int), cudaMemcpyDeviceToHost));
    if (n > max_entries) n = max_entries;
    if (n > 0 && out) CK(h, cudaMemcpy(out, h->d_log, (size_t)n * h->ntiles, cudaMemcpyDeviceToHost));
    *n_out = n;
    return AMPS_OK;
}

extern "C" int amps_get_stats(amps_handle *h, amps_stats *out)
{
    if (!h || !out) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    unsigned long long s[8];
    int flag = 0;
    CK(h, cudaMemcpy(s, h->d_stats, sizeof s, cudaMemcpyDeviceToHost));
    CK(h, cudaMemcpy(&flag, h->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
    out->steps = h->step;
    for (int k = 0; k < 3; ++k) out->tile_steps[k] = (int64_t)s[k];
    out->monitor_evals = (int64_t)s[3];
    out->promotions = (int64_t)s[4];
    out->demotions = (int64_t)s[5];
    out->tiles = h->ntiles;
    out->numeric_error = flag & 1;
    out->kernel_launches = h->launches;
    return AMPS_OK;
}

extern "C" int amps_reduce(amps_handle *h, int field, int kind, double *out)
{
    if (!h || !out || field < 0 || field >= h->nf || kind < 0 || kind > 3) return AMPS_ERR_INVALID;
    Grid g = grid_view(h, h->parity, live_tiers(h));
    CK(h, reduce_field(g, field, kind, h->d_partials, h->d_out, h->stream));
    CK(h, cudaMemcpyAsync(h->h_pinned, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *out = h->h_pinned[0];
    return AMPS_OK;
}

extern "C" int amps_compare(amps_handle *h, int field, const double *other, int on_device, double *max_abs, double *rms)
{
    if (!h || !other || field < 0 || field >= h->nf) return AMPS_ERR_INVALID;
    const double *dev = other;
    if (!on_device) {
        CK(h, cudaMemcpyAsync(h->d_stage, other, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->stream));
        dev = h->d_stage;
    }
    Grid g = grid_view(h, h->parity, live_tiers(h));
    CK(h, compare_field(g, field, dev, h->d_partials, h->d_out, h->stream));
    CK(h, cudaMemcpyAsync(h->h_pinned, h->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (max_abs) *max_abs = h->h_pinned[0];
    if (rms) *rms = h->h_pinned[1];
    return AMPS_OK;
}

// ------------------------------------------------------------ diagnostics ----
namespace {
constexpr int kDiagAcc = 2 * 32 * 32 + 8;  // boundary counters for up to 32 labels
struct DiagScratch {
    int *lab, *parent, *box;
    double *field;
    unsigned long long *acc;
};
}  // namespace

static int diag_scratch(amps_handle *h, DiagScratch *d)
{
    const size_t ints = (size_t)2 * h->n * sizeof(int), dbl = (size_t)h->n * sizeof(double);
    const size_t off_f = (ints + 255) & ~(size_t)255, off_a = off_f + ((dbl + 255) & ~(size_t)255);
    const size_t total = off_a + kDiagAcc * sizeof(unsigned long long) + 256;
    if (!h->d_diag) CK(h, cudaMalloc(&h->d_diag, total));
    d->lab = (int *)h->d_diag;
    d->parent = d->lab + h->n;
    d->field = (double *)(h->d_diag + off_f);
    d->acc = (unsigned long long *)(h->d_diag + off_a);
    d->box = (int *)(d->acc + kDiagAcc);
    return AMPS_OK;
}

// all fields, FP64 row-major, into d_stage
static int diag_gather(amps_handle *h)
{
    Grid g = grid_view(h, h->parity, live_tiers(h));
    CK(h, gather_fields(g, h->d_stage, 0, 0, h->nf, h->stream));
    return AMPS_OK;
}

extern "C" int amps_compare_all(amps_handle *h, int field, const double *other, int on_device, double out[3])
{
    if (!h || !other || !out || field < 0 || field >= h->nf) return AMPS_ERR_INVALID;
    DiagScratch d;
    if (int r = diag_scratch(h, &d)) return r;
    if (int r = diag_gather(h)) return r;
    CK(h, cudaMemcpyAsync(d.field, other, sizeof(double) * h->n,
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    CK(h, diag_compare3(h->d_stage + (int64_t)field * h->n, d.field, h->n, h->d_partials, 512, h->d_out, h->stream));
    CK(h, cudaMemcpyAsync(h->h_pinned, h->d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 3; ++k) out[k] = h->h_pinned[k];
    return AMPS_OK;
}

extern "C" int amps_interface(amps_handle *h, int field, double level, double out[7])
{
    if (!h || !out || field < 0 || field >= h->nf) return AMPS_ERR_INVALID;
    DiagScratch d;
    if (int r = diag_scratch(h, &d)) return r;
    if (int r = diag_gather(h)) return r;
    const amps_params &p = h->p;
    CK(h, diag_interface(h->d_stage + (int64_t)field * h->n, p.nx, p.ny, p.bc, level, d.acc, d.box, h->stream));
    unsigned long long acc[3];
    int box[4];
    CK(h, cudaMemcpyAsync(acc, d.acc, sizeof acc, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(box, d.box, sizeof box, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    out[0] = (double)acc[0];
    out[1] = (double)acc[0] * p.dx * p.dy;
    out[2] = (double)acc[1] * p.dy + (double)acc[2] * p.dx;
    for (int k = 0; k < 4; ++k) out[3 + k] = acc[0] ? (double)box[k] : -1.0;
    return AMPS_OK;
}

// order parameters of the model: (first field, count, concentration field or -1)
static bool order_params(const amps_handle *h, int *e0, int *q, int *cfield)
{
    if (h->p.model == AMPS_GRAINGROWTH) {
        *e0 = 0; *q = h->nf; *cfield = -1;
        return true;
    }
    if (h->p.model == AMPS_SINTERING) {
        *e0 = 1; *q = h->nf - 1; *cfield = 0;
        return true;
    }
    return false;
}

extern "C" int amps_grains(amps_handle *h, double threshold, double level, int64_t out[2], double *mean_area)
{
    int e0, q, cf;
    if (!h || !out || !order_params(h, &e0, &q, &cf)) return AMPS_ERR_INVALID;
    DiagScratch d;
    if (int r = diag_scratch(h, &d)) return r;
    if (int r = diag_gather(h)) return r;
    const amps_params &p = h->p;
    const double *conc = cf >= 0 ? h->d_stage + (int64_t)cf * h->n : nullptr;
    CK(h, diag_grains(h->d_stage, e0, q, p.nx, p.ny, p.bc, threshold, conc, level, d.lab, d.parent, d.acc,
                      h->d_flags, h->stream));
    unsigned long long acc[2];
    int flag = 0;
    CK(h, cudaMemcpyAsync(acc, d.acc, sizeof acc, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(&flag, h->d_flags, sizeof flag, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (flag & 4) FAIL(h, AMPS_ERR_TIMEOUT, "grain labelling: a union-find walk exceeded the cell count");
    out[0] = (int64_t)acc[0];
    out[1] = (int64_t)acc[1];
    if (mean_area) *mean_area = acc[0] ? (double)acc[1] * p.dx * p.dy / (double)acc[0] : 0.0;
    return AMPS_OK;
}

extern "C" int amps_boundary_lengths(amps_handle *h, double level, double *lengths)
{
    int e0, q, cf;
    if (!h || !lengths || !order_params(h, &e0, &q, &cf) || q > 32) return AMPS_ERR_INVALID;
    DiagScratch d;
    if (int r = diag_scratch(h, &d)) return r;
    if (int r = diag_gather(h)) return r;
    const amps_params &p = h->p;
    const double *conc = cf >= 0 ? h->d_stage + (int64_t)cf * h->n : nullptr;
    CK(h, diag_boundaries(h->d_stage, e0, q, p.nx, p.ny, p.bc, conc, level, d.lab, d.acc, h->stream));
    std::vector<unsigned long long> acc((size_t)2 * q * q);
    CK(h, cudaMemcpyAsync(acc.data(), d.acc, acc.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int a = 0; a < q; ++a)
        for (int b = 0; b < q; ++b) {
            const int lo = a < b ? a : b, hi = a < b ? b : a;
            const size_t k = ((size_t)lo * q + hi) * 2;
            lengths[(size_t)a * q + b] = a == b ? 0.0 : (double)acc[k] * p.dy + (double)acc[k + 1] * p.dx;
        }
    return AMPS_OK;
}

extern "C" int amps_set_profiling(amps_handle *h, int enable)
{
    if (!h) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    for (auto &e : h->evs) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    h->evs.clear();
    for (int k = 0; k < 4; ++k) { h->prof_ms[k] = 0; h->prof_launches[k] = 0; }
    CK(h, cudaMemcpy(h->prof_stats0, h->d_stats, sizeof h->prof_stats0, cudaMemcpyDeviceToHost));
    h->profiling = enable != 0;
    return AMPS_OK;
}

extern "C" int amps_get_kernel_times(amps_handle *h, double *ms, int64_t *launches, int64_t *tile_steps)
{
    if (!h) return AMPS_ERR_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    for (auto &e : h->evs) {
        float t = 0.f;
        CK(h, cudaEventElapsedTime(&t, e.a, e.b));
        h->prof_ms[e.tier] += t;
        h->prof_launches[e.tier] += e.n;
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    h->evs.clear();
    unsigned long long s[3];
    CK(h, cudaMemcpy(s, h->d_stats, sizeof s, cudaMemcpyDeviceToHost));
    int64_t total = 0;
    for (int k = 0; k < 4; ++k) {
        if (ms) ms[k] = h->prof_ms[k];
        if (launches) launches[k] = h->prof_launches[k];
        if (k < 3) {
            const int64_t ts = (int64_t)(s[k] - h->prof_stats0[k]);
            total += ts;
            if (tile_steps) tile_steps[k] = ts;
        } else if (tile_steps) {
            tile_steps[3] = total;
        }
    }
    return AMPS_OK;
}

// -------------------------------------------------------------- ensembles ----
// Many grain-growth handles advanced in lockstep: every step is ONE
// persistent launch over the (member, tile) work items of all members, and
// the period-end classification of all members is one batched launch.  A
// whole cadence period is captured once per (parity, transition) pattern of
// the members and replayed.
struct amps_ensemble {
    std::vector<amps_handle *> m;
    int T = 0, cad = 0, maxnf = 0;
    bool ref = false, mixed = false;
    cudaStream_t stream = nullptr, capture = nullptr;
    // members launched together: same occupancy class, at most kEnsCap
    struct Group {
        std::vector<int> members;  // indices into m
        std::vector<int> first;    // first work item (CTA) of each member, + the total
        size_t smem = 0;
        cudaStream_t s = nullptr;  // its branch of a period graph
        cudaEvent_t done = nullptr;
        bool pair = false;         // non-monitor steps as split tiles (gg_launch_ens_pair)
        size_t smem_pair = 0;
    };
    std::vector<Group> groups;
    cudaEvent_t fork = nullptr;
    ClassifyArgs *d_cls = nullptr;      // whole periods: advance = stat_steps = cadence
    ClassifyArgs *d_cls_tmp = nullptr;  // partial periods (eager)
    CUtensorMap *d_tmaps = nullptr;     // members' FP32 tensor maps [member][box: all fields, split][parity]
    std::vector<uint8_t> map8;          // [member]: its split-tile maps were encoded
    bool graphs = true;
    std::map<std::vector<uint8_t>, cudaGraphExec_t> periods;
    std::unique_ptr<EnsLaunch> launch;  // host staging of one launch's parameters
    std::string err;
};

#define EFAIL(e, code, ...)                                        \
    do {                                                           \
        char _b[512];                                              \
        snprintf(_b, sizeof _b, __VA_ARGS__);                      \
        (e)->err = _b;                                             \
        return (code);                                             \
    } while (0)
#define ECK(e, call)                                                                              \
    do {                                                                                          \
        cudaError_t _e = (call);                                                                  \
        if (_e != cudaSuccess) EFAIL(e, AMPS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

static void ens_free(amps_ensemble *e)
{
    for (auto &kv : e->periods)
        if (kv.second) cudaGraphExecDestroy(kv.second);
    e->periods.clear();
    for (auto &g : e->groups) {
        if (g.s) cudaStreamDestroy(g.s);
        if (g.done) cudaEventDestroy(g.done);
    }
    e->groups.clear();
    if (e->fork) cudaEventDestroy(e->fork);
    cudaFree(e->d_cls);
    cudaFree(e->d_cls_tmp);
    cudaFree(e->d_tmaps);
    if (e->capture) cudaStreamDestroy(e->capture);
}

extern "C" int amps_ensemble_create(amps_handle *const *members, int count, amps_ensemble **out)
{
    if (!out) return AMPS_ERR_INVALID;
    *out = nullptr;
    if (!members || count < 1) return AMPS_ERR_INVALID;
    amps_handle *h0 = members[0];
    for (int i = 0; i < count; ++i)
        if (members[i] && (members[i]->p.half_arith != AMPS_HALF_FP32 || members[i]->d_snap_keep)) {
            g_create_err = "amps_ensemble_create: members with binary16 arithmetic or the reference's snapshot "
                           "rule run only through amps_run";
            return AMPS_ERR_UNSUPPORTED;
        }
    for (int i = 0; i < count; ++i) {
        amps_handle *h = members[i];
        if (!h || h->p.model != AMPS_GRAINGROWTH || h->T != h0->T || h->p.cadence != h0->p.cadence ||
            h->mixed != h0->mixed || (h->p.ref_order != 0) != (h0->p.ref_order != 0) ||
            h->step % h->p.cadence != h0->step % h0->p.cadence || h->sched_n)
            return AMPS_ERR_INVALID;
        for (int j = 0; j < i; ++j)
            if (members[j] == h) return AMPS_ERR_INVALID;
    }
    amps_ensemble *e = new (std::nothrow) amps_ensemble;
    if (!e) return AMPS_ERR_ALLOC;
    e->launch.reset(new (std::nothrow) EnsLaunch);
    if (!e->launch) {
        delete e;
        return AMPS_ERR_ALLOC;
    }
    e->m.assign(members, members + count);
    e->T = h0->T;
    e->cad = h0->p.cadence;
    e->mixed = h0->mixed;
    e->ref = h0->p.ref_order != 0;
    for (int i = 0; i < count; ++i) e->maxnf = std::max(e->maxnf, members[i]->nf);
    // groups: members with more fields first; a group closes where the
    // occupancy its largest member's staging allows would change, or at kEnsCap
    std::vector<int> order(count);
    for (int i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return members[a]->nf > members[b]->nf; });
    std::vector<ClassifyArgs> cls(count);
    for (int i = 0; i < count; ++i) cls[i] = classify_args(members[i], e->cad, e->cad);
    cudaError_t ce = gg_prepare_ens(e->T, e->ref, gg_ens_smem_bytes(e->T, e->maxnf));
    std::map<int, int> occ;  // field count -> CTAs an SM
    for (int i = 0; ce == cudaSuccess && i < count; ++i) {
        const int nf = members[order[i]]->nf;
        if (!occ.count(nf)) {
            int bps = 0;
            ce = gg_ens_occupancy(e->T, e->ref, gg_ens_smem_bytes(e->T, nf), &bps);
            if (ce == cudaSuccess && bps < 1) ce = cudaErrorInvalidConfiguration;
            occ[nf] = bps;
        }
    }
    for (int i = 0; ce == cudaSuccess && i < count; ++i) {
        amps_handle *h = members[order[i]];
        if (e->groups.empty() || (int)e->groups.back().members.size() == kEnsCap ||
            occ[e->m[e->groups.back().members[0]]->nf] != occ[h->nf]) {
            e->groups.emplace_back();
            e->groups.back().smem = gg_ens_smem_bytes(e->T, h->nf);
            e->groups.back().first.push_back(0);
        }
        auto &g = e->groups.back();
        g.members.push_back(order[i]);
        g.first.push_back(g.first.back() + h->ntiles);
    }
    // split tiles (opt-in, AMPS_ENS_PAIR=1): a group whose members all have
    // 2 * kPairFields fields runs its non-monitor steps as two-CTA clusters,
    // half the fields each (32^2 tiles, the library's order).  Measured slower
    // than whole tiles on the 64-member workload (43.9 against 53.7 Gcell/s:
    // the two cluster barriers a tile cost more than the doubled occupancy
    // gains), so whole tiles stay the default.
    const char *pv = getenv("AMPS_ENS_PAIR");
    bool any_pair = false;
    for (auto &g : e->groups) {
        bool all = e->T == 32 && !e->ref && pv && pv[0] == '1';
        for (int mi : g.members) all = all && e->m[mi]->nf == 2 * kPairFields;
        g.pair = all;
        g.smem_pair = all ? gg_ens_smem_bytes(32, kPairFields) : 0;
        any_pair |= all;
    }
    if (ce == cudaSuccess && any_pair) ce = gg_prepare_ens_pair(gg_ens_smem_bytes(32, kPairFields));
    for (auto &g : e->groups) {
        if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&g.s, cudaStreamNonBlocking);
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming);
    }
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->d_cls, sizeof(ClassifyArgs) * count);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->d_cls_tmp, sizeof(ClassifyArgs) * count);
    if (ce == cudaSuccess) ce = cudaMemcpy(e->d_cls, cls.data(), sizeof(ClassifyArgs) * count, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->capture, cudaStreamNonBlocking);
    if (ce == cudaSuccess && e->T == 32) {
        // the members' tensor maps, in global memory where the ensemble kernel reads them
        e->map8.assign(count, 0);
        std::vector<CUtensorMap> maps((size_t)4 * count);
        memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
        for (int i = 0; i < count; ++i) {
            amps_handle *h = members[i];
            if (!h->tma_stage) continue;
            maps[4 * i] = h->tm[0];
            maps[4 * i + 1] = h->tm[1];
            if (h->nf == 2 * kPairFields)
                e->map8[i] = encode_field_map(&maps[4 * i + 2], h->store[TIER_FP32][0], h->px, h->nty * h->T, h->nf,
                                              kPairFields) &&
                             encode_field_map(&maps[4 * i + 3], h->store[TIER_FP32][1], h->px, h->nty * h->T, h->nf,
                                              kPairFields);
        }
        ce = cudaMalloc(&e->d_tmaps, sizeof(CUtensorMap) * maps.size());
        if (ce == cudaSuccess)
            ce = cudaMemcpy(e->d_tmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        g_create_err = std::string("amps_ensemble_create: ") + cudaGetErrorString(ce);
        cudaGetLastError();
        ens_free(e);
        delete e;
        return ce == cudaErrorMemoryAllocation ? AMPS_ERR_ALLOC : AMPS_ERR_CUDA;
    }
    *out = e;
    return AMPS_OK;
}

extern "C" int amps_ensemble_destroy(amps_ensemble *e)
{
    if (!e) return AMPS_ERR_INVALID;
    cudaStreamSynchronize(e->stream);
    ens_free(e);
    delete e;
    return AMPS_OK;
}

extern "C" int amps_ensemble_set_stream(amps_ensemble *e, void *stream)
{
    if (!e) return AMPS_ERR_INVALID;
    e->stream = (cudaStream_t)stream;
    return AMPS_OK;
}

extern "C" int amps_ensemble_set_graphs(amps_ensemble *e, int enable)
{
    if (!e) return AMPS_ERR_INVALID;
    e->graphs = enable != 0;
    return AMPS_OK;
}

extern "C" const char *amps_ensemble_last_error(const amps_ensemble *e)
{
    return e ? e->err.c_str() : g_create_err.c_str();
}

// Step arguments of steps [k0, k0+cnt) of a period for every member, from the
// members' current host-side parity/transition (table[s * M + i]).
static std::vector<StepArgs> ens_tables(const amps_ensemble *e, int k0, int cnt)
{
    const int M = (int)e->m.size();
    const bool period_end = k0 + cnt == e->cad;
    std::vector<StepArgs> t((size_t)cnt * M);
    for (int i = 0; i < M; ++i) {
        const amps_handle *h = e->m[i];
        int par = h->parity;
        bool tr = h->transition;
        for (int s = 0; s < cnt; ++s) {
            const bool mon = e->mixed && period_end && s == cnt - 1;
            t[(size_t)s * M + i] = step_args(h, par, tr, k0 + s, mon);
            if (e->d_tmaps && h->tma_stage) {
                t[(size_t)s * M + i].tmap = e->d_tmaps + 4 * i + par;
                // split-tile boxes where they were encoded (else per-thread copies)
                if (e->map8[i]) t[(size_t)s * M + i].tmap8 = e->d_tmaps + 4 * i + 2 + par;
            }
            par ^= 1;
            tr = false;
        }
    }
    return t;
}

// Step k of group g (its members' arguments by value in the launch).
static int ens_launch(amps_ensemble *e, const amps_ensemble::Group &g, const std::vector<StepArgs> &tab, int k,
                      bool mon, cudaStream_t s)
{
    const int M = (int)e->m.size();
    EnsLaunch &L = *e->launch;
    L.count = (int)g.members.size();
    for (int j = 0; j < L.count; ++j) {
        L.first[j] = g.first[j];
        L.m[j] = tab[(size_t)k * M + g.members[j]];
    }
    L.first[L.count] = g.first[L.count];
    if (g.pair && !mon) ECK(e, gg_launch_ens_pair(L, g.smem_pair, s));
    else ECK(e, gg_launch_ens(e->T, e->ref, mon, L, g.smem, s));
    return AMPS_OK;
}

// cnt steps of every group, then the period-end classification (or the tier
// maps' advance).  branches: each group's steps on its own stream, forked
// from and joined back into s (a period graph's parallel branches).
static int ens_enqueue(amps_ensemble *e, const std::vector<StepArgs> &tab, const ClassifyArgs *cls, int cnt,
                       bool period_end, cudaStream_t s, bool branches)
{
    const int M = (int)e->m.size();
    if (branches) ECK(e, cudaEventRecord(e->fork, s));
    for (auto &g : e->groups) {
        cudaStream_t gs = branches ? g.s : s;
        if (branches) ECK(e, cudaStreamWaitEvent(gs, e->fork, 0));
        for (int k = 0; k < cnt; ++k) {
            const bool mon = e->mixed && period_end && k == cnt - 1;  // as in ens_tables
            if (int r = ens_launch(e, g, tab, k, mon, gs)) return r;
        }
        if (branches) {
            ECK(e, cudaEventRecord(g.done, gs));
            ECK(e, cudaStreamWaitEvent(s, g.done, 0));
        }
    }
    if (e->mixed && period_end) ECK(e, classify_batch(cls, M, s));
    else ECK(e, advance_batch(cls, M, s));
    return AMPS_OK;
}

static void ens_advance_host(amps_ensemble *e, int cnt, bool period_end)
{
    for (amps_handle *h : e->m) {
        if (cnt & 1) h->parity ^= 1;
        if (cnt > 0) h->transition = e->mixed && period_end;
        if (e->mixed && period_end) h->all_fp64 = false;
        h->step += cnt;
    }
}

extern "C" int amps_ensemble_run(amps_ensemble *e, int nsteps)
{
    if (!e || nsteps < 0) return AMPS_ERR_INVALID;
    const int M = (int)e->m.size();
    for (amps_handle *h : e->m) {
        if (h->step % e->cad != e->m[0]->step % e->cad)
            EFAIL(e, AMPS_ERR_INVALID, "ensemble members are at different phases of the monitor cadence");
        ECK(e, cudaStreamSynchronize(h->stream));  // members' own queued work first
    }
    while (nsteps > 0) {
        const int k0 = (int)(e->m[0]->step % e->cad);
        const int cnt = nsteps < e->cad - k0 ? nsteps : e->cad - k0;
        const bool period_end = k0 + cnt == e->cad;
        if (e->graphs && k0 == 0 && cnt == e->cad) {
            std::vector<uint8_t> key(M);
            for (int i = 0; i < M; ++i) key[i] = (uint8_t)(e->m[i]->parity | (e->m[i]->transition ? 2 : 0));
            auto it = e->periods.find(key);
            if (it == e->periods.end()) {
                const std::vector<StepArgs> tab = ens_tables(e, 0, cnt);
                it = e->periods.emplace(key, nullptr).first;
                cudaGraph_t gr = nullptr;
                ECK(e, cudaStreamBeginCapture(e->capture, cudaStreamCaptureModeThreadLocal));
                const int r = ens_enqueue(e, tab, e->d_cls, cnt, true, e->capture, true);
                const cudaError_t ce = cudaStreamEndCapture(e->capture, &gr);
                if (r) {
                    if (gr) cudaGraphDestroy(gr);
                    return r;
                }
                if (ce != cudaSuccess) EFAIL(e, AMPS_ERR_CUDA, "ensemble graph capture: %s", cudaGetErrorString(ce));
                const cudaError_t ci = cudaGraphInstantiate(&it->second, gr, 0);
                cudaGraphDestroy(gr);
                if (ci != cudaSuccess) {
                    it->second = nullptr;
                    e->periods.erase(it);
                    EFAIL(e, AMPS_ERR_CUDA, "ensemble graph instantiate: %s", cudaGetErrorString(ci));
                }
            }
            ECK(e, cudaGraphLaunch(it->second, e->stream));
        } else {
            // partial period, eager: the step arguments travel in the launches;
            // the classification's arguments go to their scratch slots once free
            const std::vector<StepArgs> tab = ens_tables(e, k0, cnt);
            std::vector<ClassifyArgs> cls(M);
            for (int i = 0; i < M; ++i) cls[i] = classify_args(e->m[i], period_end ? e->cad : 0, cnt);
            ECK(e, cudaStreamSynchronize(e->stream));
            ECK(e, cudaMemcpy(e->d_cls_tmp, cls.data(), sizeof(ClassifyArgs) * M, cudaMemcpyHostToDevice));
            if (int r = ens_enqueue(e, tab, e->d_cls_tmp, cnt, period_end, e->stream, false)) return r;
        }
        ens_advance_host(e, cnt, period_end);
        nsteps -= cnt;
    }
    return AMPS_OK;
}

extern "C" int amps_ensemble_synchronize(amps_ensemble *e)
{
    if (!e) return AMPS_ERR_INVALID;
    ECK(e, cudaStreamSynchronize(e->stream));
    for (size_t i = 0; i < e->m.size(); ++i) {
        int flag = 0;
        ECK(e, cudaMemcpy(&flag, e->m[i]->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
        if (flag & 1) EFAIL(e, AMPS_ERR_NUMERIC, "member %d: NaN or Inf detected by the monitor", (int)i);
        if (flag & 2) EFAIL(e, AMPS_ERR_TIMEOUT, "member %d: a bounded device wait gave up", (int)i);
    }
    return AMPS_OK;
}
