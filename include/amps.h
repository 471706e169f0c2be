/*
 * amps.h -- C ABI of the GB300-native adaptive mixed-precision phase-field
 * stencil library (libamps.so).
 *
 * What it replaces.  The reference drives its hot path from per-app `main`
 * programs that launch `__global__` kernels on caller-owned managed arrays
 * (snowflake/purehigh.cu:3-66, snowflake/purelow.cu:3-82,
 * snowflake/end2end_mix.cu:3-147, graingrowth/{purehigh,purelow,end2end_mix}.cu,
 * sintering/main.cu:5-635), with the kernel interface in
 * {snowflake,graingrowth,sintering}/function.h and tools.h and every size and
 * constant fixed at compile time (snowflake/paras/total.h:18-47).  This header
 * exposes the same path -- initial state, the purehigh / purelow /
 * end2end_mix (+ GRAM1/GRAM2) time loops, the per-tile precision monitor and
 * tier conversion, and the field read-back used for the CSV dump -- as
 * handle-based calls with runtime parameters.  Each entry point cites the
 * reference code it stands in for.
 *
 * Conventions.  Every call returns an int status (AMPS_OK == 0) and never
 * exits the process (the reference's CHECK_ERROR exits, snowflake/paras/
 * total.h:48-56).  amps_last_error() gives the message of the last failure on
 * a handle.  Work is queued on one CUDA stream per handle (caller-suppliable);
 * a handle is not re-entrant, distinct handles are independent.
 *
 * Fields.  Kobayashi: 0 = phi, 1 = T.  Grain growth: 0..Q-1 = eta_i.
 * Sintering: 0 = c, 1..N = eta_i.  Field data crosses the ABI as row-major
 * [ny][nx] arrays of double (dtype AMPS_F64) or float (AMPS_F32), on the host
 * or on the device.
 */
#ifndef AMPS_H
#define AMPS_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMPS_ABI_VERSION 2

#if defined(__GNUC__)
#define AMPS_API __attribute__((visibility("default")))
#else
#define AMPS_API
#endif

/* status codes */
enum {
    AMPS_OK = 0,
    AMPS_ERR_INVALID = 1,     /* bad argument or parameter combination */
    AMPS_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    AMPS_ERR_ALLOC = 3,       /* device or host allocation failed */
    AMPS_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
    AMPS_ERR_NUMERIC = 5,     /* NaN or Inf seen by the monitor */
    AMPS_ERR_UNSUPPORTED = 6  /* valid request the library cannot serve */
};

/* models: the reference's three apps */
enum { AMPS_KOBAYASHI = 0, AMPS_GRAINGROWTH = 1, AMPS_SINTERING = 2 };

/* run modes: snowflake/purehigh.cu, snowflake/purelow.cu,
 * snowflake/end2end_mix.cu (AMSTENCIL), GRAM1/GRAM2 static-ratio baselines
 * (snowflake/function.h:72-79) */
enum { AMPS_PUREHIGH = 0, AMPS_PURELOW = 1, AMPS_END2END_MIX = 2, AMPS_GRAM1 = 3, AMPS_GRAM2 = 4 };

/* Largest tile count of one grid: the classification ranks each tier's
 * tiles in a 21-bit field of a packed 64-bit counter.  amps_check_params
 * rejects grids with more tiles (e.g. 16x16 tiles beyond about 23000^2). */
#define AMPS_MAX_TILES 0x1FFFFF

/* storage / arithmetic tiers of a tile */
enum { AMPS_TIER_HALF = 0, AMPS_TIER_FP32 = 1, AMPS_TIER_FP64 = 2 };

/* boundary conditions */
enum { AMPS_BC_PERIODIC = 0, AMPS_BC_NOFLUX = 1 };

/* monitors: Monitor1 = spatial range (snowflake/tools.h:177-193),
 * Monitor2 = temporal change over one cadence (snowflake/tools.h:194-211),
 * RATE = the change of the cadence's last step times the cadence (an
 * estimate of Monitor2 that needs no snapshot; no reference counterpart) */
enum { AMPS_MONITOR_SPA = 1, AMPS_MONITOR_TEM = 2, AMPS_MONITOR_RATE = 3 };

/* arithmetic of half tiles (amps_params.half_arith; grain growth, sintering) */
enum {
    AMPS_HALF_FP32 = 0,  /* binary16 storage, FP32 arithmetic (the default) */
    AMPS_HALF_REF = 1,   /* binary16 arithmetic, every +, -, *, / rounded in the reference's expression
                            order: grain growth on adjacent-column pairs (graingrowth/function.h:163-166),
                            sintering per cell with the chemical potential at each cell's owner tier
                            (sintering/function.h:245-249,401-411,556-565; FP64 high tier, one
                            threshold): the parity path of the reference's AMSTENCIL mixed mode */
    AMPS_HALF_HFMA2 = 2, /* binary16 pairs with fused multiply-adds (HFMA2) */
    AMPS_HALF_SR = 3     /* FP32 arithmetic, binary16 storage by stochastic rounding (unbiased; seeded by
                            amps_params.seed): a change below half an ulp accumulates instead of rounding away
                            (Kobayashi) */
};

/* dtypes crossing the ABI */
enum { AMPS_F64 = 0, AMPS_F32 = 1 };

/* initial states */
enum {
    AMPS_INIT_REFERENCE = 0, /* snowflake/tools.h:24-33 disc; graingrowth/tools.h:24-38 circle;
                                sintering/main.cu:45-59 two touching discs */
    AMPS_INIT_SEEDED = 1     /* seeded synthetic states: Kobayashi disc at the centre;
                                grain growth i.i.d. uniform noise; sintering N discs placed by
                                seeded rejection sampling */
};

/* reductions for amps_reduce */
enum { AMPS_REDUCE_SUM = 0, AMPS_REDUCE_MIN = 1, AMPS_REDUCE_MAX = 2, AMPS_REDUCE_SUMSQ = 3 };

typedef struct amps_params {
    int model;            /* AMPS_KOBAYASHI / AMPS_GRAINGROWTH / AMPS_SINTERING */
    int mode;             /* AMPS_PUREHIGH ... AMPS_GRAM2 */
    int nx, ny;           /* grid; multiples of tile */
    int nfields;          /* grain growth: Q order parameters; sintering: N particles */
    int bc;               /* AMPS_BC_* */
    int tile;             /* tile side: 16 (the reference's unit) or 32 */
    int high_tier;        /* the reference's `highprecision`: AMPS_TIER_FP64 or AMPS_TIER_FP32 */
    int monitor;          /* AMPS_MONITOR_SPA, AMPS_MONITOR_TEM or AMPS_MONITOR_RATE */
    int monitor_samples;  /* 0: the reference's 4x4 sample lattice; 1: every cell of the tile */
    int monitor_field;    /* monitored field index; -1 = every field (max over fields) */
    int cadence;          /* steps between monitor evaluations (reference: 10) */
    int stencil;          /* grain growth: 0 = reference 8-neighbour Laplacian, 1 = 5-point */
    int ref_order;        /* 1: FP64 tiles keep the reference's expression order and rounding
                             (no fused multiply-add) -- the parity path */
    int mu_lap_fp64;      /* sintering: chemical-potential Laplacian in FP64 on every tier */
    int max_log;          /* tier maps kept in the decision log (0 = none) */
    double thr_lo;        /* metric >= thr_lo -> FP32 tier (three-tier mode) */
    double thr_hi;        /* metric >= thr_hi -> high tier; thr_lo == thr_hi: reference two tiers */
    double gram_ratio;    /* GRAM1/GRAM2 fraction of half tiles */
    double dx, dy, dt;
    /* Kobayashi (snowflake/paras/para*.h) */
    double tau, epsb, kappa, delta, aniso, alpha, gama, teq, theta0, pi, noise;
    /* grain growth (graingrowth/paras/para*.h); gamma: cross-term coefficient */
    double mobil, grcoef, gamma;
    /* sintering (sintering/paras/para*.h); A, B: bulk free-energy coefficients */
    double coefm, coefk, coefl, dvol, dvap, dsur, dgrb, A, B;
    /* initial-state geometry: Kobayashi disc radius^2 and centre offset;
     * grain-growth circle radius; sintering particle radii range */
    double init_r2, init_r, rmin, rmax, init_amp;
    int init_offset;
    uint64_t seed;
    int half_arith;       /* AMPS_HALF_FP32 / AMPS_HALF_REF (grain growth, sintering) / AMPS_HALF_HFMA2
                             (grain growth) / AMPS_HALF_SR (Kobayashi) */
    int ref_snapshot;     /* 1: the temporal monitor's lattice snapshot as the reference keeps it: a tile
                             computed at half refreshes only the first half of its columns
                             (graingrowth/function.h:38-39,68-73, snowflake/function.h:69-70,106-113,
                             whose low tiles return from the second column block before the
                             snapshot); sintering snapshots every column (sintering/function.h:199-206),
                             so there the flag changes nothing */
} amps_params;

typedef struct amps_stats {
    int64_t steps;                 /* steps advanced */
    int64_t tile_steps[3];         /* tile-steps computed per tier (half, fp32, fp64) */
    int64_t monitor_evals;         /* monitor evaluations (classifications) */
    int64_t promotions, demotions; /* tier changes over all classifications */
    int32_t tiles;                 /* tiles in the grid */
    int32_t numeric_error;         /* 1 if the monitor saw NaN or Inf */
    int64_t kernel_launches;       /* kernels amps_run has launched (steps, classifications; graph
                                      replays count the kernels of the graph) */
} amps_stats;

typedef struct amps_handle amps_handle;

/* ---- versions and messages ---------------------------------------------- */
AMPS_API int amps_abi_version(void);
AMPS_API const char *amps_status_string(int status);
/* Message of the last failure on h (or of the last failed amps_create when h is NULL). */
AMPS_API const char *amps_last_error(const amps_handle *h);

/* ---- parameters --------------------------------------------------------- */
/* Fill *p with a preset.  preset 1..5: the reference's parameter files
 * (snowflake/paras/para1-5.h, graingrowth/paras/para1-5.h,
 * sintering/paras/para1-5.h) at the reference's 512x512, 16x16 tiles,
 * periodic boundaries, threshold 0.99 and Monitor2, i.e. the shipped
 * header state (snowflake/paras/total.h:18-28).  preset 0: the seeded
 * large-grid workloads (Kobayashi 512^2 zero-flux with noise; grain growth
 * 1024^2 Q=8 Fan-Chen gamma=1.5; sintering 1024^2 with 16 particles). */
AMPS_API int amps_preset(int model, int preset, amps_params *p);
/* Validate a parameter set without allocating anything. */
AMPS_API int amps_check_params(const amps_params *p, char *msg, size_t msg_len);
/* Number of fields of a parameter set (2, Q or N+1). */
AMPS_API int amps_num_fields(const amps_params *p);

/* ---- handle lifetime ------------------------------------------------------ */
/* Replaces the cudaMallocManaged block at the top of each driver
 * (snowflake/end2end_mix.cu:4-40, graingrowth/end2end_mix.cu:4-31,
 * sintering/main.cu:6-44).  Device memory is owned by the handle. */
AMPS_API int amps_create(const amps_params *p, amps_handle **out);
AMPS_API int amps_destroy(amps_handle *h);
/* Queue work on a caller stream (cudaStream_t passed as void*); NULL restores
 * the handle's own stream. */
AMPS_API int amps_set_stream(amps_handle *h, void *stream);
AMPS_API int amps_synchronize(amps_handle *h);

/* ---- state ------------------------------------------------------------------ */
/* Initial state (kind AMPS_INIT_*).  Replaces dataprepare_high/half/half2
 * (snowflake/tools.h:24-58, graingrowth/tools.h:24-82), the sintering host
 * init (sintering/main.cu:45-59), the warm start of the temporal monitor
 * (snowflake/end2end_mix.cu:44-46) and highdata_to_low / dataprepare
 * (snowflake/tools.h:133-146, sintering/tools.h:80-92). */
AMPS_API int amps_init(amps_handle *h, int kind);
/* Host-only: write the initial state of (p, kind) into fields[f] (row-major
 * double [ny][nx] each).  Needs no GPU. */
AMPS_API int amps_init_host(const amps_params *p, int kind, double *const *fields);
/* Set / get one field.  on_device: 0 = host pointer, 1 = device pointer.
 * amps_get_field replaces data_sychro_aftercomputation +
 * purelow2high_aftercomputing (snowflake/tools.h:108-174). */
AMPS_API int amps_set_field(amps_handle *h, int field, const void *src, int dtype, int on_device);
AMPS_API int amps_get_field(amps_handle *h, int field, void *dst, int dtype, int on_device);
/* All fields at once, contiguous [nfields][ny][nx]. */
AMPS_API int amps_set_fields(amps_handle *h, const void *src, int dtype, int on_device);
AMPS_API int amps_get_fields(amps_handle *h, void *dst, int dtype, int on_device);

/* ---- time loop ------------------------------------------------------------- */
/* Advance nsteps explicit steps (asynchronous on the handle's stream).
 * Replaces the per-step launch sequences of the drivers
 * (snowflake/purehigh.cu:23-34, snowflake/end2end_mix.cu:80-105,
 * graingrowth/end2end_mix.cu:71-98, sintering/main.cu:126-207): fused update
 * kernels, one per tier in use, with the monitor (get_max_diff1/2) fused into
 * the epilogue of every cadence-th step, then get_type, and the tier
 * conversion done in-register by the next step.  Whole cadence periods are
 * replayed from a CUDA graph, on the handle's stream (a handle on the
 * default stream captures its graphs on a private stream and replays them
 * on the default stream). */
AMPS_API int amps_run(amps_handle *h, int nsteps);
/* Enable (1) / disable (0) CUDA-graph replay of whole periods (default 1). */
AMPS_API int amps_set_graphs(amps_handle *h, int enable);
/* Kernel timing: while enabled, amps_run brackets update-kernel launches with
 * CUDA events on the stream they are launched on -- every launch of the
 * Kobayashi and sintering kernels; for grain growth one pair around each
 * run of consecutive step launches (ms / launches is then the average launch
 * duration as the launches run back to back).  With a stream set and graphs
 * on, each whole period is captured, events included, into a one-off graph,
 * so no host-side gap falls inside a pair.
 * amps_get_kernel_times fills arrays of 4: ms and launches of the per-tier
 * update kernels (index 0 half, 1 fp32, 2 fp64) and of the fused all-tier
 * update kernel (index 3); tile_steps[0..2] are the tile-steps computed per
 * tier since profiling was enabled (tile_steps[3] their sum). */
AMPS_API int amps_set_profiling(amps_handle *h, int enable);
AMPS_API int amps_get_kernel_times(amps_handle *h, double *ms, int64_t *launches, int64_t *tile_steps);

/* ---- monitor results and diagnostics ---------------------------------------- */
/* Current tier of every tile, row-major [nty][ntx] (AMPS_TIER_*).  The
 * reference keeps this as type_curr (1 = half2, 2 = high). */
AMPS_API int amps_get_tile_tiers(amps_handle *h, uint8_t *out);
/* The same map in the reference's type_curr encoding (get_type,
 * snowflake/tools.h:212-230): 1 = half2 tile, 2 = high-precision tile;
 * the FP32 tiles of a three-tier run, which have no reference counterpart,
 * are 3. */
AMPS_API int amps_get_tile_types(amps_handle *h, uint8_t *out);
/* Decision log: the tier map after each classification, oldest first,
 * up to max_entries maps of ntiles bytes.  *n_out = maps written. */
AMPS_API int amps_get_decision_log(amps_handle *h, uint8_t *out, int max_entries, int *n_out);
/* Last monitor metric per tile (double [nty][ntx]). */
AMPS_API int amps_get_tile_metric(amps_handle *h, double *out);
AMPS_API int amps_get_stats(amps_handle *h, amps_stats *out);

/* ---- tier control for the cost and selection experiments ------------------- */
/* Adaptive runs (mode END2END_MIX) only: the k-th classification from now on
 * takes its tier map from maps[min(k, n_maps - 1)] (n_maps maps of ntiles
 * bytes, e.g. a decision log) instead of the monitor, and no step carries the
 * monitor epilogue.  Replaying a monitored run's decision log therefore runs
 * the same tiles at the same tiers, with the same results, minus the
 * monitor: the compute-only time of the reference's monitor-cost harness
 * (snowflake/monitor_independent_withoutmonitor.cu:89-126, which times the
 * update kernels alone against monitor_independent_withmonitor.cu:71-104).
 * Every amps_init / amps_set_field(s) restarts at maps[0] (the initial
 * classification).  n_maps = 0 restores the monitor.  Ensembles reject
 * members with a schedule. */
AMPS_API int amps_set_tier_schedule(amps_handle *h, const uint8_t *maps, int n_maps);
/* Static modes (PUREHIGH, PURELOW, GRAM1, GRAM2): replace the tier map with
 * tiers[ntiles] and store the current state at the new tiers (the host-side
 * type_new of snowflake/motivation_mix.cu:87-109, then the mixed steps at
 * :110-115).  Each tier must be one this mode stores (GRAM: half and the
 * high tier). */
AMPS_API int amps_set_tile_tiers(amps_handle *h, const uint8_t *tiers);
/* The monitor metric of the current state, on demand, without touching the
 * tiers (get_max_diff1 / get_max_diff2 of snowflake/motivation_mix.cu:77-82),
 * on the params' monitor field and sample lattice.  kind AMPS_MONITOR_SPA:
 * out[ntiles] = each tile's range.  kind AMPS_MONITOR_TEM: out == NULL stores
 * the current samples as the temporal reference (motivation_monitor2_datasychr,
 * :64-67); out != NULL writes max |current - reference| per tile. */
AMPS_API int amps_measure_tiles(amps_handle *h, int kind, double *out);
/* FP64 reduction of one field over the grid (deterministic order).  SUM of c
 * is the sintering conserved mass. */
AMPS_API int amps_reduce(amps_handle *h, int field, int kind, double *out);
/* Max-abs and RMS difference of one field against a row-major double array
 * (host or device), computed in FP64 on the device. */
AMPS_API int amps_compare(amps_handle *h, int field, const double *other, int on_device, double *max_abs,
                 double *rms);

/* ---- microstructure diagnostics (no reference counterpart) ---------------
 * All on the device in FP64 over the current state, deterministic.
 * amps_compare_all: out = {max |f - other|, RMS, mean |f - other|} (the mean
 *   absolute difference is the reference's error metric,
 *   graingrowth/end2enderror.py:34).
 * amps_interface: the level set {f >= level}: out = {cells, area (cells*dx*dy),
 *   perimeter (4-neighbour edges crossing the level: x-edges*dy + y-edges*dx,
 *   exact for axis-aligned fronts, up to sqrt 2 long on diagonal ones),
 *   xmin, xmax, ymin, ymax (cell indices; -1 if empty)} -- e.g. the dendrite
 *   tips.
 * amps_grains: cells labelled by their dominant order parameter
 *   (grain growth: eta_0..eta_{Q-1}; sintering: eta_1..eta_N where c >= level)
 *   wherever its value is >= threshold; connected components of equal labels
 *   (4-neighbour, through periodic wraps): out = {grains, labelled cells},
 *   *mean_area = labelled cells * dx * dy / grains.
 * amps_boundary_lengths: boundary length between every pair of labels
 *   (every cell labelled by its dominant order parameter; sintering: only
 *   where c >= level, so the pair lengths are the neck widths), row-major
 *   q x q symmetric into `lengths` (q = Q or N <= 32), same edge measure as
 *   the perimeter.  Kobayashi: AMPS_ERR_INVALID for the last two. */
AMPS_API int amps_compare_all(amps_handle *h, int field, const double *other, int on_device, double out[3]);
AMPS_API int amps_interface(amps_handle *h, int field, double level, double out[7]);
AMPS_API int amps_grains(amps_handle *h, double threshold, double level, int64_t out[2], double *mean_area);
AMPS_API int amps_boundary_lengths(amps_handle *h, double level, double *lengths);

/* ---- reduction that allocates nothing ------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need the result -- e.g. an application whose device
 * memory is all handed to its own pool at start-up, or code held to a fixed
 * device-memory budget: amps_reduce needs a handle, and creating one
 * allocates.  amps_reduce_noalloc folds a caller-owned row-major double
 * array `data` of n cells on the device (kind AMPS_REDUCE_*) and writes the
 * result to the caller's device slot `out`, asynchronously on `stream`
 * (cudaStream_t as void*, NULL = default stream), in a fixed order, so the
 * result is deterministic.  Its per-block partials live in one fixed
 * device array of AMPS_REDUCE_NOALLOC_MAX_BLOCKS doubles (32 KiB per device,
 * kept until the process exits); n above AMPS_REDUCE_NOALLOC_MAX_CELLS is
 * rejected with AMPS_ERR_UNSUPPORTED.  All calls share that array: calls
 * whose kernels overlap on the GPU race; order them on one stream.  The
 * first call on a device looks the array's address up with that device
 * current; make it before any stream capture on that device. */
#define AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK 4096
#define AMPS_REDUCE_NOALLOC_MAX_BLOCKS 4096
#define AMPS_REDUCE_NOALLOC_MAX_CELLS (AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK * AMPS_REDUCE_NOALLOC_MAX_BLOCKS)
AMPS_API int amps_reduce_noalloc(const double *data, int64_t n, int kind, double *out, void *stream);

/* ---- one explicit step and its adjoint (differentiation) -----------------
 * No counterpart in the reference (it only runs forward).  Stateless: the
 * caller owns every array, all row-major on the device, `dtype` AMPS_F64 or
 * AMPS_F32 for all of them, asynchronous on `stream`.  Models
 * AMPS_KOBAYASHI (state [phi; T], 2n values) and AMPS_GRAINGROWTH (state
 * [eta_0 .. eta_{Q-1}], Q = nfields <= 32, Q*n values); the step is the one
 * amps_run takes in AMPS_PUREHIGH mode (same stencils, boundaries and noise
 * stream, `step` = the noise step index), up to floating-point order.
 *   amps_step_forward: state_out = step(state_in).
 *   amps_step_adjoint: grad_in = (d step / d state_in)^T grad_out, and adds
 *     dL/dparams into grad_params (3 device doubles, not cleared):
 *     Kobayashi [delta, kappa (latent heat K), epsb]; grain growth
 *     [mobil, grcoef, gamma].  Zero-flux boundaries are differentiated
 *     exactly.  The atan2 of the Kobayashi anisotropy has no derivative where
 *     grad phi = 0; the adjoint takes it as 0 there.
 * Sintering returns AMPS_ERR_UNSUPPORTED. */
AMPS_API int amps_step_forward(const amps_params *p, int dtype, const void *state_in, void *state_out, int64_t step,
                               void *stream);
AMPS_API int amps_step_adjoint(const amps_params *p, int dtype, const void *state_in, const void *grad_out,
                               void *grad_in, double *grad_params, int64_t step, void *stream);

/* ---- checkpointed rollout and its reverse sweep --------------------------
 * A handle for N explicit steps of one model on one grid.  amps_adjoint_forward
 * runs the N steps from state0 and keeps every `segment`-th state
 * (segment 0 = ceil(sqrt(N)); 1 keeps every state and replays nothing);
 * amps_adjoint_backward takes the cotangent of the final state and returns
 * the cotangent of state0 and dL/dparams (3 device doubles, overwritten),
 * replaying each segment from its checkpoint.  param_values: the three
 * differentiable parameters (host doubles, same order as above), which
 * override those in the amps_params; step0: noise step index of the first
 * step.  All state pointers are device pointers; both calls are asynchronous
 * on the handle's stream (set_stream; NULL = default stream).  Each sweep is
 * captured once into a CUDA graph (set_graphs(0) launches kernels directly)
 * that reads the parameters and step0 from device memory, so calls with new
 * values replay it.  Memory: amps_adjoint_memory_bytes (one allocation at
 * create).  Not re-entrant per handle. */
typedef struct amps_adjoint amps_adjoint;
AMPS_API size_t amps_adjoint_memory_bytes(const amps_params *p, int dtype, int nsteps, int segment);
AMPS_API int amps_adjoint_create(const amps_params *p, int dtype, int nsteps, int segment, amps_adjoint **out);
AMPS_API int amps_adjoint_destroy(amps_adjoint *a);
AMPS_API int amps_adjoint_set_stream(amps_adjoint *a, void *stream);
AMPS_API int amps_adjoint_set_graphs(amps_adjoint *a, int enable);
AMPS_API int amps_adjoint_segment(const amps_adjoint *a);
AMPS_API const char *amps_adjoint_last_error(const amps_adjoint *a);
AMPS_API int amps_adjoint_forward(amps_adjoint *a, const double *param_values, const void *state0, void *state_final,
                                  int64_t step0);
AMPS_API int amps_adjoint_backward(amps_adjoint *a, const void *grad_final, void *grad_state0, double *grad_params);

/* ---- ensembles of grain-growth runs --------------------------------------
 * No counterpart in the reference (one run per process there).  Advances
 * `count` grain-growth handles in lockstep.  Members are grouped by the
 * occupancy their field count allows (at most 40 a group); a step is one
 * launch per group, one CTA per (member, tile), the group's step arguments
 * passed by value, so members of different sizes, field counts, parameters
 * and tier maps share the GPU.  Each cadence period is replayed from a CUDA
 * graph whose groups run as parallel branches; the members' period-end
 * classifications are one batched launch.
 * Every member keeps its own parameters (dt, mobil, grcoef, gamma,
 * thresholds...), tier maps, statistics and step counter, and gives the same
 * results as amps_run on it alone.  Members must share tile, cadence, mode
 * class (adaptive or not) and ref_order, and stand at the same phase of the
 * cadence; they stay owned by the caller and must outlive the ensemble; do
 * not run them individually while the ensemble is in use.  Work is queued
 * on the ensemble's stream (set_stream; NULL = default stream). */
typedef struct amps_ensemble amps_ensemble;
AMPS_API int amps_ensemble_create(amps_handle *const *members, int count, amps_ensemble **out);
AMPS_API int amps_ensemble_destroy(amps_ensemble *e);
AMPS_API int amps_ensemble_set_stream(amps_ensemble *e, void *stream);
AMPS_API int amps_ensemble_set_graphs(amps_ensemble *e, int enable);
AMPS_API int amps_ensemble_run(amps_ensemble *e, int nsteps);
/* Waits for the ensemble's work; reports NaN/Inf or a timed-out wait of any member. */
AMPS_API int amps_ensemble_synchronize(amps_ensemble *e);
AMPS_API const char *amps_ensemble_last_error(const amps_ensemble *e);

#ifdef __cplusplus
}
#endif
#endif
