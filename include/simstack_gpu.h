#ifndef SIMSTACK_GPU_H
#define SIMSTACK_GPU_H

/* C ABI of the GB300 kinetics module (libsimstack_gpu.so).
 *
 * Drop-in for SimStack's GPU module: every export named by the reference's
 * GPU_EXPORT_NAMES (src/gpu/gpu_api.h:112-115) is here with the reference's
 * signature, argument meaning and error convention (0 = success, otherwise a
 * cudaError_t value cast to int32_t), so the reference's own loader
 * (src/platform/linux_gpu.cpp:7-31) can dlopen this library in place of its
 * sm_86 module. The record types passed across the boundary (GpuKinLaunch,
 * GpuInfo, KinMech, KinMethod, KinControl) have the reference's byte layout.
 *
 * New capability is added as extra exports, never by changing a reference
 * signature:
 *   - GpuKinLaunch.precision = 2: mixed precision (default: double-float state
 *     with FP32 Jacobian, LU and solves; or FP64 state with an FP64-residual
 *     refinement sweep, gpu_kin_set_mixed_variant)
 *   - gpu_kin_advance_queue: persistent kernel over a device work queue
 *   - gpu_kin_autotune / gpu_kin_get_tuning: launch-shape autotuner
 *   - gpu_kin_set_straggler_budget: FP64 straggler hand-off to the cooperative kernel
 *   - gpu_kin_coop_*: cooperative (one CTA per cell) kernels for large mechanisms
 *   - gpu_advect, gpu_serve_*: film advection, CUDA-graph coupling step, serving
 *   - kin_model_*: host-side mechanism compiler (the reference's kin_build.cpp)
 *
 * No torch types, no CUDA types: plain pointers and sizes. Device pointers are
 * plain void* / double* into memory from gpu_alloc (or any CUDA allocation).
 */

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define SGB_EXTERN extern "C"
#else
#define SGB_EXTERN extern
#endif
#define SGB_API SGB_EXTERN __attribute__((visibility("default")))

/* --------------------------------------------------------------------------
 * Mechanism tables: byte layout of src/sim/kinetics/kin_mech.h:22-120 at its
 * default capacities. gpu_kin_set_mech receives this record from the caller.
 * The capacity macros can be overridden before inclusion exactly as the
 * reference's can; the module is built with the defaults.
 */
#ifndef KIN_MAX_SPECIES
#define KIN_MAX_SPECIES 32
#endif
#ifndef KIN_MAX_REACTIONS
#define KIN_MAX_REACTIONS 96
#endif
#define KIN_MAX_REACTANTS 3
#define KIN_MAX_NET 6
#ifndef KIN_MAX_NNZ
#define KIN_MAX_NNZ 512
#endif
#ifndef KIN_MAX_LU_DIV
#define KIN_MAX_LU_DIV 512
#endif
#ifndef KIN_MAX_LU_SUB
#define KIN_MAX_LU_SUB 4096
#endif
#define KIN_MAX_STAGES 4
#define KIN_NONE 0xFF

typedef struct KinReaction {
    uint8_t reactant[KIN_MAX_REACTANTS]; /* species index or KIN_NONE */
    uint8_t reactant_count;
    uint8_t net_count;
    uint8_t net_species[KIN_MAX_NET];
    int8_t net_coef[KIN_MAX_NET];                 /* products minus reactants */
    uint16_t jac_index[KIN_MAX_REACTANTS][KIN_MAX_NET]; /* J scatter slot per (reactant, net entry) */
} KinReaction;

typedef struct KinLuDiv {
    uint16_t ik, kk, sub_begin, sub_end;
} KinLuDiv;
typedef struct KinLuSub {
    uint16_t ij, kj;
} KinLuSub;
typedef struct KinRowEntry {
    uint16_t index;
    uint8_t col;
    uint8_t pad;
} KinRowEntry;

typedef struct KinMech {
    uint32_t species_count;
    uint32_t reaction_count;
    KinReaction reactions[KIN_MAX_REACTIONS];
    uint32_t nnz;
    uint16_t diag[KIN_MAX_SPECIES];
    uint32_t lu_div_count, lu_sub_count;
    uint16_t div_begin[KIN_MAX_SPECIES + 1];
    KinLuDiv lu_div[KIN_MAX_LU_DIV];
    KinLuSub lu_sub[KIN_MAX_LU_SUB];
    uint16_t lower_begin[KIN_MAX_SPECIES + 1];
    uint16_t upper_begin[KIN_MAX_SPECIES + 1]; /* upper entries in DESCENDING column order */
    KinRowEntry lower[KIN_MAX_NNZ];
    KinRowEntry upper[KIN_MAX_NNZ];
} KinMech;

typedef struct KinMethod {
    uint32_t stages;
    uint32_t order;
    double a[6], c[6];
    double m[KIN_MAX_STAGES], e[KIN_MAX_STAGES];
    double gamma0;
    int32_t new_f[KIN_MAX_STAGES];
    const char *name;
} KinMethod;

typedef struct KinControl {
    double rtol, atol;
    double h_min, h_max;
    double h_start;
    uint32_t max_steps;
    int32_t fixed_step;
    int32_t clamp_negative;
} KinControl;

/* --------------------------------------------------------------------------
 * Launch records: src/gpu/gpu_api.h:30-44.
 */
typedef struct GpuKinLaunch {
    double *y, *h, *steps, *rejects, *pulses, *failed;            /* solver writes */
    double *k, *src, *pulse, *period, *pulse_first, *pulse_count; /* solver reads */
    uint32_t padded;     /* row stride in lanes */
    uint32_t lane_count; /* lanes [0, lane_count) are integrated; 0 = all padded lanes */
    uint32_t precision;  /* 0 f64 lanes, 1 f32 lanes (delta form), 2 mixed FP32/FP64 (this module) */
    double duration;     /* local time [0, duration] */
} GpuKinLaunch;

typedef struct GpuInfo {
    char name[128];
    uint32_t sm_major, sm_minor, multiprocessors;
    uint64_t total_bytes, free_bytes;
    uint64_t arena_bytes;
} GpuInfo;

#define SGB_PRECISION_F64 0u
#define SGB_PRECISION_F32_DELTA 1u
#define SGB_PRECISION_MIXED 2u

/* --------------------------------------------------------------------------
 * The 16 reference exports (src/gpu/gpu_api.h:46-115).
 */

/* gpu_api.h:47 -- select the device, create the module's device arena, events and
 * non-blocking stream. */
SGB_API int32_t gpu_init(uint32_t device_index, uint64_t arena_bytes, GpuInfo *info);
/* gpu_api.h:50 */
SGB_API const char *gpu_error_string(int32_t error);
/* gpu_api.h:54 -- 256-byte aligned bump allocation from the arena; 0 when full. */
SGB_API void *gpu_alloc(uint64_t size);
/* gpu_api.h:57 */
SGB_API uint64_t gpu_arena_used(void);
/* gpu_api.h:62 -- waits for the device, then rolls the arena back to empty. */
SGB_API void gpu_arena_reset(void);
/* gpu_api.h:65, :68 -- copy on the module stream, then wait for it. */
SGB_API int32_t gpu_copy_to_device(void *dst_device, const void *src_host, uint64_t size);
SGB_API int32_t gpu_copy_to_host(void *dst_host, const void *src_device, uint64_t size);
/* gpu_api.h:71 */
SGB_API int32_t gpu_sync(void);
/* gpu_api.h:75 -- advances one SoA position/velocity set by dt (the loader's demo entry point;
 * here one leapfrog step under a softened pull toward the origin). */
SGB_API int32_t gpu_step_points(float *x, float *y, float *z, float *vx, float *vy, float *vz, uint32_t count, float dt);
/* gpu_api.h:80 -- upload mechanism, method and control; cudaErrorInvalidValue when the
 * mechanism does not fit. Selects the build-time straight-line kernels when the
 * mechanism's FNV-1a signature matches one, else the table-driven kernels. */
SGB_API int32_t gpu_kin_set_mech(const KinMech *mech, const KinMethod *method, const KinControl *control);
/* gpu_api.h:85 -- advance every lane over [0, duration] and wait; kernel time in ms. */
SGB_API int32_t gpu_kin_advance(const GpuKinLaunch *launch, float *kernel_ms);
/* gpu_api.h:89, :91 -- page-lock a host range (already registered counts as success). */
SGB_API int32_t gpu_host_register(void *host, uint64_t size);
SGB_API int32_t gpu_host_unregister(void *host);
/* gpu_api.h:99 -- upload lanes [0, lane_count) of a [rows][padded] f64 block, advance,
 * download the first mutable_rows rows; returns without waiting. */
SGB_API int32_t gpu_kin_advance_async(const GpuKinLaunch *launch, void *host_block, void *device_block, uint64_t rows,
                                      uint64_t mutable_rows);
/* gpu_api.h:105 */
SGB_API int32_t gpu_kin_wait(float *kernel_ms, float *total_ms);
/* gpu_api.h:109 -- 0 = one thread per cell, 1 = one warp per cell (FP64 and mixed advances run the
 * cooperative kernel with 32 threads per cell; FP64 keeps the same bits). */
SGB_API int32_t gpu_kin_set_mode(uint32_t mode);

/* --------------------------------------------------------------------------
 * Extra exports (no reference counterpart unless cited).
 */

/* Persistent kernel: resident CTAs draw cells from a device work queue (atomic
 * cursor in module-owned device memory), so cells with few steps do not idle
 * warps next to stiff ones. Same results as gpu_kin_advance for every lane. */
SGB_API int32_t gpu_kin_advance_queue(const GpuKinLaunch *launch, float *kernel_ms);

/* An addition built on gpu_api.h:99 (gpu_kin_advance_async) and :105 (gpu_kin_wait): the two
 * with the copies overlapped: lanes [0, lane_count) of the
 * host block (page-locked for overlap) are split into `chunks` (1..16) column ranges; chunk c+1
 * uploads while chunk c integrates and chunk c-1 downloads its first mutable_rows rows. Same
 * results per cell; waits; total_ms = device time from the first upload to the last download. */
SGB_API int32_t gpu_kin_advance_pipelined(const GpuKinLaunch *launch, void *host_block, void *device_block, uint64_t rows,
                                          uint64_t mutable_rows, uint32_t chunks, float *total_ms);

/* Launch tuning. kind: 0 static one-cell-per-thread, 1 persistent queue
 * (warp-synchronous), 2 persistent queue with the CTA's warps stepping
 * together (default), 3 cooperative: one cell per CTA of `block` threads
 * (32 = one warp per cell; 64..256 = 1/2..1/8 of a cell per warp; FP64 and
 * mixed only; FP64 gives the same bits as kinds 0-2). For kinds 0-2, block =
 * threads per CTA (multiple of 32; <= 128, 256 with variant 2, 512 with
 * variant 3), chunk = resident CTAs per SM for the queue kernels (0: as many
 * as fit), variant = compiled register-budget variant (0: up to 255 registers
 * at 128 threads, 1: 128 registers, 2: 255 registers at 256 threads, kind 2
 * only; 3: 128 registers at 512 threads, kind 2 only); for kind 3, chunk =
 * CTAs per SM (1..8, 0 = 8).
 * gpu_kin_autotune times the candidates of `kind` on the given launch (which
 * it advances repeatedly on a scratch copy it restores) and keeps the fastest;
 * kind 4 times kinds 2 and 3 together, so the cells-per-warp decomposition is
 * chosen by measurement as well. */
typedef struct GpuKinTuning {
    uint32_t kind, block, chunk, variant;
    float ms;
} GpuKinTuning;
SGB_API int32_t gpu_kin_set_tuning(const GpuKinTuning *tuning);
SGB_API int32_t gpu_kin_get_tuning(uint32_t precision, GpuKinTuning *tuning);
SGB_API int32_t gpu_kin_autotune(const GpuKinLaunch *launch, uint32_t kind, GpuKinTuning *best);

/* Kernel advances issued so far and the last one's kernel time. */
SGB_API int32_t gpu_kin_last_stats(uint64_t *kernel_launches, float *last_kernel_ms);

/* Mixed path (precision 2): iterative-refinement sweeps per stage solve, 1 (default) or 2. */
SGB_API int32_t gpu_kin_set_refinement(uint32_t sweeps);
/* Mixed path (precision 2) variant: 0 = FP32 Jacobian / LU / solves with an FP64-residual refinement
 * sweep per stage, FP64 state; 1 = double-float state (hi + lo FP32 pairs) with FP32 stage vectors,
 * LU and solves, stage right-hand sides accumulated in double-float, almost no FP64 work per species
 * (only the scalar step controller stays FP64). Default 1. */
SGB_API int32_t gpu_kin_set_mixed_variant(uint32_t variant);
/* Straggler hand-off for precision 0 (0 = off; default 600): in one advance, a cell still
 * stepping after `attempts` step attempts on its lane is parked and finished right after by the
 * FP64 cooperative kernel (one CTA per cell, every thread sharing the cell's work), so a few very
 * stiff cells no longer run alone on single lanes at the end of the launch; the results keep
 * the same bits. The mixed path does not hand off: its lanes' FP32-pipe steps are shorter
 * than the cooperative FP64 steps. */
SGB_API int32_t gpu_kin_set_straggler_budget(uint32_t attempts);
/* Per-thread stack (local memory) reservation of the current context: set it when set_bytes
 * is nonzero; *current receives the value in force. */
SGB_API int32_t gpu_stack_limit(uint64_t set_bytes, uint64_t *current);
/* Threads of the cooperative kernel per parked cell (32..256, multiple of 32; default 128). */
SGB_API int32_t gpu_kin_set_straggler_block(uint32_t threads);
/* Cells parked by the last advance that used the hand-off (waits for the module stream). */
SGB_API int32_t gpu_kin_parked_cells(uint32_t *count);
SGB_API uint32_t gpu_kin_get_mixed_variant(void);
/* Poll limit of the bounded waits with which the table-driven kernels stage a mechanism's
 * tables into shared memory (default 16,777,216 polls). A wait that runs out sets the launch's
 * error flag and its CTA returns without touching a lane; the advance then returns
 * cudaErrorTimeout. 0 makes every such wait give up at once: a way to exercise a caller's
 * error path without a fault. */
SGB_API int32_t gpu_kin_set_wait_limit(uint32_t polls);

/* Measured instruction throughput of this device, operations per second (an
 * FMA is one operation): kind 0 FP64 FMA, 1 FP32 FMA, 2 FP32->FP64->FP32
 * conversion pairs, 3 FP64 add, 4 FP64 reciprocal, 5 FP64 sqrt. The roofline
 * of the integrator is reported against these. */
SGB_API int32_t gpu_probe_throughput(uint32_t kind, double *ops_per_s);

/* Device-to-device copy on the module stream; returns without waiting. */
SGB_API int32_t gpu_copy_on_device(void *dst_device, const void *src_device, uint64_t size);

/* The module's stream (a cudaStream_t), for callers ordering their own work against it. */
SGB_API void *gpu_stream(void);

/* No counterpart in the reference. The persistent work-queue advance for
 * callers that cannot allocate device memory: a caller whose device memory is
 * all owned by its own arena (SimStack's platform hands the simulation one
 * fixed block), or a real-time loop that may not take cudaMalloc's device-wide
 * synchronisation. It needs no gpu_init and calls no cudaMalloc, cudaFree or
 * other allocating routine. Its scratch -- queue cursor, error flag and, for
 * mechanisms without generated code, the staged tables -- lives in a static
 * device array of 32 KiB that every GPU holds from library load to process
 * exit; a call whose scratch would exceed it returns
 * cudaErrorMemoryAllocation. mech / method / control are as for
 * gpu_kin_set_mech, the launch as for gpu_kin_advance (device pointers); the
 * kernel and launch shape are gpu_kin_advance_queue's defaults (CTA-synchronous
 * queue, 128 threads per CTA) with the module's mixed variant and refinement
 * sweeps. The work is enqueued on `stream` (a cudaStream_t, 0 = default
 * stream) and, if `wait` is nonzero, waited for and its error flag checked
 * (with wait = 0 a bounded-wait timeout of the table path is not reported: the
 * next call clears the flag). Set-up, once per device with that device
 * current and before any stream capture: the first call looks up the array's
 * device address, and the context's per-thread stack reservation must cover
 * the kernel's frame (gpu_init sets 3,840 bytes, which covers the generated
 * kernels of the shipped mechanism; the table-driven kernels of any other
 * mechanism need up to 10,752; without gpu_init, call gpu_stack_limit) -- a
 * call whose kernel needs more returns cudaErrorLaunchOutOfResources instead
 * of letting the driver grow it. Every
 * call shares the array and clears what must start at zero; calls that
 * overlap on the GPU (other streams, other host threads) race on it. */
SGB_API int32_t gpu_kin_advance_noalloc(const KinMech *mech, const KinMethod *method, const KinControl *control,
                                        const GpuKinLaunch *launch, void *stream, int32_t wait);

/* ---------------------------------------------------------------------------
 * The DBD zone driver on the device: src/sim/dbd.cpp:118-158 (dbd_zones_prepare_source,
 * dbd_zones_commit_pulses) and 466-483 (dbd_flow_exchange) as kernels on the module stream,
 * with the same bits as the reference's host driver. The zone block is the reference's
 * DbdZones block (dbd.cpp:40-83) mirrored in device memory, host-only rows included, so a
 * multi-step run keeps it device-resident and uploads nothing between master steps (the
 * reference uploads the whole block before every advance, dbd.cpp:279). Rate constants and
 * the source's temperature factors stay host-computed (libm): upload them when T or p change,
 * as dbd_zones_prepare_rates is called. Shipped humid-air mechanism only (17 species).
 */
typedef struct GpuDbdZones {
    double *y, *h, *steps, *rejects, *pulses, *failed;            /* the solver's rows */
    double *k, *src, *pulse, *period, *pulse_first, *pulse_count;
    double *pulse_index, *T_K, *p_Pa, *x_H2O, *power_W_cm3, *freq_Hz; /* DbdZones' host rows, on the device */
    double *source_temp;   /* [5][padded] temperature factors (kin_air_source_temperature) */
    uint32_t count, padded, n_species, n_reactions;
} GpuDbdZones;

/* AirSourceModel (src/sim/kinetics/air_mech.cpp:133-148) with its G-values resolved (per 100
 * eV at the reference gas's mole fractions; for the Boltzmann option pass the table's values
 * at the reduced field); filament_J_cm3 > 0 selects the filament pulse rate. NULL = defaults. */
typedef struct GpuAirSource {
    double g_O2_diss, f_O1D, g_N2A, g_N2_diss, g_OH_per_100eV, filament_J_cm3;
} GpuAirSource;

/* Host: the source's five temperature factors per zone, (T/300)^0.55 and exp(c/T) for c = 110,
 * 55, 60, 20 (air_mech.cpp:230, 265-270), into a [5][padded] block. */
SGB_API void kin_air_source_temperature(const double *T_K, uint32_t count, uint32_t padded, double *tf);
/* dbd.cpp:123-152: this master step's source (averaged: per second; pulsed: per pulse) and the
 * f64 pulse schedule in local time, for every padded zone. Waits. */
SGB_API int32_t gpu_dbd_prepare_source(const GpuDbdZones *zones, const GpuAirSource *source, uint32_t pulsed, double t0,
                                       double t1);
/* dbd.cpp:156-158: pulse_index += pulse_count. Waits. */
SGB_API int32_t gpu_dbd_commit_pulses(const GpuDbdZones *zones);
/* dbd.cpp:468-483: explicit upwind plug flow along zones [0, count), zone 0 fed by humid air at
 * its operating point; cudaErrorInvalidValue when dt count / residence_s > 1. Waits. */
SGB_API int32_t gpu_dbd_flow_exchange(const GpuDbdZones *zones, double residence_s, double dt);
/* One master step [t0, t0 + dt] as dbd_scene_step runs it (src/sim/dbd_scene.cpp:226-266): source,
 * advance of every padded lane over dt (gpu_kin_advance's kernel and tuning), pulse commit, and
 * the plug flow when `chained`; all on the module stream, nothing copied. Waits; step_ms =
 * device time of the whole step. */
SGB_API int32_t gpu_dbd_step(const GpuDbdZones *zones, const GpuAirSource *source, uint32_t pulsed, double t0, double dt,
                             uint32_t precision, uint32_t chained, double residence_s, float *step_ms);

/* ---------------------------------------------------------------------------
 * Large mechanisms (new capability; the reference's u16 KinMech tables stop
 * at 65,535 LU updates, and a 200-species / 1,200-reaction mechanism needs
 * ~1.8 M). The cooperative kernels take a finalized host model (kin_model_*
 * below) of up to 256 species and integrate one cell per CTA, every thread of
 * the CTA sharing the cell's RHS, Jacobian, elimination and solves.
 * precision 0: FP64, the same bits as the reference's solver on any mechanism
 * (each LU element gets the reference's IKJ updates in the same order);
 * precision 2: mixed (FP32 LU and solves in shared memory, FP64 RHS, Jacobian,
 * residual refinement, state and control). The launch is a GpuKinLaunch over
 * a zone block with the model's n and R rows; the work runs on the module
 * stream (gpu_init first) and is waited for. */
typedef struct KinModelHandle KinModelHandle;
SGB_API int32_t gpu_kin_coop_set_mech(const KinModelHandle *model, const KinMethod *method, const KinControl *control);
SGB_API int32_t gpu_kin_coop_advance(const GpuKinLaunch *launch, float *kernel_ms);
/* out[8]: n, R, LU non-zeros, Jacobian entries, L entries, U entries, LU updates, image bytes. */
SGB_API int32_t gpu_kin_coop_info(uint64_t *out);
/* Launch shape of the cooperative kernels per precision (0 or 2): threads per CTA (64..512,
 * multiple of 32) and resident CTAs per SM (1..2; capped by occupancy). Defaults: FP64 256 x 2
 * (measured fastest on 200 species), mixed 512 x 1 (its FP32 LU fills one SM's shared memory). */
SGB_API int32_t gpu_kin_coop_set_shape(uint32_t precision, uint32_t block, uint32_t ctas_per_sm);
/* Shared-memory bytes per CTA up to which the cooperative kernel also stages the RHS / Jacobian term
 * lists (precision 0 or 2; default 0 = never: the L1 it takes is worth more to a global-memory LU). */
SGB_API int32_t gpu_kin_coop_set_smem_budget(uint32_t precision, uint32_t bytes);
/* Clock cycles per phase of the cooperative kernel (rhs, Jacobian, factor, solves, -, whole
 * attempts), summed over CTAs' thread 0, in a build with -DSGB_COOP_PROFILE (zeros otherwise);
 * reading resets them. */
SGB_API int32_t gpu_kin_coop_phase_cycles(uint64_t *out6);
/* Refinement sweeps per stage solve of the mixed cooperative path (0..4, default 1). */
SGB_API int32_t gpu_kin_coop_set_refinement(uint32_t sweeps);

/* ---------------------------------------------------------------------------
 * Film advection and the served coupling step (new capability; the reference
 * has no GPU transport and no serving).
 *
 * gpu_advect: explicit upwind transport of a [species][padded] device block
 * whose first `cells` columns are laid out channel after channel
 * (`channel_cells` each, at most 4,096): `substeps` sweeps of
 * x_j = fma(c, x_{j-1} - x_j, x_j), cell 0 of every channel reading
 * inlet_device[species]. The flux form and the outlet-to-inlet sweep of
 * src/sim/nft.cpp:1066-1079 in FP64. Enqueued on `stream`.
 */
SGB_API int32_t gpu_advect(double *y, uint32_t padded, uint32_t species, uint32_t cells, uint32_t channel_cells,
                           const double *inlet_device, double courant, uint32_t substeps, void *stream);

/* Serving. A request is a block of cells integrated over `coupling_steps`
 * steps of `dt` seconds; every step is chemistry over dt (persistent queue
 * kernel), then film advection (operator split in the order of
 * src/sim/dbd_scene.cpp:263-265), captured once per request as a CUDA graph
 * and replayed on the request's own stream. Substeps follow the Courant-0.9
 * rule of src/sim/nft.cpp:531-536: ceil(dt / (0.9 dx / v)). The inlet of every
 * channel is the request's cell-0 initial state. State stays in device memory
 * from admission to completion. Requests are admitted in arrival order while
 * their device footprint fits the HBM budget; running requests share the GPU
 * (continuous batching: a request joins as soon as it fits, its steps run
 * beside everyone else's). Not thread-safe: one host thread drives it. */
typedef struct GpuServeRequest {
    const double *y0;          /* host [n][cells] initial state (copied at submit) */
    const double *k;           /* host [R][cells] rate constants (copied at submit) */
    uint32_t cells;
    uint32_t channel_cells;    /* cells per film channel, 1..4096 */
    uint32_t coupling_steps;
    uint32_t precision;        /* 0 FP64, 1 f32 Delta lanes, 2 mixed */
    uint32_t mechanism;        /* 0 the shipped mechanism (generated kernels), 1 the engine's table mechanism,
                                  2 the engine's large mechanism (cooperative kernels; precision 0 or 2) */
    uint32_t reserved;
    double dt;                 /* coupling step, s */
    double velocity_m_s;       /* film flow speed */
    double dx_m;               /* channel cell length */
} GpuServeRequest;

typedef struct GpuServeStatus {
    uint32_t state;            /* 0 waiting, 1 running, 2 done, 3 failed, 4 cancelled */
    int32_t error;             /* cudaError_t of a failed request (cudaErrorTimeout: a bounded wait ran out) */
    uint32_t steps_completed;
    uint32_t substeps;
    double courant;
    double admit_s;            /* submission to admission, s (-1 while waiting) */
    double latency_s;          /* submission to completion, s (-1 until finished) */
} GpuServeStatus;

typedef struct GpuServeStats {
    uint64_t budget_bytes, in_use_bytes, peak_bytes;
    uint64_t graph_launches;
    uint32_t running, waiting, finished, reserved;
} GpuServeStats;

/* Opens the engine on the current device. Budget: min(hbm_budget_bytes, free
 * memory - 1 GiB); 0 = all of it. control: NULL = rtol 1e-4, atol 6.022e8. */
SGB_API int32_t gpu_serve_open(uint64_t hbm_budget_bytes, const KinControl *control);
/* Table mechanism (mechanism = 1) and its method; only while the engine is empty. */
SGB_API int32_t gpu_serve_set_mech(const KinMech *mech, const KinMethod *method);
/* Large mechanism (mechanism = 2) from a finalized host model, up to 256 species; only while
 * the engine is empty. control: the step control of its requests (tolerances in the model's own
 * concentration units); NULL = the engine's control of gpu_serve_open. */
SGB_API int32_t gpu_serve_set_coop_mech(const KinModelHandle *model, const KinMethod *method, const KinControl *control);
/* Queues a request; cudaErrorMemoryAllocation if it could never fit the budget. */
SGB_API int32_t gpu_serve_submit(const GpuServeRequest *request, uint64_t *id);
/* One scheduling round, non-blocking apart from uploads of newly admitted and
 * downloads of finished requests: retires finished and cancelled requests,
 * launches the next step of every running request whose last step completed,
 * admits waiting requests that fit. */
SGB_API int32_t gpu_serve_progress(uint32_t *running, uint32_t *waiting, uint32_t *finished);
SGB_API int32_t gpu_serve_cancel(uint64_t id);
SGB_API int32_t gpu_serve_poll(uint64_t id, GpuServeStatus *status);
/* Final state [n][cells], accepted steps and failed flags per cell of a done request. */
SGB_API int32_t gpu_serve_result(uint64_t id, double *y_out, double *steps_out, double *failed_out);
/* Drops a finished request's record and result. */
SGB_API int32_t gpu_serve_forget(uint64_t id);
SGB_API int32_t gpu_serve_stats(GpuServeStats *stats);
SGB_API int32_t gpu_serve_close(void);

/* ---------------------------------------------------------------------------
 * NFT film transport of one coupling window (replaces src/sim/nft.cpp:1028-1106,
 * nft_transport<V>, called per group from nft_group_window, nft.cpp:1142-1152).
 * Device copies of the reference's group arrays in the reference's byte layout
 * (nft.cpp:134-178), packed group after group (groups of 8 channels = lanes):
 *   rows    [groups][cells]  NftRow      f32 f[9][8]                   288 B  in/out
 *   hot     [groups][cells]  NftCellHot  f32 c, kT, bT, ko [8]         128 B  reads c, ko; writes kT, bT
 *   cold    [groups][cells]  NftCellCold f64 vol_L[8], f32 inv_v, kw, kr, ge, ev, depth, phi, vel [8]
 *                                                                    320 B  reads kw, kr, ge, ev
 *   sites   [groups][sites]  NftSiteRow                               1,152 B reads drop, accumulates removed
 *   out_sum [groups][9][8]   sum over substeps of the outlet deltas (NftGroup::out_sum)   out
 *   evap_kg [groups][8]      film evaporation this window (NftGroup::lp.evap_kg)         out
 * ref[9] = this window's inlet (NftSystem::ref); T_amb, radiant, e0, es_slope from
 * NftEnv. flush_denormals = 1 reproduces the reference as it runs on x86-64 hosts
 * (NftFlushDenormals: FTZ/DAZ around the group's work), 0 as it runs elsewhere (IEEE);
 * either way the result is bit-identical to nft_transport<f32x8> / <f32> there.
 * rows, hot, cold and sites 16-byte aligned; cells >= 1. Synchronous on the module
 * stream; kernel_ms = device time. */
typedef struct GpuNftTransport {
    float *rows;
    float *hot;
    const float *cold;
    float *sites;
    float *out_sum;
    float *evap_kg;
    uint32_t groups, cells, sites_count, site_offset, site_stride, substeps;
    uint32_t flush_denormals;
    float ref[9];
    float T_amb, radiant, e0, es_slope;
} GpuNftTransport;
SGB_API int32_t gpu_nft_transport(const GpuNftTransport *t, float *kernel_ms);

/* ---------------------------------------------------------------------------
 * Host-side mechanism compiler: src/sim/kinetics/kin_build.cpp:78-244 and
 * air_mech.cpp:30-108, 205-276. Builds the reference-layout KinMech (same
 * pattern, pivot order and bytes as kin_mech_finalize), rate constants and
 * the discharge source. A handle is an opaque model.
 */
/* Rate-law kinds and parameters (kin_build.cpp:42-53, 226-244):
 *   0 Arrhenius  p = {A, n, E}           k = A (T/300)^n exp(-E/T)
 *   1 third body p = {A, n, E}           same times [M]
 *   2 Troe       p = {A0, n0, Ainf, ninf, fc}
 *   3 eq-reverse p = {Keq_A, Keq_B}, ref = forward reaction index */
SGB_API KinModelHandle *kin_model_new(void);
SGB_API KinModelHandle *kin_model_air(void); /* the shipped 17-species humid-air mechanism, finalized */
SGB_API void kin_model_free(KinModelHandle *model);
SGB_API uint32_t kin_model_add_species(KinModelHandle *model, const char *name, int32_t abstract_species);
SGB_API uint32_t kin_model_add_reaction(KinModelHandle *model, const char *equation, int32_t kind, const double *params,
                                        int32_t ref);
SGB_API int32_t kin_model_finalize(KinModelHandle *model); /* 0 ok, else see kin_model_error */
SGB_API const char *kin_model_error(const KinModelHandle *model);
SGB_API int32_t kin_model_equation(const KinModelHandle *model, uint32_t r, char *out, uint32_t size); /* 0 if out of range */
/* counts[0..6] = species, reactions, nnz, lu divisions, lu updates, lower, upper */
SGB_API void kin_model_counts(const KinModelHandle *model, uint64_t *counts);
/* Reference-layout tables; cudaErrorInvalidValue (1) if the mechanism exceeds them. */
SGB_API int32_t kin_model_kinmech(const KinModelHandle *model, KinMech *out);
SGB_API uint64_t kin_mech_signature(const KinMech *mech); /* FNV-1a over the record */
/* The cooperative kernels' wide-index image (pattern bitmask, term lists, elimination lists) of a
 * finalized model or of a KinMech; returns its size (0 if it cannot be built) and copies it to
 * `out` when `capacity` suffices. The same mechanism gives the same bytes from either source. */
SGB_API uint64_t kin_model_coop_image(const KinModelHandle *model, void *out, uint64_t capacity);
SGB_API uint64_t kin_mech_coop_image(const KinMech *mech, void *out, uint64_t capacity);
SGB_API void kin_model_rate_constants(const KinModelHandle *model, double T, double M, double *k);
/* Rate constants for `cells` cells of a [reactions][padded] block from T and M per cell. */
SGB_API void kin_model_rate_block(const KinModelHandle *model, const double *T, const double *M, uint32_t cells,
                                  uint32_t padded, double *k);
SGB_API KinMethod kin_method_coefficients(uint32_t method_id); /* 0 ros2, 1 ros3, 2 rodas3 */
/* Averaged-discharge source per second for the shipped mechanism (air_mech.cpp:205-276). */
SGB_API void kin_air_source_delta(const double *y, uint32_t species, double energy_J_cm3, double T_K, double *delta);

#endif /* SIMSTACK_GPU_H */
