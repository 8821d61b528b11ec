// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// Thin C ABI over the reference's own CPU solver, compiled from the reference
// sources where they lie (include path REF_DIR/src, nothing copied) by
// oracle/Makefile into oracle/_ref/. The tests use it here to pin the oracle
// restatement (kin_oracle.cpp) bit for bit and to generate tests/golden/.
// It is never built on a machine without the reference sources.
//
// What it calls: kin_mech_finalize and air_mech_build (kin_build.cpp,
// air_mech.cpp), kin_eval_rate_constants, kin_integrate (kin_solver.h),
// dbd_advance_cpu / dbd_advance_group (dbd.cpp, dbd_lanes.h) with the
// generated AirGenOps or the table walk, f64 / f64x4 / f32 / f32x8 lanes,
// and air_source_delta; and, with a GPU module loaded by the reference's own
// loader (linux_load_gpu_module), the hybrid CPU+GPU driver dbd_advance_hybrid.

// Profiler shim: the reference's base_debug.h reads the x86 TSC; the solver
// only uses its TIMED_FUNCTION() markers, which compile to nothing here.
#define BASE_DEBUG_H
#define TIMED_BLOCK(name)
#define TIMED_FUNCTION()
struct DebugTable;

#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <dlfcn.h>
#include <time.h>

#include <atomic>
#include <thread>
#include <vector>

#include "sim_platform.h"
#include "sim/dbd.cpp"
#include "platform/linux_gpu.cpp"

#define REF_API extern "C" __attribute__((visibility("default")))

static KinModel g_air;
static AirSpecies g_air_sp;
static int g_air_built;

static KinModel *air_model() {
    if (!g_air_built) {
        air_mech_build(&g_air, &g_air_sp);
        g_air_built = 1;
    }
    return &g_air;
}

REF_API u64 ref_kinmech_size(void) { return sizeof(KinMech); }

// The shipped mechanism's KinMech bytes, and the generated kernels' signature.
REF_API s32 ref_air_kinmech(void *out, u64 *signature, u64 *generated_signature) {
    KinModel *m = air_model();
    if (m->error) return 0;
    memcpy(out, &m->mech, sizeof(KinMech));
    if (signature) *signature = hash_fnv1a_64(&m->mech, sizeof(KinMech));
    if (generated_signature) *generated_signature = AirGenOps::signature;
    return 1;
}

REF_API void ref_air_rate_constants(f64 T, f64 M, f64 *k) { kin_eval_rate_constants(air_model(), T, M, k); }

REF_API void ref_air_source_delta(const f64 *y, f64 energy_J_cm3, f64 T_K, f64 *delta) {
    AirSourceModel src = air_source_defaults();
    air_source_delta(&g_air_sp, &src, y, air_model()->mech.species_count, energy_J_cm3, delta, T_K);
}

struct RefControl {
    f64 rtol, atol, h_min, h_max, h_start;
    u32 max_steps;
    s32 fixed_step, clamp_negative;
};

static KinControl to_control(const RefControl *c) {
    KinControl k = {};
    k.rtol = c->rtol; k.atol = c->atol; k.h_min = c->h_min; k.h_max = c->h_max; k.h_start = c->h_start;
    k.max_steps = c->max_steps; k.fixed_step = c->fixed_step; k.clamp_negative = c->clamp_negative;
    return k;
}

struct RefLaneArrays {
    f64 *y, *h, *steps, *rejects, *pulses, *failed;
    const f64 *k, *src, *pulse, *period, *pulse_first, *pulse_count;
    u32 padded;
};

// Lanes [first, end) of a zone block with the shipped mechanism.
// variant 0: f64x4 generated (the production CPU path), 1: f64x4 table walk,
// 2: f64 scalar table walk, 3: f32x8 generated (Delta), 4: f32 scalar generated (Delta).
REF_API s32 ref_air_advance(s32 method_id, const RefControl *rc, const RefLaneArrays *a, u32 first, u32 end,
                            f64 duration, s32 variant) {
    KinModel *model = air_model();
    KinMethod method = kin_method((KinMethodId)method_id);
    KinControl ctl = to_control(rc);
    DbdZones z = {};
    z.padded = a->padded;
    z.n_species = model->mech.species_count;
    z.n_reactions = model->mech.reaction_count;
    z.y = a->y; z.h = a->h; z.steps = a->steps; z.rejects = a->rejects; z.pulses = a->pulses; z.failed = a->failed;
    z.k = (f64 *)a->k; z.src = (f64 *)a->src; z.pulse = (f64 *)a->pulse; z.period = (f64 *)a->period;
    z.pulse_first = (f64 *)a->pulse_first; z.pulse_count = (f64 *)a->pulse_count;
    if ((variant == 0 || variant == 1) && (first % 4 || end % 4)) return -1;
    if (variant == 3 && (first % 8 || end % 8)) return -1;
    switch (variant) {
        case 0: dbd_advance_cpu<f64x4, AirGenOps>(&z, &model->mech, &method, &ctl, duration, first, end); break;
        case 1: dbd_advance_cpu<f64x4>(&z, &model->mech, &method, &ctl, duration, first, end); break;
        case 2: dbd_advance_cpu<f64>(&z, &model->mech, &method, &ctl, duration, first, end); break;
        case 3: dbd_advance_cpu<f32x8, AirGenOps, true>(&z, &model->mech, &method, &ctl, duration, first, end); break;
        case 4: dbd_advance_cpu<f32, AirGenOps, true>(&z, &model->mech, &method, &ctl, duration, first, end); break;
        default: return -1;
    }
    return 0;
}

// Rate constants of `cells` cells from T and M per cell into a [reaction][padded] block:
// the reference's kin_eval_rate_constants, cell by cell.
REF_API void ref_air_rate_block(const f64 *T, const f64 *M, u32 cells, u32 padded, f64 *k) {
    KinModel *model = air_model();
    const u32 R = model->mech.reaction_count;
    f64 kk[KIN_MAX_REACTIONS];
    for (u32 i = 0; i < cells; ++i) {
        kin_eval_rate_constants(model, T[i], M[i], kk);
        for (u32 r = 0; r < R; ++r) k[(u64)r * padded + i] = kk[r];
    }
}

// A work queue behind the reference's PlatformAPI (sim_platform.h:41-62), so the
// reference's own threaded advance runs here unchanged: add_work_entry records an
// entry, complete_all_work runs every recorded entry on `threads` threads (the
// caller among them) and returns when all have finished.
struct PlatformWorkQueue {
    struct Entry { platform_work_queue_callback *fn; void *data; };
    std::vector<Entry> entries;
    u32 threads;
};

static PLATFORM_ADD_WORK_ENTRY(ref_add_work_entry) { queue->entries.push_back({callback, data}); }

static PLATFORM_COMPLETE_ALL_WORK(ref_complete_all_work) {
    std::atomic<u32> next{0};
    const u32 count = (u32)queue->entries.size();
    auto worker = [&]() {
        for (u32 i = next.fetch_add(1); i < count; i = next.fetch_add(1)) queue->entries[i].fn(queue, queue->entries[i].data);
    };
    std::vector<std::thread> pool;
    for (u32 t = 1; t < queue->threads; ++t) pool.emplace_back(worker);
    worker();
    for (std::thread &th : pool) th.join();
    queue->entries.clear();
}

// Lanes [first, end) of a zone block through the reference's production CPU path,
// dbd_advance_threads (dbd.cpp:213-250): f64x4 lanes with the generated AirGenOps,
// about four contiguous lane chunks per thread, on `threads` host threads.
REF_API s32 ref_air_advance_threads(s32 method_id, const RefControl *rc, const RefLaneArrays *a, u32 first, u32 end,
                                    f64 duration, u32 threads) {
    KinModel *model = air_model();
    KinMethod method = kin_method((KinMethodId)method_id);
    KinControl ctl = to_control(rc);
    if (first % 8 || end % 8 || threads == 0) return -1;
    DbdZones z = {};
    z.padded = a->padded;
    z.n_species = model->mech.species_count;
    z.n_reactions = model->mech.reaction_count;
    z.y = a->y; z.h = a->h; z.steps = a->steps; z.rejects = a->rejects; z.pulses = a->pulses; z.failed = a->failed;
    z.k = (f64 *)a->k; z.src = (f64 *)a->src; z.pulse = (f64 *)a->pulse; z.period = (f64 *)a->period;
    z.pulse_first = (f64 *)a->pulse_first; z.pulse_count = (f64 *)a->pulse_count;
    PlatformAPI api = {};
    api.add_work_entry = ref_add_work_entry;
    api.complete_all_work = ref_complete_all_work;
    PlatformWorkQueue queue;
    queue.threads = threads;
    static u8 frame_memory[1 << 20];
    Arena frame = arena_make(frame_memory, sizeof(frame_memory));
    dbd_advance_threads(&z, &model->mech, &method, &ctl, duration, 1, DbdPrecision_F64, &api, &queue, threads, &frame,
                        first, end);
    return 0;
}

// `steps` master steps of dt of the reference's own zone driver on a DbdZones block in the
// reference's layout (dbd.cpp:60-83: the solver's rows, then pulse_index, T_K, p_Pa, x_H2O,
// power_W_cm3, freq_Hz): dbd_zones_prepare_source, dbd_advance_cpu<f64x4, AirGenOps>,
// dbd_zones_commit_pulses and, when chained, dbd_flow_exchange -- dbd_scene_step's sequence
// (dbd_scene.cpp:232-265) without the scene around it. mode 0 pulsed, 1 averaged; the advance
// on `threads` host threads (dbd_advance_threads) when threads > 1, f32x8 Delta lanes when
// f32_lanes (the sweep scene's default precision), else f64x4 lanes.
// The zone block's rows in the reference's order (dbd.cpp:60-83), over a caller's f64 block.
static DbdZones zones_over(f64 *block, u32 count, u32 padded, const KinModel *model) {
    DbdZones z = {};
    z.count = count;
    z.padded = padded;
    z.n_species = model->mech.species_count;
    z.n_reactions = model->mech.reaction_count;
    u64 p = padded, ns = z.n_species, nr = z.n_reactions;
    f64 **rows[] = {&z.y, &z.h, &z.steps, &z.rejects, &z.pulses, &z.failed, &z.k, &z.src, &z.pulse, &z.period,
                    &z.pulse_first, &z.pulse_count, &z.pulse_index, &z.T_K, &z.p_Pa, &z.x_H2O, &z.power_W_cm3, &z.freq_Hz};
    u64 counts[] = {ns * p, p, p, p, p, p, nr * p, ns * p, ns * p, p, p, p, p, p, p, p, p, p};
    u64 off = 0;
    for (u32 i = 0; i < 18; ++i) {
        *rows[i] = block + off;
        off += counts[i];
    }
    z.block = block;
    z.block_count = off;
    z.mutable_count = (ns + 5) * p;   // y, h, steps, rejects, pulses, failed: the solver-written prefix
    return z;
}

REF_API s32 ref_dbd_run(f64 *block, u32 count, u32 padded, s32 mode, u32 steps, f64 dt, s32 chained, f64 residence_s,
                        const RefControl *rc, u32 threads, u32 f32_lanes) {
    KinModel *model = air_model();
    if (padded % 8) return -1;
    KinMethod method = kin_method(KinMethod_Rodas3);
    KinControl ctl = to_control(rc);
    AirSourceModel source = air_source_defaults();
    DbdZones z = zones_over(block, count, padded, model);
    f64 t = 0.0;   // the scene clock: t1 = t + dt, then t = t1 (dbd_scene.cpp:232, 266)
    for (u32 s = 0; s < steps; ++s) {
        f64 t0 = t, t1 = t + dt;
        dbd_zones_prepare_source(&z, &g_air_sp, &source, (DbdDischargeMode)mode, t0, t1);
        if (threads > 1) {   // the sim's own threaded advance (dbd_scene.cpp:261)
            PlatformAPI api = {};
            api.add_work_entry = ref_add_work_entry;
            api.complete_all_work = ref_complete_all_work;
            PlatformWorkQueue queue;
            queue.threads = threads;
            static u8 frame_memory[1 << 20];
            Arena frame = arena_make(frame_memory, sizeof(frame_memory));
            dbd_advance_threads(&z, &model->mech, &method, &ctl, dt, 1, f32_lanes ? DbdPrecision_F32 : DbdPrecision_F64, &api,
                                &queue, threads, &frame);
        } else if (f32_lanes) {
            dbd_advance_cpu<f32x8, AirGenOps, true>(&z, &model->mech, &method, &ctl, dt);
        } else {
            dbd_advance_cpu<f64x4, AirGenOps>(&z, &model->mech, &method, &ctl, dt);
        }
        dbd_zones_commit_pulses(&z);
        if (chained) dbd_flow_exchange(&z, &g_air_sp, residence_s, dt);
        t = t1;
    }
    return 0;
}

// The reference's GPU module table, filled by its own loader from the module at `path`
// (platform/linux_gpu.cpp:7-31: dlopen, the 16 exports by name, gpu_init(0, arena)).
// Loaded once per process; a second path is refused.
static GpuAPI g_gpu;
static char g_gpu_path[1024];

REF_API s32 ref_gpu_load(const char *path, u64 arena_bytes) {
    if (g_gpu.available) return strcmp(path, g_gpu_path) == 0 ? 0 : -2;
    if (!linux_load_gpu_module(path, arena_bytes, &g_gpu)) return -1;
    snprintf(g_gpu_path, sizeof(g_gpu_path), "%s", path);
    return 0;
}

static u64 ref_now_ns(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (u64)ts.tv_sec * 1000000000ull + (u64)ts.tv_nsec;
}

// `steps` master steps of dt of dbd_scene_step's sequence (dbd_scene.cpp:232-265) with the
// reference's hybrid advance, dbd_advance_hybrid (dbd.cpp:336-463): lanes [0, split) on the
// loaded GPU module (gpu_kin_set_mech, gpu_host_register, gpu_kin_advance_async,
// gpu_kin_wait), lanes [split, padded) on `threads` host threads through
// dbd_advance_threads, the split chosen by its own measured search (force_split < 0) or
// fixed (force_split >= 0). Per step: the split used, the step's wall time (ms), and the
// module's launch-to-completion time (ms, 0 for a CPU-only step). The block is page-locked
// for the run and released at the end. precision: 0 FP64 lanes, 1 f32 Delta lanes.
REF_API s32 ref_dbd_hybrid_run(f64 *block, u32 count, u32 padded, s32 mode, u32 steps, f64 dt, s32 chained,
                               f64 residence_s, const RefControl *rc, u32 threads, u32 precision, s32 force_split,
                               u32 *split_out, f32 *step_ms_out, f32 *gpu_ms_out) {
    if (!g_gpu.available) return -1;
    KinModel *model = air_model();
    if (padded % 8 || threads == 0) return -1;
    KinMethod method = kin_method(KinMethod_Rodas3);
    KinControl ctl = to_control(rc);
    AirSourceModel source = air_source_defaults();
    DbdZones z = zones_over(block, count, padded, model);
    s32 err = g_gpu.gpu_kin_set_mech(&model->mech, &method, &ctl);
    if (err) return err;
    g_gpu.gpu_arena_reset();
    PlatformAPI api = {};
    api.add_work_entry = ref_add_work_entry;
    api.complete_all_work = ref_complete_all_work;
    api.now_ns = ref_now_ns;
    PlatformWorkQueue queue;
    queue.threads = threads;
    static u8 frame_memory[1 << 20];
    DbdGpu g = {};
    DbdHybrid *hy = (DbdHybrid *)calloc(1, sizeof(DbdHybrid));
    hy->force_split = force_split;
    f64 t = 0.0;
    for (u32 s = 0; s < steps && !err; ++s) {
        f64 t0 = t, t1 = t + dt;
        dbd_zones_prepare_source(&z, &g_air_sp, &source, (DbdDischargeMode)mode, t0, t1);
        u32 split = force_split >= 0 ? (u32)force_split : hy->split;
        split = Minimum(split & ~7u, padded);
        Arena frame = arena_make(frame_memory, sizeof(frame_memory));
        u64 a = ref_now_ns();
        err = dbd_advance_hybrid(&z, &g_gpu, &g, hy, dt, precision, &model->mech, &method, &ctl, 1, &api, &queue,
                                 threads, &frame);
        u64 b = ref_now_ns();
        if (split_out) split_out[s] = split;
        if (step_ms_out) step_ms_out[s] = (f32)((f64)(b - a) * 1e-6);
        if (gpu_ms_out) gpu_ms_out[s] = split ? hy->last_gpu_ms : 0.0f;
        dbd_zones_commit_pulses(&z);
        if (chained) dbd_flow_exchange(&z, &g_air_sp, residence_s, dt);
        t = t1;
    }
    if (hy->registered) g_gpu.gpu_host_unregister(hy->registered_block);
    free(hy);
    g_gpu.gpu_arena_reset();
    return err;
}

// Robertson (test_kinetics.cpp:151-180 set-up): one scalar integration.
REF_API s32 ref_robertson(s32 method_id, const RefControl *rc, f64 t_end, f64 *y3, f64 *stats4) {
    KinModel *model = (KinModel *)calloc(1, sizeof(KinModel));
    kin_add_species(model, "A", 1);
    kin_add_species(model, "B", 1);
    kin_add_species(model, "C", 1);
    kin_add_reaction(model, "A -> B", kin_arr(0.04));
    kin_add_reaction(model, "B + B -> C + B", kin_arr(3.0e7));
    kin_add_reaction(model, "B + C -> A + C", kin_arr(1.0e4));
    kin_mech_finalize(model);
    f64 k[3];
    kin_eval_rate_constants(model, 300.0, 1.0, k);
    KinMethod method = kin_method((KinMethodId)method_id);
    KinControl ctl = to_control(rc);
    f64 src[3] = {}, t = 0.0, h = 0.0;
    KinLaneStats<f64> st = {};
    kin_integrate(&model->mech, &method, &ctl, k, src, y3, t, t_end, h, st);
    stats4[0] = st.steps; stats4[1] = st.rejects; stats4[2] = st.pulses; stats4[3] = st.failed;
    free(model);
    return 0;
}
