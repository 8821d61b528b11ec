// Exports of the GB300 kinetics module: the reference's 16-entry GPU C ABI
// (src/gpu/gpu_api.h) plus the module's extra entry points. One device, one
// module-owned non-blocking stream; every copy and kernel of the module is
// ordered on it (the reference's rule, src/gpu/kernels.cu:333-348), except in
// gpu_kin_advance_pipelined, whose upload, download and second kernel streams
// start after the module stream's earlier work and are drained before it returns.

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/simstack_gpu.h"
#include "kin_kernels.cuh"
#include "kin_table.cuh"
#include "mech.h"
#include "mech_tables.h"
#include "coop.h"

#include <vector>

namespace sgb {
cudaError_t launch_air_p0(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t launch_air_p1(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t launch_air_p2(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t occupancy_air_p0(uint32_t, uint32_t, uint32_t, int *);
cudaError_t occupancy_air_p1(uint32_t, uint32_t, uint32_t, int *);
cudaError_t occupancy_air_p2(uint32_t, uint32_t, uint32_t, int *);
cudaError_t launch_table_p0(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t launch_table_p1(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t launch_table_p2(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t occupancy_table_p0(uint32_t, uint32_t, size_t, int *);
cudaError_t occupancy_table_p1(uint32_t, uint32_t, size_t, int *);
cudaError_t occupancy_table_p2(uint32_t, uint32_t, size_t, int *);
cudaError_t launch_air_p3(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t occupancy_air_p3(uint32_t, uint32_t, uint32_t, int *);
cudaError_t launch_table_p3(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t occupancy_table_p3(uint32_t, uint32_t, size_t, int *);
cudaError_t launch_air_p4(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t occupancy_air_p4(uint32_t, uint32_t, uint32_t, int *);
cudaError_t launch_table_p4(const Shape &, const DevArgs &, cudaStream_t);
cudaError_t occupancy_table_p4(uint32_t, uint32_t, size_t, int *);
cudaError_t local_air_p4(uint32_t, uint32_t, size_t *);
cudaError_t local_table_p4(uint32_t, size_t *);
cudaError_t local_air_p0(uint32_t, uint32_t, size_t *);
cudaError_t local_air_p1(uint32_t, uint32_t, size_t *);
cudaError_t local_air_p2(uint32_t, uint32_t, size_t *);
cudaError_t local_air_p3(uint32_t, uint32_t, size_t *);
cudaError_t local_table_p0(uint32_t, size_t *);
cudaError_t local_table_p1(uint32_t, size_t *);
cudaError_t local_table_p2(uint32_t, size_t *);
cudaError_t local_table_p3(uint32_t, size_t *);
uint64_t air_ops_signature();
size_t coop_smem_bytes_for(int prec, const CoopMech &h);
size_t coop_scratch_doubles_for(int prec, const CoopMech &h);
cudaError_t coop_launch(int prec, const DevArgs &A, const CoopMech &head, double *scratch, uint32_t grid,
                               uint32_t block, cudaStream_t s);
cudaError_t run_probe(uint32_t kind, int sms, cudaStream_t stream, double *ops_per_s);
}   // namespace sgb

using namespace sgb;

namespace {

struct Module {
    bool ready = false;
    int device = 0, sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t kin_start = nullptr, kin_stop = nullptr, async_begin = nullptr, async_end = nullptr;
    uint8_t *arena = nullptr;
    uint64_t arena_size = 0, arena_used = 0;
    // mechanism
    bool have_mech = false, generated = false;
    KinMech mech;
    KinMethod method;
    KinControl control;
    void *d_tables = nullptr;      // KinMech image, kTableBytes
    uint32_t *d_cursor = nullptr;  // work-queue cursor
    uint32_t *d_error = nullptr;   // bounded-wait error flag
    uint32_t mode = 0;
    GpuKinTuning tuning[3];
    uint32_t ir_sweeps = 1;
    uint32_t wait_polls = kSpinLimit;   // poll limit of the table-staging waits
    // precision 2: 0 FP64-residual refinement, 1 double-float state, 2 double-float state with
    // refined stages (default: the variant that tracks the FP64 path to its tolerance)
    uint32_t mixed_variant = 2;
    uint64_t launches = 0;
    float last_ms = 0.0f;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;   // pipelined advance: upload and download streams
    cudaStream_t kern2 = nullptr;                         // ... and a second kernel stream
    static constexpr int kMaxChunks = 16;
    cudaEvent_t ev_in[kMaxChunks] = {}, ev_kern[kMaxChunks] = {};
    cudaEvent_t pipe_begin = nullptr, pipe_end = nullptr, pipe_after = nullptr;
    // straggler hand-off: cells past `straggler_budget` step attempts in one launch are parked
    // and finished by the cooperative kernel (one CTA per cell) on the same stream
    uint32_t straggler_budget = 600;  // FP64 step attempts per launch before a cell is handed on
    uint32_t straggler_block = 128;   // threads per parked cell
    SuspendRec *d_suspend = nullptr;
    uint32_t *d_suspend_count = nullptr;
    void *d_coop_image = nullptr;
    CoopMech coop_head;
    double *d_coop_scratch = nullptr;
    uint32_t coop_grid = 0;
    void *d_dbd_scratch = nullptr;   // zone driver: the y rows before a plug-flow exchange
    size_t dbd_scratch_bytes = 0;
};
Module g;
constexpr uint32_t kSuspendCap = 1u << 16;       // parked cells per launch
// The context's per-thread stack (local memory) reservation, set once at gpu_init before any
// launch so that it is never resized: the mixed kernel spills to local memory, and its speed
// depends on where that memory lands (measured on GB300: 397-548 ms for the same launch at
// different reservations and reallocations); 3,840 bytes covers every default-path kernel of
// the shipped mechanism (the FP64 lanes need 3,680) and was the fastest such size measured.
constexpr size_t kStackReserveBytes = 3840;
constexpr uint32_t kResumeCtasPerSm = 8;         // cooperative CTAs per SM for parked cells


const GpuKinTuning kDefaultTuning = {2u, 128u, 0u, 0u, 0.0f};   // CTA-synchronous queue, 128 threads, 255 registers

void fill_args(const GpuKinLaunch *L, DevArgs *A) {
    memset(A, 0, sizeof(*A));
    A->y = L->y; A->h = L->h; A->steps = L->steps; A->rejects = L->rejects; A->pulses = L->pulses; A->failed = L->failed;
    A->k = L->k; A->src = L->src; A->pulse = L->pulse; A->period = L->period;
    A->pulse_first = L->pulse_first; A->pulse_count = L->pulse_count;
    A->padded = L->padded;
    A->lanes = L->lane_count ? L->lane_count : L->padded;
    A->duration = L->duration;
    A->ctl = g.control;
    memcpy(A->ma, g.method.a, sizeof(A->ma));
    memcpy(A->mc, g.method.c, sizeof(A->mc));
    memcpy(A->mm, g.method.m, sizeof(A->mm));
    memcpy(A->me, g.method.e, sizeof(A->me));
    A->gamma0 = g.method.gamma0;
    memcpy(A->new_f, g.method.new_f, sizeof(A->new_f));
    A->stages = g.method.stages;
    A->order = g.method.order;
    A->ir_sweeps = g.ir_sweeps;
    A->cursor = g.d_cursor;
    A->error_flag = g.d_error;
    A->wait_polls = g.wait_polls;
    A->tables = g.d_tables;
    A->table_bytes = kTableBytes;
}

cudaError_t occupancy(uint32_t prec, const GpuKinTuning &t, int *blocks) {
    if (prec == 2 && g.mixed_variant == 2)
        return g.generated ? occupancy_air_p4(t.kind, t.variant, t.block, blocks)
                           : occupancy_table_p4(t.kind, t.block, kTableBytes, blocks);
    if (prec == 2 && g.mixed_variant == 1)
        return g.generated ? occupancy_air_p3(t.kind, t.variant, t.block, blocks)
                           : occupancy_table_p3(t.kind, t.block, kTableBytes, blocks);
    if (g.generated) {
        if (prec == 0) return occupancy_air_p0(t.kind, t.variant, t.block, blocks);
        if (prec == 1) return occupancy_air_p1(t.kind, t.variant, t.block, blocks);
        return occupancy_air_p2(t.kind, t.variant, t.block, blocks);
    }
    if (prec == 0) return occupancy_table_p0(t.kind, t.block, kTableBytes, blocks);
    if (prec == 1) return occupancy_table_p1(t.kind, t.block, kTableBytes, blocks);
    return occupancy_table_p2(t.kind, t.block, kTableBytes, blocks);
}

cudaError_t launch_lanes(uint32_t prec, const GpuKinTuning &t, const DevArgs &A, cudaStream_t stream = nullptr);

// Local memory per thread the kernel of (precision, tuning) needs.
cudaError_t local_bytes(uint32_t prec, const GpuKinTuning &t, size_t *bytes) {
    if (t.kind == 3) {   // the cooperative kernel keeps its state in shared and global memory
        *bytes = 0;
        return cudaSuccess;
    }
    const bool df = prec == 2 && g.mixed_variant == 1;
    if (prec == 2 && g.mixed_variant == 2) return g.generated ? local_air_p4(t.kind, t.variant, bytes) : local_table_p4(t.kind, bytes);
    if (g.generated) {
        if (df) return local_air_p3(t.kind, t.variant, bytes);
        return prec == 0 ? local_air_p0(t.kind, t.variant, bytes) : prec == 1 ? local_air_p1(t.kind, t.variant, bytes)
                                                                              : local_air_p2(t.kind, t.variant, bytes);
    }
    if (df) return local_table_p3(t.kind, bytes);
    return prec == 0 ? local_table_p0(t.kind, bytes) : prec == 1 ? local_table_p1(t.kind, bytes) : local_table_p2(t.kind, bytes);
}

// Launches one advance of `A` with tuning `t` on the module stream; with a
// straggler budget (precision 0), cells still stepping after that many
// attempts are parked and finished by the FP64 cooperative kernel right after,
// with the same bits. (The mixed lanes' FP32-pipe steps are shorter than the
// cooperative FP64 steps, so they keep their cells.)
cudaError_t launch_advance(uint32_t prec, const GpuKinTuning &t, const DevArgs &A0) {
    if (A0.lanes == 0) return cudaSuccess;
    if (t.kind == 3) {   // cooperative decomposition: one cell per CTA of t.block threads (32: one warp per cell)
        if (!g.d_coop_image || prec == 1) return cudaErrorInvalidValue;
        DevArgs R = A0;
        R.budget = 0;
        R.resume = 0;
        R.tables = g.d_coop_image;
        R.table_bytes = g.coop_head.bytes;
        const uint32_t per_sm = t.chunk ? (t.chunk < kResumeCtasPerSm ? t.chunk : kResumeCtasPerSm) : kResumeCtasPerSm;
        uint32_t grid = (uint32_t)g.sms * per_sm;
        if (grid > A0.lanes) grid = A0.lanes;
        cudaError_t e = cudaMemsetAsync(A0.cursor, 0, sizeof(uint32_t), g.stream);
        if (e != cudaSuccess) return e;
        return coop_launch((int)prec, R, g.coop_head, g.d_coop_scratch, grid, t.block, g.stream);
    }
    const bool handoff = g.straggler_budget && g.d_coop_image && prec == 0;
    if (!handoff) return launch_lanes(prec, t, A0);
    DevArgs A = A0;
    A.budget = g.straggler_budget;
    A.suspend_cap = kSuspendCap;
    A.suspend_count = g.d_suspend_count;
    A.suspend = g.d_suspend;
    cudaError_t e = cudaMemsetAsync(g.d_suspend_count, 0, sizeof(uint32_t), g.stream);
    if (e == cudaSuccess) e = launch_lanes(prec, t, A);
    if (e != cudaSuccess) return e;
    DevArgs R = A;
    R.budget = 0;
    R.resume = 1;
    R.tables = g.d_coop_image;
    R.table_bytes = g.coop_head.bytes;
    e = cudaMemsetAsync(g.d_cursor, 0, sizeof(uint32_t), g.stream);
    if (e != cudaSuccess) return e;
    return coop_launch(0, R, g.coop_head, g.d_coop_scratch, g.coop_grid, g.straggler_block, g.stream);
}

// The lane kernels (one cell per thread) for `A`, on `stream` (default: the module stream); the
// queue kernels take their cells from A.cursor.
cudaError_t launch_lanes(uint32_t prec, const GpuKinTuning &t, const DevArgs &A, cudaStream_t stream) {
    if (A.lanes == 0) return cudaSuccess;
    if (!stream) stream = g.stream;
    Shape s;
    s.kind = t.kind;
    s.block = t.block;
    s.variant = t.variant;
    s.smem = g.generated ? 0 : kTableBytes;
    if (t.kind == 0) {
        s.grid = (A.lanes + t.block - 1) / t.block;
    } else {   // queue kernels: persistent grid, the cursor starts at zero
        int per_sm = 0;
        cudaError_t e = occupancy(prec, t, &per_sm);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        if (t.chunk > 0 && (int)t.chunk < per_sm) per_sm = (int)t.chunk;   // chunk: CTAs per SM (0 = as many as fit)
        uint32_t resident = (uint32_t)per_sm * (uint32_t)g.sms;
        uint32_t needed = (A.lanes + t.block - 1) / t.block;
        s.grid = resident < needed ? resident : needed;
        e = cudaMemsetAsync(A.cursor, 0, sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
    }
    if (prec == 2 && g.mixed_variant == 2) {
        if (g.generated) return launch_air_p4(s, A, stream);
        s.variant = 0;
        return launch_table_p4(s, A, stream);
    }
    if (prec == 2 && g.mixed_variant == 1) {
        if (g.generated) return launch_air_p3(s, A, stream);
        s.variant = 0;
        return launch_table_p3(s, A, stream);
    }
    if (g.generated) {
        if (prec == 0) return launch_air_p0(s, A, stream);
        if (prec == 1) return launch_air_p1(s, A, stream);
        return launch_air_p2(s, A, stream);
    }
    s.variant = 0;
    if (prec == 0) return launch_table_p0(s, A, stream);
    if (prec == 1) return launch_table_p1(s, A, stream);
    return launch_table_p2(s, A, stream);
}

cudaError_t check_launch(const GpuKinLaunch *L) {
    if (!g.ready) return cudaErrorInitializationError;
    if (!g.have_mech) return cudaErrorInvalidValue;
    if (!L || L->precision > 2 || L->padded == 0) return cudaErrorInvalidValue;
    if (L->lane_count > L->padded) return cudaErrorInvalidValue;
    if (!(L->duration >= 0.0) || L->duration > 1.0e300) return cudaErrorInvalidValue;   // NaN, negative or infinite
    if (!L->y || !L->h || !L->steps || !L->rejects || !L->pulses || !L->failed || !L->k || !L->src || !L->pulse ||
        !L->period || !L->pulse_first || !L->pulse_count)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t read_error_flag() {
    uint32_t flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, g.d_error, sizeof(flag), cudaMemcpyDeviceToHost, g.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.stream);
    if (e != cudaSuccess) return e;
    if (flag) {
        cudaMemsetAsync(g.d_error, 0, sizeof(uint32_t), g.stream);
        cudaStreamSynchronize(g.stream);
        return cudaErrorTimeout;
    }
    return cudaSuccess;
}

// Timed advance on the module stream; waits for completion.
cudaError_t advance_sync(const GpuKinLaunch *L, const GpuKinTuning &t, float *kernel_ms) {
    cudaError_t e = check_launch(L);
    if (e != cudaSuccess) return e;
    DevArgs A;
    fill_args(L, &A);
    cudaEventRecord(g.kin_start, g.stream);
    e = launch_advance(L->precision, t, A);
    cudaEventRecord(g.kin_stop, g.stream);
    if (e != cudaSuccess) return e;
    e = cudaEventSynchronize(g.kin_stop);
    if (e != cudaSuccess) return e;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, g.kin_start, g.kin_stop);
    g.last_ms = ms;
    ++g.launches;
    if (kernel_ms) *kernel_ms = ms;
    e = read_error_flag();
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}   // namespace

// ===========================================================================
// The reference's exports (src/gpu/gpu_api.h:46-115).

SGB_API int32_t gpu_init(uint32_t device_index, uint64_t arena_bytes, GpuInfo *info) {
    memset(info, 0, sizeof(*info));
    cudaError_t e = cudaSetDevice((int)device_index);
    if (e != cudaSuccess) return (int32_t)e;
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, (int)device_index);
    if (e != cudaSuccess) return (int32_t)e;
    snprintf(info->name, sizeof(info->name), "%s", prop.name);
    info->sm_major = (uint32_t)prop.major;
    info->sm_minor = (uint32_t)prop.minor;
    info->multiprocessors = (uint32_t)prop.multiProcessorCount;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    info->free_bytes = free_b;
    info->total_bytes = total_b;
    if (g.ready) {   // re-init: release the previous arena and scratch
        cudaDeviceSynchronize();
        cudaFree(g.arena);
        cudaFree(g.d_tables);
        cudaFree(g.d_cursor);
        if (g.d_dbd_scratch) cudaFree(g.d_dbd_scratch);
        g.d_dbd_scratch = nullptr;
        g.dbd_scratch_bytes = 0;
        g.arena = nullptr;
        g.d_tables = nullptr;
        g.d_cursor = nullptr;
        g.ready = false;
    }
    void *base = nullptr;
    if (arena_bytes) {
        e = cudaMalloc(&base, arena_bytes);
        if (e != cudaSuccess) return (int32_t)e;
    }
    g.arena = (uint8_t *)base;
    g.arena_size = arena_bytes;
    g.arena_used = 0;
    info->arena_bytes = arena_bytes;
    e = cudaMalloc(&g.d_tables, kTableBytes);
    if (e != cudaSuccess) return (int32_t)e;
    // cursor at +0, error flag at +128, the pipelined advance's per-chunk cursors from +256 (128 B apart)
    const size_t cursor_bytes = 256 + (size_t)Module::kMaxChunks * 128;
    e = cudaMalloc((void **)&g.d_cursor, cursor_bytes);
    if (e != cudaSuccess) return (int32_t)e;
    g.d_error = (uint32_t *)((uint8_t *)g.d_cursor + 128);
    cudaMemset(g.d_cursor, 0, cursor_bytes);
    if (!g.d_suspend) {
        e = cudaMalloc((void **)&g.d_suspend, (size_t)kSuspendCap * sizeof(SuspendRec) + 256);
        if (e != cudaSuccess) return (int32_t)e;
        g.d_suspend_count = (uint32_t *)((uint8_t *)g.d_suspend + (size_t)kSuspendCap * sizeof(SuspendRec));
    }
    if (!g.stream) {
        cudaEventCreate(&g.kin_start);
        cudaEventCreate(&g.kin_stop);
        cudaEventCreate(&g.async_begin);
        cudaEventCreate(&g.async_end);
        cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking);
    }
    size_t stack = 0;
    if (cudaDeviceGetLimit(&stack, cudaLimitStackSize) == cudaSuccess && stack != kStackReserveBytes) {
        e = cudaDeviceSetLimit(cudaLimitStackSize, kStackReserveBytes);
        if (e != cudaSuccess) return (int32_t)e;
    }
    g.device = (int)device_index;
    g.sms = prop.multiProcessorCount;
    for (int p = 0; p < 3; ++p) g.tuning[p] = kDefaultTuning;
    g.have_mech = false;
    g.ready = true;
    return (int32_t)cudaGetLastError();
}

SGB_API const char *gpu_error_string(int32_t error) { return cudaGetErrorString((cudaError_t)error); }

SGB_API void *gpu_alloc(uint64_t size) {
    uint64_t aligned = (size + 255) & ~255ull;
    if (!g.arena || g.arena_used + aligned > g.arena_size) return nullptr;
    void *p = g.arena + g.arena_used;
    g.arena_used += aligned;
    return p;
}

SGB_API uint64_t gpu_arena_used(void) { return g.arena_used; }

SGB_API void gpu_arena_reset(void) {
    cudaDeviceSynchronize();
    g.arena_used = 0;
}

SGB_API int32_t gpu_copy_to_device(void *dst_device, const void *src_host, uint64_t size) {
    cudaError_t e = cudaMemcpyAsync(dst_device, src_host, size, cudaMemcpyHostToDevice, g.stream);
    if (e != cudaSuccess) return (int32_t)e;
    return (int32_t)cudaStreamSynchronize(g.stream);
}

SGB_API int32_t gpu_copy_to_host(void *dst_host, const void *src_device, uint64_t size) {
    cudaError_t e = cudaMemcpyAsync(dst_host, src_device, size, cudaMemcpyDeviceToHost, g.stream);
    if (e != cudaSuccess) return (int32_t)e;
    return (int32_t)cudaStreamSynchronize(g.stream);
}

SGB_API int32_t gpu_sync(void) { return (int32_t)cudaStreamSynchronize(g.stream); }

namespace {
// The loader's demo entry point: each point falls toward the origin under a
// softened inverse-square pull, a = -x / (|x|^2 + eps^2)^(3/2), advanced by one
// kick-drift-kick leapfrog step of dt (time-reversible, so orbits neither
// gain nor lose energy over many calls).
__device__ __forceinline__ void pull(float px, float py, float pz, float &ax, float &ay, float &az) {
    const float eps2 = 0.01f;
    const float r2 = fmaf(px, px, fmaf(py, py, fmaf(pz, pz, eps2)));
    const float inv_r = rsqrtf(r2);
    const float s = -(inv_r * inv_r * inv_r);
    ax = s * px;
    ay = s * py;
    az = s * pz;
}
__global__ void step_points_kernel(float *x, float *y, float *z, float *vx, float *vy, float *vz, uint32_t count, float dt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float half = 0.5f * dt;
    float px = x[i], py = y[i], pz = z[i], ax, ay, az;
    pull(px, py, pz, ax, ay, az);
    float ux = fmaf(ax, half, vx[i]), uy = fmaf(ay, half, vy[i]), uz = fmaf(az, half, vz[i]);
    px = fmaf(ux, dt, px);
    py = fmaf(uy, dt, py);
    pz = fmaf(uz, dt, pz);
    pull(px, py, pz, ax, ay, az);
    x[i] = px;
    y[i] = py;
    z[i] = pz;
    vx[i] = fmaf(ax, half, ux);
    vy[i] = fmaf(ay, half, uy);
    vz[i] = fmaf(az, half, uz);
}
}   // namespace

SGB_API int32_t gpu_step_points(float *x, float *y, float *z, float *vx, float *vy, float *vz, uint32_t count, float dt) {
    if (count == 0) return 0;
    step_points_kernel<<<(count + 255) / 256, 256, 0, g.stream>>>(x, y, z, vx, vy, vz, count, dt);
    return (int32_t)cudaGetLastError();
}

SGB_API int32_t gpu_kin_set_mech(const KinMech *mech, const KinMethod *method, const KinControl *control) {
    if (!g.ready) return (int32_t)cudaErrorInitializationError;
    if (!mech || !method || !control) return (int32_t)cudaErrorInvalidValue;
    // every table index must stay inside the tables (the kernels do not re-check)
    if (!mech_tables_valid(mech, method)) return (int32_t)cudaErrorInvalidValue;
    static unsigned char image[kTableBytes];
    table_image(mech, image);
    cudaError_t e = cudaMemcpyAsync(g.d_tables, image, kTableBytes, cudaMemcpyHostToDevice, g.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.stream);
    if (e != cudaSuccess) return (int32_t)e;
    g.mech = *mech;
    g.method = *method;
    g.control = *control;
    g.generated = fnv1a(mech, sizeof(KinMech)) == air_ops_signature() && method_is_rodas3(method);
    g.have_mech = true;
    // the cooperative image of the same mechanism, for the straggler hand-off (none: no hand-off)
    if (g.d_coop_image) cudaFree(g.d_coop_image);
    if (g.d_coop_scratch) cudaFree(g.d_coop_scratch);
    g.d_coop_image = nullptr;
    g.d_coop_scratch = nullptr;
    std::vector<uint8_t> coop;
    if (coop_image(*mech, &coop)) {
        memcpy(&g.coop_head, coop.data(), sizeof(CoopMech));
        g.coop_grid = (uint32_t)g.sms * kResumeCtasPerSm;
        const size_t a = coop_scratch_doubles_for(0, g.coop_head), b = coop_scratch_doubles_for(2, g.coop_head);
        e = cudaMalloc(&g.d_coop_image, coop.size());
        if (e == cudaSuccess) e = cudaMemcpy(g.d_coop_image, coop.data(), coop.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc((void **)&g.d_coop_scratch, (a > b ? a : b) * 8 * g.coop_grid);
        if (e != cudaSuccess) {
            if (g.d_coop_image) cudaFree(g.d_coop_image);
            g.d_coop_image = nullptr;
            return (int32_t)e;
        }
    }
    return 0;
}

// The tuning an advance of precision p runs: mode 1 (the reference's warp per cell) is the
// cooperative decomposition with one warp per cell for FP64 and mixed; f32 lanes keep one thread
// per cell in either mode.
GpuKinTuning tuning_for(uint32_t p) {
    GpuKinTuning t = g.tuning[p];
    if (g.mode == 1 && p != 1 && t.kind != 3) {
        t.kind = 3;
        t.block = 32;
        t.chunk = 0;
    }
    return t;
}

SGB_API int32_t gpu_kin_advance(const GpuKinLaunch *launch, float *kernel_ms) {
    uint32_t p = launch ? launch->precision : 0;
    if (p > 2) return (int32_t)cudaErrorInvalidValue;
    return (int32_t)advance_sync(launch, tuning_for(p), kernel_ms);
}

SGB_API int32_t gpu_host_register(void *host, uint64_t size) {
    cudaError_t e = cudaHostRegister(host, size, cudaHostRegisterDefault);
    if (e == cudaErrorHostMemoryAlreadyRegistered) {
        cudaGetLastError();
        return 0;
    }
    return (int32_t)e;
}

SGB_API int32_t gpu_host_unregister(void *host) {
    cudaStreamSynchronize(g.stream);
    return (int32_t)cudaHostUnregister(host);
}

SGB_API int32_t gpu_kin_advance_async(const GpuKinLaunch *launch, void *host_block, void *device_block, uint64_t rows,
                                      uint64_t mutable_rows) {
    cudaError_t e = check_launch(launch);
    if (e != cudaSuccess) return (int32_t)e;
    if (!host_block || !device_block || mutable_rows > rows) return (int32_t)cudaErrorInvalidValue;
    const uint64_t pitch = (uint64_t)launch->padded * sizeof(double);
    const uint64_t width = (uint64_t)(launch->lane_count ? launch->lane_count : launch->padded) * sizeof(double);
    cudaEventRecord(g.async_begin, g.stream);
    e = cudaMemcpy2DAsync(device_block, pitch, host_block, pitch, width, rows, cudaMemcpyHostToDevice, g.stream);
    if (e != cudaSuccess) return (int32_t)e;
    DevArgs A;
    fill_args(launch, &A);
    cudaEventRecord(g.kin_start, g.stream);
    e = launch_advance(launch->precision, tuning_for(launch->precision), A);
    cudaEventRecord(g.kin_stop, g.stream);
    if (e != cudaSuccess) return (int32_t)e;
    e = cudaMemcpy2DAsync(host_block, pitch, device_block, pitch, width, mutable_rows, cudaMemcpyDeviceToHost, g.stream);
    if (e != cudaSuccess) return (int32_t)e;
    cudaEventRecord(g.async_end, g.stream);
    return (int32_t)cudaGetLastError();
}

// The same work as gpu_kin_advance_async + gpu_kin_wait, with lanes [0, lane_count) split into
// `chunks` column ranges whose uploads, kernels and downloads overlap: chunk c+1 uploads on one
// stream while chunk c integrates and chunk c-1 downloads on another. Each chunk's kernel is a
// full advance of its lanes (same results per cell). Chunk kernels alternate between two kernel
// streams, each queue kernel with its own cursor, so chunk c+1's CTAs take the SMs that chunk
// c's last cells leave idle; the kernels never wait on one another. With the FP64 straggler
// hand-off on (it shares one suspension list) the chunk kernels run in order on the module
// stream. Waits; total_ms is the time on the device from the first upload to the last download.
SGB_API int32_t gpu_kin_advance_pipelined(const GpuKinLaunch *launch, void *host_block, void *device_block, uint64_t rows,
                                          uint64_t mutable_rows, uint32_t chunks, float *total_ms) {
    cudaError_t e = check_launch(launch);
    if (e != cudaSuccess) return (int32_t)e;
    if (!host_block || !device_block || mutable_rows > rows || chunks == 0 || chunks > (uint32_t)Module::kMaxChunks)
        return (int32_t)cudaErrorInvalidValue;
    if (!g.copy_in) {
        e = cudaStreamCreateWithFlags(&g.copy_in, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g.copy_out, cudaStreamNonBlocking);
        for (int c = 0; c < Module::kMaxChunks && e == cudaSuccess; ++c) {
            e = cudaEventCreateWithFlags(&g.ev_in[c], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g.ev_kern[c], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreate(&g.pipe_begin);
        if (e == cudaSuccess) e = cudaEventCreate(&g.pipe_end);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g.pipe_after, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g.kern2, cudaStreamNonBlocking);
        if (e != cudaSuccess) return (int32_t)e;
    }
    const bool serial = g.straggler_budget && g.d_coop_image && launch->precision == 0;
    const uint64_t P = launch->padded, lanes = launch->lane_count ? launch->lane_count : launch->padded;
    const uint64_t pitch = P * sizeof(double);
    const uint64_t per = (lanes + chunks - 1) / chunks;
    uint8_t *hb = (uint8_t *)host_block, *db = (uint8_t *)device_block;
    // everything already queued on the module stream (an earlier async advance) comes first
    e = cudaEventRecord(g.pipe_after, g.stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(g.copy_in, g.pipe_after, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(g.kern2, g.pipe_after, 0);
    if (e == cudaSuccess) e = cudaEventRecord(g.pipe_begin, g.copy_in);
    for (uint32_t c = 0; c < chunks && e == cudaSuccess; ++c) {
        const uint64_t first = (uint64_t)c * per, count = first < lanes ? (lanes - first < per ? lanes - first : per) : 0;
        if (count == 0) break;
        cudaStream_t ks = serial || (c & 1) == 0 ? g.stream : g.kern2;
        e = cudaMemcpy2DAsync(db + first * 8, pitch, hb + first * 8, pitch, count * 8, rows, cudaMemcpyHostToDevice, g.copy_in);
        if (e == cudaSuccess) e = cudaEventRecord(g.ev_in[c], g.copy_in);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ks, g.ev_in[c], 0);
        if (e != cudaSuccess) break;
        GpuKinLaunch Lc = *launch;   // the chunk: every row pointer moved to its first lane
        double **rowp[12] = {&Lc.y, &Lc.h, &Lc.steps, &Lc.rejects, &Lc.pulses, &Lc.failed,
                             &Lc.k, &Lc.src, &Lc.pulse, &Lc.period, &Lc.pulse_first, &Lc.pulse_count};
        for (double **r : rowp) *r += first;
        Lc.lane_count = (uint32_t)count;
        DevArgs A;
        fill_args(&Lc, &A);
        if (serial) {
            e = launch_advance(launch->precision, g.tuning[launch->precision], A);
        } else {
            A.cursor = (uint32_t *)((uint8_t *)g.d_cursor + 256 + (size_t)c * 128);
            e = launch_lanes(launch->precision, g.tuning[launch->precision], A, ks);
        }
        if (e == cudaSuccess) e = cudaEventRecord(g.ev_kern[c], ks);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(g.copy_out, g.ev_kern[c], 0);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(hb + first * 8, pitch, db + first * 8, pitch, count * 8, mutable_rows, cudaMemcpyDeviceToHost,
                                  g.copy_out);
    }
    if (e == cudaSuccess) e = cudaEventRecord(g.pipe_end, g.copy_out);
    if (e == cudaSuccess) e = cudaEventSynchronize(g.pipe_end);
    if (e != cudaSuccess) {   // nothing may still be copying into the caller's block when it gets the error
        cudaStreamSynchronize(g.copy_in);
        cudaStreamSynchronize(g.stream);
        cudaStreamSynchronize(g.kern2);
        cudaStreamSynchronize(g.copy_out);
        return (int32_t)e;
    }
    if (total_ms) cudaEventElapsedTime(total_ms, g.pipe_begin, g.pipe_end);
    ++g.launches;
    e = read_error_flag();
    if (e != cudaSuccess) return (int32_t)e;
    return (int32_t)cudaGetLastError();
}

SGB_API int32_t gpu_kin_wait(float *kernel_ms, float *total_ms) {
    cudaError_t e = cudaEventSynchronize(g.async_end);
    if (e != cudaSuccess) return (int32_t)e;
    if (kernel_ms) cudaEventElapsedTime(kernel_ms, g.kin_start, g.kin_stop);
    if (total_ms) cudaEventElapsedTime(total_ms, g.async_begin, g.async_end);
    ++g.launches;
    e = read_error_flag();
    if (e != cudaSuccess) return (int32_t)e;
    return (int32_t)cudaGetLastError();
}

// Mode 1 (one warp per cell, gpu_api.h:108-110): FP64 and mixed advances run the cooperative
// kernel with 32 threads per cell (FP64: the same bits as one thread per cell). Needs a
// mechanism whose cooperative image could be built (any KinMech).
SGB_API int32_t gpu_kin_set_mode(uint32_t mode) {
    if (mode > 1) return (int32_t)cudaErrorInvalidValue;
    g.mode = mode;
    return 0;
}

// ===========================================================================
// Extra exports.

SGB_API int32_t gpu_kin_advance_queue(const GpuKinLaunch *launch, float *kernel_ms) {
    uint32_t p = launch ? launch->precision : 0;
    if (p > 2) return (int32_t)cudaErrorInvalidValue;
    GpuKinTuning t = g.tuning[p];
    if (t.kind == 0) {   // a static tuning: run the CTA-synchronous queue at its default shape
        t.kind = 2;
        t.block = 128;
        t.variant = 0;
        t.chunk = 0;
    }
    return (int32_t)advance_sync(launch, t, kernel_ms);
}

SGB_API int32_t gpu_kin_set_tuning(const GpuKinTuning *t) {
    if (!t || t->kind > 3 || t->block == 0 || (t->block & 31) || t->variant > 3 || t->chunk > 64) return (int32_t)cudaErrorInvalidValue;
    if (t->kind == 3) {   // cooperative: 32..256 threads per cell
        if (t->block > 256) return (int32_t)cudaErrorInvalidValue;
        for (int p = 0; p < 3; ++p) g.tuning[p] = *t;
        return 0;
    }
    const uint32_t max_block = t->variant == 3 ? 512u : t->variant == 2 ? 256u : 128u;   // the variant's __launch_bounds__
    if (t->block > max_block || (t->variant >= 2 && t->kind != 2)) return (int32_t)cudaErrorInvalidValue;
    for (int p = 0; p < 3; ++p) g.tuning[p] = *t;
    return 0;
}

SGB_API int32_t gpu_kin_get_tuning(uint32_t precision, GpuKinTuning *t) {
    if (precision > 2 || !t) return (int32_t)cudaErrorInvalidValue;
    *t = g.tuning[precision];
    return 0;
}

// Times every (block, variant) candidate of `kind` on the caller's launch and
// keeps the fastest for that precision. The solver-written arrays are saved
// before and restored after each run, so the caller's data is unchanged.
SGB_API int32_t gpu_kin_autotune(const GpuKinLaunch *launch, uint32_t kind, GpuKinTuning *best) {
    cudaError_t e = check_launch(launch);
    if (e != cudaSuccess) return (int32_t)e;
    if (kind > 4 || ((kind == 3 || kind == 4) && (!g.d_coop_image || launch->precision == 1))) return (int32_t)cudaErrorInvalidValue;
    const uint64_t P = launch->padded, n = g.mech.species_count;
    const uint64_t bytes_y = n * P * sizeof(double), bytes_v = P * sizeof(double);
    double *save = nullptr;
    e = cudaMalloc(&save, bytes_y + 5 * bytes_v);
    if (e != cudaSuccess) return (int32_t)e;
    double *outs[6] = {launch->y, launch->h, launch->steps, launch->rejects, launch->pulses, launch->failed};
    uint64_t sizes[6] = {bytes_y, bytes_v, bytes_v, bytes_v, bytes_v, bytes_v};
    auto copy_all = [&](bool to_save) {
        uint64_t off = 0;
        for (int i = 0; i < 6; ++i) {
            uint8_t *s = (uint8_t *)save + off;
            if (to_save) cudaMemcpyAsync(s, outs[i], sizes[i], cudaMemcpyDeviceToDevice, g.stream);
            else cudaMemcpyAsync(outs[i], s, sizes[i], cudaMemcpyDeviceToDevice, g.stream);
            off += sizes[i];
        }
    };
    copy_all(true);
    // candidates: block size x register budget x resident CTAs per SM (lane kernels); threads per
    // cell x CTAs per SM (cooperative kernel: cells per warp 1, 1/2, 1/4, 1/8); kind 4 = all of
    // kind 2's and kind 3's, so the cells-per-warp decomposition is chosen by measurement too
    struct Cand { uint32_t kind, block, variant, ctas; };
    const Cand cands[] = {{1, 32, 0, 0}, {1, 64, 0, 0}, {1, 128, 0, 0}, {1, 64, 1, 0}, {1, 128, 1, 0},
                          {1, 128, 0, 1}, {1, 64, 0, 2}, {1, 64, 0, 3}, {1, 128, 1, 2}, {1, 128, 1, 3}};
    const Cand sync_cands[] = {{2, 128, 0, 2}, {2, 256, 2, 1}, {2, 128, 0, 1}, {2, 128, 1, 4}, {2, 512, 3, 1}};
    const Cand coop_cands[] = {{3, 32, 0, 8}, {3, 64, 0, 4}, {3, 128, 0, 2}, {3, 256, 0, 1}};
    std::vector<Cand> list;
    if (kind == 0 || kind == 1)
        for (const Cand &c : cands)
            if (kind == 1 || c.ctas == 0) list.push_back(Cand{kind, c.block, c.variant, c.ctas});
    if (kind == 2 || kind == 4) list.insert(list.end(), std::begin(sync_cands), std::end(sync_cands));
    if (kind == 3 || kind == 4) list.insert(list.end(), std::begin(coop_cands), std::end(coop_cands));
    GpuKinTuning winner = g.tuning[launch->precision];
    winner.ms = 1e30f;
    // candidates that would grow the context's stack reservation are skipped, unless none fits
    size_t have = 0, least = (size_t)-1;
    cudaDeviceGetLimit(&have, cudaLimitStackSize);
    for (const Cand &c : list) {
        GpuKinTuning t = {c.kind, c.block, c.ctas, c.variant, 0.0f};
        size_t need = 0;
        if (local_bytes(launch->precision, t, &need) == cudaSuccess && need < least) least = need;
    }
    const bool keep_reservation = least <= have;
    for (const Cand &c : list) {
        if (e != cudaSuccess) break;
        GpuKinTuning t = {c.kind, c.block, c.ctas, c.variant, 0.0f};
        size_t need = 0;
        if (keep_reservation && local_bytes(launch->precision, t, &need) == cudaSuccess && need > have) continue;
        float ms = 0.0f, best_ms = 1e30f;
        for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {   // the faster of two runs
            e = advance_sync(launch, t, &ms);
            copy_all(false);
            if (ms < best_ms) best_ms = ms;
        }
        if (e != cudaSuccess) break;
        if (best_ms < winner.ms) {
            winner = t;
            winner.ms = best_ms;
        }
    }
    cudaStreamSynchronize(g.stream);
    cudaFree(save);
    if (e != cudaSuccess) return (int32_t)e;
    g.tuning[launch->precision] = winner;
    if (best) *best = winner;
    return 0;
}

SGB_API int32_t gpu_kin_last_stats(uint64_t *kernel_launches, float *last_kernel_ms) {
    if (kernel_launches) *kernel_launches = g.launches;
    if (last_kernel_ms) *last_kernel_ms = g.last_ms;
    return 0;
}

// Mixed path refinement sweeps per stage solve (1 or 2).
SGB_API int32_t gpu_kin_set_refinement(uint32_t sweeps) {
    if (sweeps < 1 || sweeps > 2) return (int32_t)cudaErrorInvalidValue;
    g.ir_sweeps = sweeps;
    return 0;
}

// Per-thread stack (local memory) reservation of the context: it grows to the largest
// frame any launched kernel needs and stays there; a launch needing more grows it again.
SGB_API int32_t gpu_stack_limit(uint64_t set_bytes, uint64_t *current) {
    cudaError_t e = cudaSuccess;
    if (set_bytes) e = cudaDeviceSetLimit(cudaLimitStackSize, (size_t)set_bytes);
    size_t v = 0;
    if (e == cudaSuccess && current) e = cudaDeviceGetLimit(&v, cudaLimitStackSize);
    if (current) *current = v;
    return (int32_t)e;
}

SGB_API int32_t gpu_kin_set_straggler_budget(uint32_t attempts) {
    g.straggler_budget = attempts;
    return 0;
}

SGB_API int32_t gpu_kin_set_straggler_block(uint32_t threads) {
    if (threads < 32 || threads > 256 || (threads & 31)) return (int32_t)cudaErrorInvalidValue;
    g.straggler_block = threads;
    return 0;
}

SGB_API int32_t gpu_kin_parked_cells(uint32_t *count) {
    if (!g.ready || !count) return (int32_t)cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyAsync(count, g.d_suspend_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, g.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.stream);
    return (int32_t)e;
}

SGB_API int32_t gpu_kin_set_mixed_variant(uint32_t variant) {
    if (variant > 2) return (int32_t)cudaErrorInvalidValue;
    g.mixed_variant = variant;
    return 0;
}

SGB_API uint32_t gpu_kin_get_mixed_variant(void) { return g.mixed_variant; }

SGB_API int32_t gpu_kin_set_wait_limit(uint32_t polls) {
    g.wait_polls = polls;
    return 0;
}

namespace sgb {
// Module settings read by the allocation-free advance (which needs no gpu_init).
uint32_t module_wait_polls() { return g.wait_polls; }
uint32_t module_ir_sweeps() { return g.ir_sweeps; }

// For the device zone driver (dbd_driver.cu): the advance enqueued on the module stream at
// the precision's tuning (what gpu_kin_advance runs), bracketed by the module's timing events.
cudaStream_t module_stream() { return g.stream; }
cudaError_t module_enqueue_advance(const GpuKinLaunch *L) {
    cudaError_t e = check_launch(L);
    if (e != cudaSuccess) return e;
    DevArgs A;
    fill_args(L, &A);
    return launch_advance(L->precision, g.tuning[L->precision], A);
}
cudaError_t module_mark_start() {
    if (!g.ready) return cudaErrorInitializationError;
    return cudaEventRecord(g.kin_start, g.stream);
}
cudaError_t module_finish(float *device_ms) {
    cudaError_t e = cudaEventRecord(g.kin_stop, g.stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(g.kin_stop);
    if (e != cudaSuccess) return e;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, g.kin_start, g.kin_stop);
    g.last_ms = ms;
    ++g.launches;
    if (device_ms) *device_ms = ms;
    e = read_error_flag();
    return e != cudaSuccess ? e : cudaGetLastError();
}
// Module-owned scratch of at least `bytes`, grown (after the stream drains) when too small.
cudaError_t module_scratch(size_t bytes, void **out) {
    if (!g.ready) return cudaErrorInitializationError;
    if (g.dbd_scratch_bytes < bytes) {
        cudaError_t e = cudaStreamSynchronize(g.stream);
        if (e != cudaSuccess) return e;
        if (g.d_dbd_scratch) cudaFree(g.d_dbd_scratch);
        g.d_dbd_scratch = nullptr;
        g.dbd_scratch_bytes = 0;
        e = cudaMalloc(&g.d_dbd_scratch, bytes);
        if (e != cudaSuccess) return e;
        g.dbd_scratch_bytes = bytes;
    }
    *out = g.d_dbd_scratch;
    return cudaSuccess;
}
}   // namespace sgb

// Measured instruction throughput (operations per second over the device):
// kind 0 DFMA, 1 FFMA, 2 FP32<->FP64 conversion pairs, 3 DADD, 4 FP64 reciprocal, 5 FP64 sqrt.
SGB_API int32_t gpu_probe_throughput(uint32_t kind, double *ops_per_s) {
    if (!g.ready || !ops_per_s || kind > 5) return (int32_t)cudaErrorInvalidValue;
    return (int32_t)run_probe(kind, g.sms, g.stream, ops_per_s);
}

// Device-to-device copy enqueued on the module stream (returns without waiting).
SGB_API int32_t gpu_copy_on_device(void *dst_device, const void *src_device, uint64_t size) {
    return (int32_t)cudaMemcpyAsync(dst_device, src_device, size, cudaMemcpyDeviceToDevice, g.stream);
}

// The module stream, for callers that order their own work against it.
SGB_API void *gpu_stream(void) { return (void *)g.stream; }
