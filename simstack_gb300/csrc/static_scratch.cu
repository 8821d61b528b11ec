// gpu_kin_advance_noalloc: the persistent work-queue advance for callers that
// cannot allocate device memory.
//
// Who needs it: a caller that owns all device memory through its own arena
// (SimStack's platform layer hands the simulation one fixed block and never
// allocates again), or a caller on a real-time loop that may not take
// cudaMalloc's implicit device-wide synchronisation. gpu_init allocates the
// module's arena and scratch, so such callers cannot use the regular entry
// points; this one needs no gpu_init.
//
// What it uses instead: the queue kernel's scratch -- the work-queue cursor,
// the bounded-wait error flag and, for mechanisms without generated code, the
// staged copy of the mechanism tables -- lives in g_kin_static_scratch below,
// a file-scope device array of kStaticScratchBytes (32 KiB) that every GPU
// holds from the moment the library is loaded until the process exits. The
// kernel is the one gpu_kin_advance_queue launches at the module's default
// launch shape (the CTA-synchronous persistent queue, 128 threads per CTA),
// with the module's mixed-path variant and refinement setting; only where its
// scratch lives differs. Inputs and outputs are the caller's zone block, as
// for every other advance.
//
// Local memory: the context's per-thread stack reservation (cudaLimitStackSize)
// must already cover the kernel's frame, since a launch that needs more makes
// the driver grow the reservation -- a device allocation. gpu_init fixes it
// once; a caller without gpu_init sets it with gpu_stack_limit at set-up. The
// entry point checks it and returns cudaErrorLaunchOutOfResources otherwise.

#include <cuda_runtime.h>
#include <string.h>

#include "../../include/simstack_gpu.h"
#include "kin_kernels.cuh"
#include "kin_table.cuh"
#include "mech.h"
#include "mech_tables.h"

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
cudaError_t local_air_p0(uint32_t, uint32_t, size_t *);
cudaError_t local_air_p1(uint32_t, uint32_t, size_t *);
cudaError_t local_air_p2(uint32_t, uint32_t, size_t *);
cudaError_t local_air_p3(uint32_t, uint32_t, size_t *);
cudaError_t local_table_p0(uint32_t, size_t *);
cudaError_t local_table_p1(uint32_t, size_t *);
cudaError_t local_table_p2(uint32_t, size_t *);
cudaError_t local_table_p3(uint32_t, size_t *);
cudaError_t local_air_p4(uint32_t, uint32_t, size_t *);
cudaError_t local_table_p4(uint32_t, size_t *);
uint64_t air_ops_signature();
uint32_t module_wait_polls();
uint32_t module_ir_sweeps();
}   // namespace sgb

using namespace sgb;

namespace {

// Layout: queue cursor at +0, error flag at +128 (separate 128-byte lines),
// mechanism table image (table-driven kernels only) at +256.
constexpr uint32_t kStaticScratchBytes = 32768;
constexpr uint32_t kQueueHeaderBytes = 256;
static_assert(kQueueHeaderBytes + kTableBytes <= kStaticScratchBytes, "table image must fit the static scratch");

static __device__ __align__(256) unsigned char g_kin_static_scratch[kStaticScratchBytes];

// Device address of g_kin_static_scratch per device ordinal, looked up once
// per device with that device current (the array's name in host code is only
// a host-side stand-in and must never be passed to a kernel).
constexpr int kMaxDevices = 64;
unsigned char *g_scratch_ptr[kMaxDevices];

cudaError_t scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_kin_static_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = (unsigned char *)p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}   // namespace

// Advances lanes [0, lane_count) of a zone block with the persistent work-queue
// kernel, allocating no device memory. See include/simstack_gpu.h.
SGB_API int32_t gpu_kin_advance_noalloc(const KinMech *mech, const KinMethod *method, const KinControl *control,
                                        const GpuKinLaunch *L, void *stream, int32_t wait) {
    if (!mech || !method || !control || !L) return (int32_t)cudaErrorInvalidValue;
    if (L->precision > 2 || L->padded == 0 || L->lane_count > L->padded) return (int32_t)cudaErrorInvalidValue;
    if (!(L->duration >= 0.0) || L->duration > 1.0e300) return (int32_t)cudaErrorInvalidValue;
    if (!L->y || !L->h || !L->steps || !L->rejects || !L->pulses || !L->failed || !L->k || !L->src || !L->pulse ||
        !L->period || !L->pulse_first || !L->pulse_count)
        return (int32_t)cudaErrorInvalidValue;
    if (!mech_tables_valid(mech, method)) return (int32_t)cudaErrorInvalidValue;
    const bool generated = fnv1a(mech, sizeof(KinMech)) == air_ops_signature() && method_is_rodas3(method);

    // scratch this call needs: the queue header, plus the table image for the table-driven kernels
    const uint64_t needed = kQueueHeaderBytes + (generated ? 0u : kTableBytes);
    if (needed > kStaticScratchBytes) return (int32_t)cudaErrorMemoryAllocation;   // needs more than the static array holds

    unsigned char *scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) return (int32_t)e;
    cudaStream_t s = (cudaStream_t)stream;

    // the cursor and the error flag must start at zero; the array keeps the last call's contents
    e = cudaMemsetAsync(scratch, 0, kQueueHeaderBytes, s);
    if (e != cudaSuccess) return (int32_t)e;
    if (!generated) {
        // copied on every call from a per-host-thread image in pageable memory (the runtime has
        // consumed it by the time cudaMemcpyAsync returns)
        static thread_local unsigned char image[kTableBytes];
        table_image(mech, image);
        e = cudaMemcpyAsync(scratch + kQueueHeaderBytes, image, kTableBytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return (int32_t)e;
    }

    DevArgs A;
    memset(&A, 0, sizeof(A));
    A.y = L->y; A.h = L->h; A.steps = L->steps; A.rejects = L->rejects; A.pulses = L->pulses; A.failed = L->failed;
    A.k = L->k; A.src = L->src; A.pulse = L->pulse; A.period = L->period;
    A.pulse_first = L->pulse_first; A.pulse_count = L->pulse_count;
    A.padded = L->padded;
    A.lanes = L->lane_count ? L->lane_count : L->padded;
    A.duration = L->duration;
    A.ctl = *control;
    memcpy(A.ma, method->a, sizeof(A.ma));
    memcpy(A.mc, method->c, sizeof(A.mc));
    memcpy(A.mm, method->m, sizeof(A.mm));
    memcpy(A.me, method->e, sizeof(A.me));
    A.gamma0 = method->gamma0;
    memcpy(A.new_f, method->new_f, sizeof(A.new_f));
    A.stages = method->stages;
    A.order = method->order;
    A.ir_sweeps = module_ir_sweeps();
    A.cursor = (uint32_t *)scratch;
    A.error_flag = (uint32_t *)(scratch + 128);
    A.wait_polls = module_wait_polls();
    A.tables = scratch + kQueueHeaderBytes;
    A.table_bytes = kTableBytes;
    if (A.lanes == 0) return 0;

    // the module's default launch shape: CTA-synchronous persistent queue, 128 threads, 255 registers
    const uint32_t kind = 2, variant = 0;
    // precision 2 runs the module's current mixed variant (gpu_kin_set_mixed_variant): lane code
    // 0 FP64, 1 f32 Delta, 2 FP64-state refinement, 3 double-float state, 4 double-float refined
    const uint32_t mv = gpu_kin_get_mixed_variant();
    const uint32_t p = L->precision == 2 ? (mv == 0 ? 2u : mv == 1 ? 3u : 4u) : L->precision;
    size_t frame = 0, reserved = 0;
    if (generated) e = p == 0 ? local_air_p0(kind, variant, &frame) : p == 1 ? local_air_p1(kind, variant, &frame)
                       : p == 2 ? local_air_p2(kind, variant, &frame) : p == 3 ? local_air_p3(kind, variant, &frame)
                       : local_air_p4(kind, variant, &frame);
    else e = p == 0 ? local_table_p0(kind, &frame) : p == 1 ? local_table_p1(kind, &frame)
             : p == 2 ? local_table_p2(kind, &frame) : p == 3 ? local_table_p3(kind, &frame) : local_table_p4(kind, &frame);
    if (e == cudaSuccess) e = cudaDeviceGetLimit(&reserved, cudaLimitStackSize);
    if (e != cudaSuccess) return (int32_t)e;
    if (frame > reserved) return (int32_t)cudaErrorLaunchOutOfResources;   // the launch would grow the reservation

    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int32_t)e;
    Shape sh;
    sh.kind = kind;
    sh.block = 128;
    sh.variant = variant;
    sh.smem = generated ? 0 : kTableBytes;
    if (generated) e = p == 0 ? occupancy_air_p0(kind, variant, sh.block, &per_sm) : p == 1 ? occupancy_air_p1(kind, variant, sh.block, &per_sm)
                       : p == 2 ? occupancy_air_p2(kind, variant, sh.block, &per_sm) : p == 3 ? occupancy_air_p3(kind, variant, sh.block, &per_sm)
                       : occupancy_air_p4(kind, variant, sh.block, &per_sm);
    else e = p == 0 ? occupancy_table_p0(kind, sh.block, sh.smem, &per_sm) : p == 1 ? occupancy_table_p1(kind, sh.block, sh.smem, &per_sm)
             : p == 2 ? occupancy_table_p2(kind, sh.block, sh.smem, &per_sm) : p == 3 ? occupancy_table_p3(kind, sh.block, sh.smem, &per_sm)
             : occupancy_table_p4(kind, sh.block, sh.smem, &per_sm);
    if (e != cudaSuccess) return (int32_t)e;
    if (per_sm < 1) per_sm = 1;
    const uint32_t resident = (uint32_t)per_sm * (uint32_t)sms, needed_ctas = (A.lanes + sh.block - 1) / sh.block;
    sh.grid = resident < needed_ctas ? resident : needed_ctas;
    if (generated) e = p == 0 ? launch_air_p0(sh, A, s) : p == 1 ? launch_air_p1(sh, A, s) : p == 2 ? launch_air_p2(sh, A, s)
                       : p == 3 ? launch_air_p3(sh, A, s) : launch_air_p4(sh, A, s);
    else e = p == 0 ? launch_table_p0(sh, A, s) : p == 1 ? launch_table_p1(sh, A, s) : p == 2 ? launch_table_p2(sh, A, s)
             : p == 3 ? launch_table_p3(sh, A, s) : launch_table_p4(sh, A, s);
    if (e != cudaSuccess) return (int32_t)e;
    if (!wait) return 0;
    uint32_t flag = 0;
    e = cudaMemcpyAsync(&flag, scratch + 128, sizeof(flag), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int32_t)e;
    return flag ? (int32_t)cudaErrorTimeout : (int32_t)cudaGetLastError();
}
