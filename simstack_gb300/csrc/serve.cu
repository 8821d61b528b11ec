// Coupled chemistry + film advection, captured as a CUDA graph per request,
// and the serving engine that admits integration requests as device memory
// frees up.
//
// Advection: the NFT film's explicit upwind transport (src/sim/nft.cpp:
// 1066-1079, flux form x_j = x_j + c (x_{j-1} - x_j) as one fma, swept outlet
// to inlet so every cell reads its upstream neighbour's old value; the
// substep count follows the Courant-0.9 rule of nft.cpp:531-536). A request's
// cells are laid out channel after channel (cell = channel * channel_cells +
// j); one CTA owns one (channel, species) row: it loads the row into shared
// memory with coalesced loads, runs every substep there, and writes it back
// once -- 16 bytes of HBM traffic per cell and species per coupling step.
//
// Coupling step (operator split, chemistry first, as dbd_scene.cpp:263-265):
// [cursor reset] -> [chemistry over the request's zone block, 1 s: the
// persistent queue kernel for the shipped or a KinMech table mechanism, the
// cooperative one-CTA-per-cell kernel for a large mechanism] -> [advection].
// Captured once per request into a CUDA graph and replayed every step on the
// request's own stream; each request has its own queue scratch, so requests
// run side by side.
//
// Serving: requests are admitted first-in first-out while their device
// footprint (zone block + queue scratch + tables) fits the HBM budget (set at
// open from the device's free memory); their state stays device-resident across coupling
// steps; the host drives the engine with gpu_serve_progress(), which retires
// finished requests (result copied to host, memory freed), admits waiting
// ones, and launches the next coupling step of every running request whose
// previous step has completed. Several requests' steps are on the GPU at once.

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <chrono>
#include <deque>
#include <map>
#include <vector>

#include "../../include/simstack_gpu.h"
#include "kin_kernels.cuh"
#include "kin_table.cuh"
#include "mech.h"
#include "mech_tables.h"
#include "coop.h"

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
uint64_t air_ops_signature();
size_t coop_smem_bytes_for(int prec, const CoopMech &h);
size_t coop_scratch_doubles_for(int prec, const CoopMech &h);
cudaError_t coop_launch(int prec, const DevArgs &A, const CoopMech &head, double *scratch, uint32_t grid, uint32_t block,
                        cudaStream_t s);
const Model *model_of(const KinModelHandle *h);
}   // namespace sgb

using namespace sgb;

// ---------------------------------------------------------------------------
// Advection kernel

namespace {

constexpr uint32_t kAdvectThreads = 256;
constexpr uint32_t kMaxChannelCells = 4096;   // one row in shared memory: 32 KiB

// grid (channels, species); row (ch, s) = y[s * padded + cell_begin + ch * cc .. + len)
__global__ void __launch_bounds__(kAdvectThreads) advect_kernel(double *__restrict__ y, uint32_t padded, uint32_t cells,
                                                                uint32_t cc, const double *__restrict__ inlet, double courant,
                                                                uint32_t substeps) {
    extern __shared__ __align__(16) double row[];
    const uint32_t ch = blockIdx.x, s = blockIdx.y;
    const uint32_t begin = ch * cc;
    if (begin >= cells) return;
    const uint32_t len = min(cc, cells - begin);
    double *g = y + (size_t)s * padded + begin;
    for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) row[j] = g[j];
    const double up0 = inlet[s];
    __syncthreads();
    constexpr uint32_t kPer = kMaxChannelCells / kAdvectThreads;
    double next[kPer];
    for (uint32_t it = 0; it < substeps; ++it) {
#pragma unroll
        for (uint32_t q = 0; q < kPer; ++q) {
            const uint32_t j = threadIdx.x + q * blockDim.x;
            if (j < len) {
                const double v = row[j];
                const double up = j == 0 ? up0 : row[j - 1];
                next[q] = fma(courant, up - v, v);
            }
        }
        __syncthreads();
#pragma unroll
        for (uint32_t q = 0; q < kPer; ++q) {
            const uint32_t j = threadIdx.x + q * blockDim.x;
            if (j < len) row[j] = next[q];
        }
        __syncthreads();
    }
    for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) g[j] = row[j];
}

}   // namespace

// Upwind advection of `cells` cells (columns [0, cells) of a [species][padded]
// block laid out channel after channel) on the module stream; see serve.cu.
SGB_API int32_t gpu_advect(double *y, uint32_t padded, uint32_t species, uint32_t cells, uint32_t channel_cells,
                           const double *inlet_device, double courant, uint32_t substeps, void *stream) {
    if (!y || !inlet_device || channel_cells == 0 || channel_cells > kMaxChannelCells || cells > padded || species == 0)
        return (int32_t)cudaErrorInvalidValue;
    if (cells == 0 || substeps == 0) return 0;
    const uint32_t channels = (cells + channel_cells - 1) / channel_cells;
    dim3 grid(channels, species);
    advect_kernel<<<grid, kAdvectThreads, channel_cells * sizeof(double), (cudaStream_t)stream>>>(y, padded, cells, channel_cells,
                                                                                                inlet_device, courant, substeps);
    return (int32_t)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Serving engine

namespace {

using Clock = std::chrono::steady_clock;

enum : uint32_t { kWaiting = 0, kRunning = 1, kDone = 2, kFailed = 3, kCancelled = 4 };

struct Request {
    uint64_t id = 0;
    GpuServeRequest desc;
    uint32_t n = 0, R = 0, padded = 0, rows = 0;
    bool generated = true;
    bool coop = false;          // mechanism 2: the cooperative kernels
    std::vector<double> host;   // the zone block until admission, then the result rows
    uint64_t footprint = 0;     // device bytes while running
    double *d_block = nullptr;  // zone block [rows][padded]
    double *d_inlet = nullptr;  // [n] inlet state
    unsigned char *d_scratch = nullptr;   // queue cursor (+0), error flag (+128), table image (+256)
    double *d_coop = nullptr;             // cooperative mechanism: per-CTA LU / Jacobian scratch
    uint32_t coop_grid = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t step_done = nullptr;
    cudaGraphExec_t graph = nullptr;
    uint32_t launched = 0, completed = 0;
    uint32_t state = kWaiting;
    bool cancel = false;
    int32_t error = 0;
    Clock::time_point t_submit, t_admit, t_done;
    double courant = 0.0;
    uint32_t substeps = 1;
};

struct Engine {
    bool open = false;
    uint64_t budget = 0, in_use = 0, peak = 0;
    uint64_t next_id = 1;
    std::deque<Request *> waiting;
    std::vector<Request *> running;
    std::map<uint64_t, Request *> all;
    uint32_t finished = 0;
    uint64_t graph_launches = 0;
    KinMech table_mech;
    KinMethod table_method;
    bool have_table_mech = false;
    void *d_coop_image = nullptr;   // mechanism 2
    CoopMech coop_head;
    KinMethod coop_method;
    KinControl coop_control;        // mechanism 2's step control (its own concentration units)
    bool have_coop = false;
    KinControl control;
    int sms = 0;
};
Engine E;

uint32_t pad8(uint32_t c) { return (c + 7u) / 8u * 8u; }

// p: 0 FP64, 1 f32 Delta, 2 mixed with FP64 refinement, 3 mixed with double-float state,
// 4 mixed with double-float state and refined stages
cudaError_t launch_chem(bool generated, uint32_t p, const Shape &sh, const DevArgs &A, cudaStream_t s) {
    if (generated)
        return p == 0 ? launch_air_p0(sh, A, s) : p == 1 ? launch_air_p1(sh, A, s) : p == 2 ? launch_air_p2(sh, A, s)
               : p == 3 ? launch_air_p3(sh, A, s) : launch_air_p4(sh, A, s);
    return p == 0 ? launch_table_p0(sh, A, s) : p == 1 ? launch_table_p1(sh, A, s) : p == 2 ? launch_table_p2(sh, A, s)
           : p == 3 ? launch_table_p3(sh, A, s) : launch_table_p4(sh, A, s);
}

cudaError_t occupancy_chem(bool generated, uint32_t p, uint32_t block, size_t smem, int *per_sm) {
    if (generated)
        return p == 0 ? occupancy_air_p0(2, 0, block, per_sm) : p == 1 ? occupancy_air_p1(2, 0, block, per_sm)
               : p == 2 ? occupancy_air_p2(2, 0, block, per_sm) : p == 3 ? occupancy_air_p3(2, 0, block, per_sm)
               : occupancy_air_p4(2, 0, block, per_sm);
    return p == 0 ? occupancy_table_p0(2, block, smem, per_sm) : p == 1 ? occupancy_table_p1(2, block, smem, per_sm)
           : p == 2 ? occupancy_table_p2(2, block, smem, per_sm) : p == 3 ? occupancy_table_p3(2, block, smem, per_sm)
           : occupancy_table_p4(2, block, smem, per_sm);
}

// Frees a request's device resources in stream order (no device-wide synchronisation).
void release(Request *r) {
    if (r->graph) cudaGraphExecDestroy(r->graph);
    if (r->stream) {
        if (r->d_block) cudaFreeAsync(r->d_block, r->stream);
        if (r->d_inlet) cudaFreeAsync(r->d_inlet, r->stream);
        if (r->d_scratch) cudaFreeAsync(r->d_scratch, r->stream);
        if (r->d_coop) cudaFreeAsync(r->d_coop, r->stream);
        cudaStreamDestroy(r->stream);
    }
    if (r->step_done) cudaEventDestroy(r->step_done);
    r->graph = nullptr;
    r->stream = nullptr;
    r->step_done = nullptr;
    r->d_block = r->d_inlet = nullptr;
    r->d_scratch = nullptr;
    r->d_coop = nullptr;
}

// Allocates and uploads an admitted request, then captures its coupling step.
cudaError_t admit(Request *r) {
    const GpuServeRequest &q = r->desc;
    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->step_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&r->d_block, r->host.size() * sizeof(double), r->stream);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&r->d_inlet, r->n * sizeof(double), r->stream);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&r->d_scratch, 256 + kTableBytes, r->stream);
    if (e == cudaSuccess && r->coop)
        e = cudaMallocAsync((void **)&r->d_coop,
                            coop_scratch_doubles_for(q.precision, E.coop_head) * sizeof(double) * r->coop_grid, r->stream);
    if (e != cudaSuccess) return e;
    std::vector<double> inlet(r->n);
    for (uint32_t s = 0; s < r->n; ++s) inlet[s] = r->host[(size_t)s * r->padded];   // cell 0's initial state
    e = cudaMemcpyAsync(r->d_block, r->host.data(), r->host.size() * sizeof(double), cudaMemcpyHostToDevice, r->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->d_inlet, inlet.data(), r->n * sizeof(double), cudaMemcpyHostToDevice, r->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->d_scratch, 0, 256, r->stream);   // cursor and error flag
    std::vector<unsigned char> image;
    if (e == cudaSuccess && !r->generated && !r->coop) {
        image.resize(kTableBytes);
        table_image(&E.table_mech, image.data());
        e = cudaMemcpyAsync(r->d_scratch + 256, image.data(), kTableBytes, cudaMemcpyHostToDevice, r->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);   // host buffers may go after this
    if (e != cudaSuccess) return e;
    r->host.clear();
    r->host.shrink_to_fit();

    const uint32_t P = r->padded;
    DevArgs A;
    memset(&A, 0, sizeof(A));
    double *b = r->d_block;
    A.y = b;
    A.h = b + (size_t)r->n * P;
    A.steps = A.h + P;
    A.rejects = A.steps + P;
    A.pulses = A.rejects + P;
    A.failed = A.pulses + P;
    A.k = A.failed + P;
    A.src = A.k + (size_t)r->R * P;
    A.pulse = A.src + (size_t)r->n * P;
    A.period = A.pulse + (size_t)r->n * P;
    A.pulse_first = A.period + P;
    A.pulse_count = A.pulse_first + P;
    A.padded = P;
    A.lanes = q.cells;
    A.duration = q.dt;
    A.ctl = r->coop ? E.coop_control : E.control;
    const KinMethod M = r->generated ? method_coefficients(2) : r->coop ? E.coop_method : E.table_method;
    memcpy(A.ma, M.a, sizeof(A.ma));
    memcpy(A.mc, M.c, sizeof(A.mc));
    memcpy(A.mm, M.m, sizeof(A.mm));
    memcpy(A.me, M.e, sizeof(A.me));
    A.gamma0 = M.gamma0;
    memcpy(A.new_f, M.new_f, sizeof(A.new_f));
    A.stages = M.stages;
    A.order = M.order;
    A.ir_sweeps = 1;
    A.cursor = (uint32_t *)r->d_scratch;
    A.error_flag = (uint32_t *)(r->d_scratch + 128);
    A.wait_polls = kSpinLimit;
    A.tables = r->d_scratch + 256;
    A.table_bytes = kTableBytes;

    if (r->coop) {   // the cooperative kernel: one CTA per cell
        A.tables = E.d_coop_image;
        A.table_bytes = E.coop_head.bytes;
        const uint32_t block = q.precision == 0 ? 256u : 512u;
        DevArgs idle = A;   // loads the kernel and sets its shared-memory size outside the capture
        idle.lanes = 0;
        e = coop_launch(q.precision, idle, E.coop_head, r->d_coop, 1, block, r->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
        if (e != cudaSuccess) return e;
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t ce = cudaMemsetAsync(r->d_scratch, 0, sizeof(uint32_t), r->stream);
        if (ce == cudaSuccess) ce = coop_launch(q.precision, A, E.coop_head, r->d_coop, r->coop_grid, block, r->stream);
        if (ce == cudaSuccess)
            ce = (cudaError_t)gpu_advect(A.y, P, r->n, q.cells, q.channel_cells, r->d_inlet, r->courant, r->substeps, r->stream);
        e = cudaStreamEndCapture(r->stream, &graph);
        if (ce != cudaSuccess || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return ce != cudaSuccess ? ce : e;
        }
        e = cudaGraphInstantiate(&r->graph, graph, 0);
        cudaGraphDestroy(graph);
        return e;
    }

    Shape sh;
    sh.kind = 2;   // CTA-synchronous persistent queue
    sh.block = 128;
    sh.variant = 0;
    sh.smem = r->generated ? 0 : kTableBytes;
    int per_sm = 0;
    // precision 2 runs the module's current mixed variant (gpu_kin_set_mixed_variant), fixed at admission
    const uint32_t mv = gpu_kin_get_mixed_variant();
    const uint32_t kp = q.precision == 2 && mv == 1 ? 3u : q.precision == 2 && mv == 2 ? 4u : q.precision;
    e = occupancy_chem(r->generated, kp, sh.block, sh.smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const uint32_t resident = (uint32_t)per_sm * (uint32_t)E.sms, needed = (q.cells + sh.block - 1) / sh.block;
    sh.grid = resident < needed ? resident : needed;

    // one launch with no lanes outside the capture: loads the kernel and sets
    // its attributes (it returns right after staging its tables)
    DevArgs idle = A;
    idle.lanes = 0;
    e = launch_chem(r->generated, kp, sh, idle, r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    if (e != cudaSuccess) return e;

    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t ce = cudaMemsetAsync(r->d_scratch, 0, sizeof(uint32_t), r->stream);   // the cursor; the error flag stays sticky
    if (ce == cudaSuccess) ce = launch_chem(r->generated, kp, sh, A, r->stream);
    if (ce == cudaSuccess)
        ce = (cudaError_t)gpu_advect(A.y, P, r->n, q.cells, q.channel_cells, r->d_inlet, r->courant, r->substeps, r->stream);
    e = cudaStreamEndCapture(r->stream, &graph);
    if (ce != cudaSuccess || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return ce != cudaSuccess ? ce : e;
    }
    e = cudaGraphInstantiate(&r->graph, graph, 0);
    cudaGraphDestroy(graph);
    return e;
}

cudaError_t launch_step(Request *r) {
    cudaError_t e = cudaGraphLaunch(r->graph, r->stream);
    if (e == cudaSuccess) e = cudaEventRecord(r->step_done, r->stream);
    if (e == cudaSuccess) {
        ++r->launched;
        ++E.graph_launches;
    }
    return e;
}

// Copies the result rows (state and the solver's per-lane records) back and reads the error flag.
void collect(Request *r) {
    const size_t bytes = (size_t)(r->n + 5) * r->padded * sizeof(double);
    r->host.resize((size_t)(r->n + 5) * r->padded);
    uint32_t flag = 0;
    cudaError_t e = cudaMemcpyAsync(r->host.data(), r->d_block, bytes, cudaMemcpyDeviceToHost, r->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, r->d_scratch + 128, sizeof(flag), cudaMemcpyDeviceToHost, r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    if (e != cudaSuccess) {
        r->state = kFailed;
        r->error = (int32_t)e;
    } else if (flag) {
        r->state = kFailed;
        r->error = (int32_t)cudaErrorTimeout;   // a kernel's bounded wait ran out
    } else {
        r->state = kDone;
    }
}

void finish(Request *r, uint32_t state, int32_t error) {
    r->state = state;
    if (error) r->error = error;
    r->t_done = Clock::now();
    release(r);
    E.in_use -= r->footprint;
    ++E.finished;
}

}   // namespace

SGB_API int32_t gpu_serve_open(uint64_t hbm_budget_bytes, const KinControl *control) {
    if (E.open) return (int32_t)cudaErrorInvalidValue;
    int dev = 0;
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&E.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return (int32_t)e;
    const uint64_t reserve = 1ull << 30;   // left to the driver, graphs and other users of the device
    const uint64_t usable = free_b > reserve ? free_b - reserve : 0;
    E.budget = hbm_budget_bytes && hbm_budget_bytes < usable ? hbm_budget_bytes : usable;
    E.in_use = E.peak = 0;
    E.finished = 0;
    E.graph_launches = 0;
    E.have_table_mech = false;
    E.have_coop = false;
    E.control = control ? *control : KinControl{1e-4, 6.02214076e8, 1e-14, 0.0, 1e-9, 1000000u, 0, 1};
    E.open = true;
    return 0;
}

SGB_API int32_t gpu_serve_set_mech(const KinMech *mech, const KinMethod *method) {
    if (!E.open || !mech || !method) return (int32_t)cudaErrorInvalidValue;
    if (!mech_tables_valid(mech, method)) return (int32_t)cudaErrorInvalidValue;
    if (!E.running.empty() || !E.waiting.empty()) return (int32_t)cudaErrorNotReady;   // requests hold the old tables
    E.table_mech = *mech;
    E.table_method = *method;
    E.have_table_mech = true;
    return 0;
}

// Large mechanism (mechanism = 2, the cooperative kernels) from a finalized host model; only
// while the engine is empty.
SGB_API int32_t gpu_serve_set_coop_mech(const KinModelHandle *model, const KinMethod *method, const KinControl *control) {
    if (!E.open || !model || !method || method->stages < 2 || method->stages > 4) return (int32_t)cudaErrorInvalidValue;
    if (!E.running.empty() || !E.waiting.empty()) return (int32_t)cudaErrorNotReady;
    const Model *m = model_of(model);
    std::vector<uint8_t> img;
    if (!m || !coop_image(*m, &img)) return (int32_t)cudaErrorInvalidValue;
    CoopMech h;
    memcpy(&h, img.data(), sizeof(h));
    int max_smem = 0;
    cudaError_t e = cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0);
    if (e != cudaSuccess) return (int32_t)e;
    if (coop_smem_bytes_for(2, h) > (size_t)max_smem) return (int32_t)cudaErrorInvalidValue;
    if (E.d_coop_image) cudaFree(E.d_coop_image);
    E.d_coop_image = nullptr;
    E.have_coop = false;
    e = cudaMalloc(&E.d_coop_image, img.size());
    if (e == cudaSuccess) e = cudaMemcpy(E.d_coop_image, img.data(), img.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return (int32_t)e;
    E.coop_head = h;
    E.coop_method = *method;
    E.coop_control = control ? *control : E.control;
    E.have_coop = true;
    return 0;
}

SGB_API int32_t gpu_serve_submit(const GpuServeRequest *q, uint64_t *id) {
    if (!E.open || !q || !id || q->cells == 0 || !q->y0 || !q->k || q->coupling_steps == 0 || q->channel_cells == 0 ||
        q->channel_cells > kMaxChannelCells || !(q->dt > 0.0) || !(q->dt < 1e300) || !(q->velocity_m_s >= 0.0) ||
        !(q->velocity_m_s < 1e300) || !(q->dx_m > 0.0) || q->precision > 2 || q->mechanism > 2)
        return (int32_t)cudaErrorInvalidValue;
    if (q->mechanism == 1 && !E.have_table_mech) return (int32_t)cudaErrorInvalidValue;
    if (q->mechanism == 2 && (!E.have_coop || q->precision == 1)) return (int32_t)cudaErrorInvalidValue;
    // Courant-0.9 substeps (nft.cpp:531-536)
    const double v = q->velocity_m_s;
    const double sub = v > 0.0 ? ceil(q->dt / (0.9 * q->dx_m / v)) : 1.0;
    if (!(sub >= 1.0) || sub > 1e6) return (int32_t)cudaErrorInvalidValue;
    Request *r = new Request();
    r->desc = *q;
    r->generated = q->mechanism == 0;
    r->coop = q->mechanism == 2;
    r->n = r->generated ? 17u : r->coop ? E.coop_head.n : E.table_mech.species_count;
    r->R = r->generated ? 44u : r->coop ? E.coop_head.R : E.table_mech.reaction_count;
    if (r->coop) {
        const uint32_t per_sm = q->precision == 0 ? 2u : 1u;
        r->coop_grid = (uint32_t)E.sms * per_sm < q->cells ? (uint32_t)E.sms * per_sm : q->cells;
    }
    r->padded = pad8(q->cells);
    r->rows = 3 * r->n + r->R + 8;
    r->substeps = (uint32_t)sub;
    r->courant = v * (q->dt / r->substeps) / q->dx_m;
    r->footprint = (uint64_t)r->rows * r->padded * sizeof(double) + r->n * sizeof(double) + 256 + kTableBytes;
    if (r->coop) r->footprint += coop_scratch_doubles_for(q->precision, E.coop_head) * sizeof(double) * r->coop_grid;
    if (r->footprint > E.budget) {   // could never be admitted
        delete r;
        return (int32_t)cudaErrorMemoryAllocation;
    }
    const uint32_t P = r->padded, c = q->cells;
    r->host.assign((size_t)r->rows * P, 0.0);
    for (uint32_t s = 0; s < r->n; ++s) memcpy(&r->host[(size_t)s * P], q->y0 + (size_t)s * c, c * sizeof(double));
    const size_t k_row = (size_t)(r->n + 5) * P;
    for (uint32_t j = 0; j < r->R; ++j) memcpy(&r->host[k_row + (size_t)j * P], q->k + (size_t)j * c, c * sizeof(double));
    r->id = E.next_id++;
    r->t_submit = Clock::now();
    E.waiting.push_back(r);
    E.all[r->id] = r;
    *id = r->id;
    return 0;
}

SGB_API int32_t gpu_serve_progress(uint32_t *running, uint32_t *waiting, uint32_t *finished) {
    if (!E.open) return (int32_t)cudaErrorInvalidValue;
    // 1. running requests: retire the finished and cancelled, launch the next step of the idle
    for (size_t i = 0; i < E.running.size();) {
        Request *r = E.running[i];
        if (r->launched != r->completed) {
            const cudaError_t q = cudaEventQuery(r->step_done);
            if (q == cudaSuccess) {
                r->completed = r->launched;
            } else if (q != cudaErrorNotReady) {
                finish(r, kFailed, (int32_t)q);
                E.running.erase(E.running.begin() + (long)i);
                continue;
            }
        }
        const bool idle = r->launched == r->completed;
        if (idle && (r->cancel || r->completed == r->desc.coupling_steps)) {
            if (r->cancel) {
                finish(r, kCancelled, 0);
            } else {
                collect(r);
                finish(r, r->state, r->error);
            }
            E.running.erase(E.running.begin() + (long)i);
            continue;
        }
        if (idle) {
            const cudaError_t e = launch_step(r);
            if (e != cudaSuccess) {
                finish(r, kFailed, (int32_t)e);
                E.running.erase(E.running.begin() + (long)i);
                continue;
            }
        }
        ++i;
    }
    // 2. admission in arrival order while the next request fits the HBM budget
    while (!E.waiting.empty() && E.in_use + E.waiting.front()->footprint <= E.budget) {
        Request *r = E.waiting.front();
        E.waiting.pop_front();
        E.in_use += r->footprint;
        if (E.in_use > E.peak) E.peak = E.in_use;
        r->t_admit = Clock::now();
        r->state = kRunning;
        cudaError_t e = admit(r);
        if (e == cudaSuccess) e = launch_step(r);
        if (e != cudaSuccess) {
            cudaGetLastError();
            finish(r, kFailed, (int32_t)e);
            continue;
        }
        E.running.push_back(r);
    }
    if (running) *running = (uint32_t)E.running.size();
    if (waiting) *waiting = (uint32_t)E.waiting.size();
    if (finished) *finished = E.finished;
    return 0;
}

SGB_API int32_t gpu_serve_cancel(uint64_t id) {
    auto it = E.all.find(id);
    if (!E.open || it == E.all.end()) return (int32_t)cudaErrorInvalidValue;
    Request *r = it->second;
    if (r->state == kWaiting) {
        for (auto w = E.waiting.begin(); w != E.waiting.end(); ++w)
            if (*w == r) {
                E.waiting.erase(w);
                break;
            }
        r->state = kCancelled;
        r->t_done = Clock::now();
        r->host.clear();
        r->host.shrink_to_fit();
        ++E.finished;
    } else if (r->state == kRunning) {
        r->cancel = true;   // retired by gpu_serve_progress once its step in flight completes
    }
    return 0;
}

SGB_API int32_t gpu_serve_poll(uint64_t id, GpuServeStatus *st) {
    auto it = E.all.find(id);
    if (!E.open || !st || it == E.all.end()) return (int32_t)cudaErrorInvalidValue;
    const Request *r = it->second;
    st->state = r->state;
    st->error = r->error;
    st->steps_completed = r->completed;
    st->substeps = r->substeps;
    st->courant = r->courant;
    st->admit_s = r->state != kWaiting && r->t_admit.time_since_epoch().count()
                      ? std::chrono::duration<double>(r->t_admit - r->t_submit).count() : -1.0;
    st->latency_s = r->state >= kDone ? std::chrono::duration<double>(r->t_done - r->t_submit).count() : -1.0;
    return 0;
}

SGB_API int32_t gpu_serve_result(uint64_t id, double *y_out, double *steps_out, double *failed_out) {
    auto it = E.all.find(id);
    if (!E.open || it == E.all.end() || it->second->state != kDone) return (int32_t)cudaErrorInvalidValue;
    const Request *r = it->second;
    const uint32_t P = r->padded, c = r->desc.cells;
    if (y_out)
        for (uint32_t s = 0; s < r->n; ++s) memcpy(y_out + (size_t)s * c, &r->host[(size_t)s * P], c * sizeof(double));
    if (steps_out) memcpy(steps_out, &r->host[(size_t)(r->n + 1) * P], c * sizeof(double));
    if (failed_out) memcpy(failed_out, &r->host[(size_t)(r->n + 4) * P], c * sizeof(double));
    return 0;
}

SGB_API int32_t gpu_serve_forget(uint64_t id) {
    auto it = E.all.find(id);
    if (!E.open || it == E.all.end() || it->second->state < kDone) return (int32_t)cudaErrorInvalidValue;
    delete it->second;
    E.all.erase(it);
    return 0;
}

SGB_API int32_t gpu_serve_stats(GpuServeStats *st) {
    if (!E.open || !st) return (int32_t)cudaErrorInvalidValue;
    st->budget_bytes = E.budget;
    st->in_use_bytes = E.in_use;
    st->peak_bytes = E.peak;
    st->graph_launches = E.graph_launches;
    st->running = (uint32_t)E.running.size();
    st->waiting = (uint32_t)E.waiting.size();
    st->finished = E.finished;
    return 0;
}

SGB_API int32_t gpu_serve_close(void) {
    if (!E.open) return 0;
    for (Request *r : E.running)
        if (r->stream) cudaStreamSynchronize(r->stream);
    for (auto &kv : E.all) {
        release(kv.second);
        delete kv.second;
    }
    E.all.clear();
    E.waiting.clear();
    E.running.clear();
    E.in_use = 0;
    E.open = false;
    if (E.d_coop_image) cudaFree(E.d_coop_image);
    E.d_coop_image = nullptr;
    E.have_coop = false;
    return (int32_t)cudaDeviceSynchronize();
}
