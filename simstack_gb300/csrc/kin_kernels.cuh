// Kernels of the batched integrator, instantiated per (ops, method, precision)
// in separate translation units so the module builds in parallel.
//
//   static  one cell per thread, grid = ceil(lanes / block): the reference's
//           launch shape (src/gpu/kernels.cu:263-274), each thread running its
//           cell to completion
//   queue   persistent: grid = SMs x resident CTAs; each thread claims a cell
//           from a device work queue (atomic cursor), runs it, and claims the
//           next the moment it finishes, so lanes whose cells need few steps do
//           not sit idle beside stiff ones (warp lanes stay busy, CTAs never
//           wait for a tail of long cells)
// Register-budget variants: 0 = __launch_bounds__(128, 1) (up to 255 regs),
// 1 = __launch_bounds__(128, 4) (128 regs).

#pragma once
#include <cuda_runtime.h>

#include "kin_device.cuh"

namespace sgb {

template <int V> struct Budget;
template <> struct Budget<0> { static constexpr int kThreads = 128, kMinBlocks = 1; };
template <> struct Budget<1> { static constexpr int kThreads = 128, kMinBlocks = 4; };
template <> struct Budget<2> { static constexpr int kThreads = 256, kMinBlocks = 1; };
template <> struct Budget<3> { static constexpr int kThreads = 512, kMinBlocks = 1; };   // 128 registers

// Build-time switch: the double-float mixed lanes keep their LU in shared memory
// (generated ops, CTAs of up to 256 threads) instead of registers / local memory.
#ifndef SGB_SHARED_LU
#define SGB_SHARED_LU 0
#endif

// The lane type of a precision: 0 FP64, 1 f32 Delta, 2 mixed with FP64
// refinement, 3 mixed with double-float state, 4 mixed with double-float state
// and refined stages.
template <class Ops, class M, int PREC, int V> struct LaneOf { typedef Lane<Ops, M, PREC> type; };
template <class Ops, class M, int V> struct LaneOf<Ops, M, 3, V> {
    static constexpr int kStride = (SGB_SHARED_LU && Ops::kStridedLu && Budget<V>::kThreads <= 256) ? Budget<V>::kThreads : 0;
    typedef LaneDf<Ops, M, kStride> type;
};
// Build-time switch (default on): the refined double-float lanes keep their FP32 LU in shared
// memory, which frees registers for their double-float vectors (measured 619 against 753 ms on
// 1,048,576 cells x 10 s).
#ifndef SGB_IR_SHARED_LU
#define SGB_IR_SHARED_LU 1
#endif
// Build-time switch (default on): the refined lanes keep their stage vectors in tensor memory,
// 256 columns per 128 threads of the launch bound (measured 568 against 580 ms on 1,048,576
// cells x 10 s: the stage vectors leave local memory). Only with the shared-memory LU, whose
// footprint (NNZ x launch bound x 4 bytes: 109 KB at 128 threads, 218 KB at 256 for the shipped
// mechanism) caps how many CTAs an SM holds (228 KB of shared memory) so that together they
// never ask for more than the SM's 512 columns: an allocation never waits.
#ifndef SGB_IR_TMEM
#define SGB_IR_TMEM 1
#endif
constexpr uint32_t kSmemPerSm = 233472;   // 228 KB
template <class Ops, class M, int V> struct LaneOf<Ops, M, 4, V> {
    static constexpr int kStride = (SGB_IR_SHARED_LU && Ops::kStridedLu && Budget<V>::kThreads <= 256) ? Budget<V>::kThreads : 0;
    static constexpr uint32_t kCols = 256u * (uint32_t)(Budget<V>::kThreads / 128);
    static constexpr uint32_t kLuBytes = (uint32_t)Ops::NNZ * (uint32_t)(kStride > 0 ? kStride : 1) * 4u;
    static constexpr bool kFits = kStride > 0 && (kSmemPerSm / kLuBytes) * kCols <= 512u;
    static constexpr int kTmem = (SGB_IR_TMEM && kFits) ? (int)kCols : 0;
    typedef LaneIr<Ops, M, kStride, kTmem> type;
};

// Tensor-memory columns of the lanes that keep data there: one warp allocates them for the CTA
// before the lanes start and frees them after every lane is done (all threads pass both calls).
template <class L> struct TmemCols { static constexpr uint32_t value = 0; };
template <class Ops, class M, int S, int C> struct TmemCols<LaneIr<Ops, M, S, C>> { static constexpr uint32_t value = (uint32_t)C; };

template <class L> __device__ __forceinline__ void lanes_tmem_open(L &lane, uint32_t *slot) {
    if constexpr (TmemCols<L>::value > 0) {
        if (threadIdx.x < 32) tmem_alloc(slot, TmemCols<L>::value);
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
        lane.bind_tmem(*slot);
    }
}
template <class L> __device__ __forceinline__ void lanes_tmem_close(const uint32_t *slot) {
    if constexpr (TmemCols<L>::value > 0) {
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
        if (threadIdx.x < 32) tmem_dealloc(*slot, TmemCols<L>::value);
    }
}

// Both kernels keep every lane of a warp in the loop until the whole warp is
// out of work, and vote (__any_sync) once per iteration: the vote is a
// reconvergence point, so all lanes that need a step attempt run it together
// and the attempt's straight-line code issues once per warp, not once per
// diverged group of lanes. Blocks are whole warps.

template <class Ops, class M, int PREC, int V>
__global__ void __launch_bounds__(Budget<V>::kThreads, Budget<V>::kMinBlocks) kin_static_kernel(const __grid_constant__ DevArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    typename LaneOf<Ops, M, PREC, V>::type L;
    if (!L.ops.init(A, smem)) {
        if (threadIdx.x == 0) atomicExch(A.error_flag, 1u);
        return;
    }
    L.bind(smem);
    __shared__ uint32_t tmem_slot;
    lanes_tmem_open(L, &tmem_slot);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool have = i < A.lanes;
    if (have) L.load(A, i);
    else if (TmemCols<decltype(L)>::value > 0) L.load(A, 0);   // a finite state for lanes that attempt with no cell
    for (;;) {
        bool need = false;
        if (have) {
            need = L.settle(A, i);
            if (!need) {
                L.store(A, i);
                have = false;
            }
        }
        if (!__any_sync(0xffffffffu, need)) break;
        if constexpr (TmemCols<decltype(L)>::value > 0) L.attempt(A, need);   // warp-collective TMEM access: every lane
        else if (need) L.attempt(A);
    }
    lanes_tmem_close<decltype(L)>(&tmem_slot);
}

template <class Ops, class M, int PREC, int V>
__global__ void __launch_bounds__(Budget<V>::kThreads, Budget<V>::kMinBlocks) kin_queue_kernel(const __grid_constant__ DevArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    typename LaneOf<Ops, M, PREC, V>::type L;
    if (!L.ops.init(A, smem)) {
        if (threadIdx.x == 0) atomicExch(A.error_flag, 1u);
        return;
    }
    L.bind(smem);
    __shared__ uint32_t tmem_slot;
    lanes_tmem_open(L, &tmem_slot);
    if (TmemCols<decltype(L)>::value > 0) L.load(A, 0);   // a finite state for lanes that attempt with no cell
    bool have = false, exhausted = false;
    uint32_t cell = 0;
    for (;;) {
        bool need = false;
        while (!exhausted) {   // this lane: finish, store and replace cells until one needs an attempt
            if (!have) {
                cell = atomicAdd(A.cursor, 1u);
                if (cell >= A.lanes) {
                    exhausted = true;
                    break;
                }
                L.load(A, cell);
                have = true;
            }
            if (L.settle(A, cell)) {
                need = true;
                break;
            }
            L.store(A, cell);
            have = false;
        }
        if (!__any_sync(0xffffffffu, need)) break;
        if constexpr (TmemCols<decltype(L)>::value > 0) L.attempt(A, need);   // warp-collective TMEM access: every lane
        else if (need) L.attempt(A);
    }
    lanes_tmem_close<decltype(L)>(&tmem_slot);
}

// CTA-synchronous persistent queue: like kin_queue_kernel, but the whole CTA
// votes (__syncthreads_or) and runs every step attempt together, with
// barriers between its phases, so the CTA's warps fetch the same stretch of
// the straight-line step code instead of one stretch each (the step code is
// far larger than the instruction caches). Lanes without a cell compute on
// their last state and commit nothing; a lane that never had one starts from
// a copy of cell 0.
template <class Ops, class M, int PREC, int V>
__global__ void __launch_bounds__(Budget<V>::kThreads, Budget<V>::kMinBlocks) kin_queue_cta_kernel(const __grid_constant__ DevArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    typename LaneOf<Ops, M, PREC, V>::type L;
    if (!L.ops.init(A, smem)) {
        if (threadIdx.x == 0) atomicExch(A.error_flag, 1u);
        return;
    }
    L.bind(smem);
    if (A.lanes == 0) return;
    __shared__ uint32_t tmem_slot;
    lanes_tmem_open(L, &tmem_slot);
    L.load(A, 0);   // a finite state for lanes that never get a cell
    bool have = false, exhausted = false;
    uint32_t cell = 0;
    for (;;) {
        bool need = false;
        while (!exhausted) {
            if (!have) {
                cell = atomicAdd(A.cursor, 1u);
                if (cell >= A.lanes) {
                    exhausted = true;
                    break;
                }
                L.load(A, cell);
                have = true;
            }
            if (L.settle(A, cell)) {
                need = true;
                break;
            }
            L.store(A, cell);
            have = false;
        }
        if (!__syncthreads_or(need)) break;
        L.template attempt<true>(A, need);
    }
    lanes_tmem_close<decltype(L)>(&tmem_slot);
}

// Launch shape chosen by the host (module tuning or the autotuner).
struct Shape {
    uint32_t kind;      // 0 static, 1 queue
    uint32_t block;     // threads per CTA, multiple of 32, <= 128
    uint32_t grid;      // CTAs
    uint32_t variant;   // register budget
    size_t smem;        // dynamic shared memory (table ops: staged tables)
};

// kVariants: how many register-budget variants are instantiated (1: variant 0 only).
template <class Ops, class M, int PREC, int kVariants>
void (*kernel_for(uint32_t kind, uint32_t variant))(DevArgs) {
    if (kind == 2) {   // CTA-synchronous queue: 128 threads (variants 0, 1), 256 threads (2) or 512 threads (3)
        if (kVariants > 1 && variant == 1) return kin_queue_cta_kernel<Ops, M, PREC, (kVariants > 1 ? 1 : 0)>;
        if (kVariants > 1 && variant == 2) return kin_queue_cta_kernel<Ops, M, PREC, (kVariants > 1 ? 2 : 0)>;
        if (kVariants > 1 && variant == 3) return kin_queue_cta_kernel<Ops, M, PREC, (kVariants > 1 ? 3 : 0)>;
        return kin_queue_cta_kernel<Ops, M, PREC, 0>;
    }
    if (kVariants > 1 && variant == 1)
        return kind == 0 ? kin_static_kernel<Ops, M, PREC, (kVariants > 1 ? 1 : 0)> : kin_queue_kernel<Ops, M, PREC, (kVariants > 1 ? 1 : 0)>;
    return kind == 0 ? kin_static_kernel<Ops, M, PREC, 0> : kin_queue_kernel<Ops, M, PREC, 0>;
}

// Shared memory the lane itself needs (a shared-memory LU), per kernel variant.
template <class Ops, class M, int PREC, int kVariants>
size_t lane_smem_for(uint32_t kind, uint32_t variant) {
    constexpr int V1 = kVariants > 1 ? 1 : 0, V2 = kVariants > 1 ? 2 : 0, V3 = kVariants > 1 ? 3 : 0;
    if (kVariants > 1 && variant == 1) return LaneOf<Ops, M, PREC, V1>::type::kSmemBytes;
    if (kind == 2 && kVariants > 1 && variant == 2) return LaneOf<Ops, M, PREC, V2>::type::kSmemBytes;
    if (kind == 2 && kVariants > 1 && variant == 3) return LaneOf<Ops, M, PREC, V3>::type::kSmemBytes;
    return LaneOf<Ops, M, PREC, 0>::type::kSmemBytes;
}

template <class Ops, class M, int PREC, int kVariants = 2>
cudaError_t launch_one(const Shape &s, const DevArgs &A, cudaStream_t stream) {
    void (*fn)(DevArgs) = kernel_for<Ops, M, PREC, kVariants>(s.kind, s.variant);
    const size_t smem = s.smem + lane_smem_for<Ops, M, PREC, kVariants>(s.kind, s.variant);
    if (smem == 0) {   // no shared memory: give the unified L1/shared array to L1 (local-memory spills live there)
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        if (e != cudaSuccess) return e;
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    fn<<<s.grid, s.block, smem, stream>>>(A);
    return cudaGetLastError();
}

// Local memory (stack frame) a kernel variant needs per thread.
template <class Ops, class M, int PREC, int kVariants = 2>
cudaError_t local_bytes_one(uint32_t kind, uint32_t variant, size_t *bytes) {
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, kernel_for<Ops, M, PREC, kVariants>(kind, variant));
    *bytes = e == cudaSuccess ? attr.localSizeBytes : 0;
    return e;
}

template <class Ops, class M, int PREC, int kVariants = 2>
cudaError_t occupancy_one(uint32_t kind, uint32_t variant, uint32_t block, size_t smem, int *blocks_per_sm) {
    void (*fn)(DevArgs) = kernel_for<Ops, M, PREC, kVariants>(kind, variant);
    smem += lane_smem_for<Ops, M, PREC, kVariants>(kind, variant);
    if (smem > 48 * 1024) {   // the occupancy query honours the attribute, so set it first
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, (int)block, smem);
}

}   // namespace sgb
