// Tensor memory (TMEM, 256 KB per SM) as per-thread storage for the integrator's lanes. The
// integrator has no matrix product to give the tensor cores, but its lanes' working set is
// larger than the register file, and TMEM is a second on-chip array of the same size: a warp
// reads and writes its own 32 TMEM lanes, one per thread, with tcgen05.ld / tcgen05.st of
// consecutive 32-bit columns. A CTA allocates its columns once (one warp, tcgen05.alloc), every
// thread addresses its lane quarter and column range, and the CTA frees them before it exits.
//
// Each load and store here waits for its own completion inside the same asm statement, so no
// register is read before the data has arrived. All are warp-collective (.sync.aligned): callers
// reconverge the warp first (__syncwarp).

#pragma once
#include <stdint.h>

#include "ptx.cuh"

namespace sgb {

// Allocates `ncols` columns (a power of two, 32..512) for the CTA and writes their base address
// to *slot (shared memory); called by one whole warp.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t base, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// This thread's address: the warp's lane quarter (warp % 4) in bits 31:16, `col` in bits 15:0.
__device__ __forceinline__ uint32_t tmem_lane_addr(uint32_t base, uint32_t col) {
    const uint32_t warp = threadIdx.x >> 5;
    return base + (((warp & 3u) * 32u) << 16) + col;
}

// 32 consecutive columns of this thread's lane <-> v[0..31]
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float *v) {
    asm volatile("{\n tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};\n tcgen05.wait::st.sync.aligned;\n}"
                 :: "r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
                 "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
                 "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
                 "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])),
                 "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])), "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])),
                 "r"(__float_as_uint(v[20])), "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
                 "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])), "r"(__float_as_uint(v[27])),
                 "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])), "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t u[32];
    asm volatile("{\n tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n tcgen05.wait::ld.sync.aligned;\n}"
                 : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]),
                 "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
                 "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]),
                 "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]),
                 "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]),
                 "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]),
                 "=r"(u[24]), "=r"(u[25]), "=r"(u[26]), "=r"(u[27]),
                 "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31])
                 : "r"(taddr)
                 : "memory");
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(u[i]);
}
// 2 consecutive columns <-> v[0..1]
__device__ __forceinline__ void tmem_st2(uint32_t taddr, float a, float b) {
    asm volatile("{\n tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};\n tcgen05.wait::st.sync.aligned;\n}"
                 :: "r"(taddr), "r"(__float_as_uint(a)), "r"(__float_as_uint(b)) : "memory");
}
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float &a, float &b) {
    uint32_t x, y;
    asm volatile("{\n tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];\n tcgen05.wait::ld.sync.aligned;\n}"
                 : "=r"(x), "=r"(y) : "r"(taddr) : "memory");
    a = __uint_as_float(x);
    b = __uint_as_float(y);
}

}   // namespace sgb
