// Table-driven kernels (any mechanism within the KinMech capacities, any
// method of up to four stages), one precision per compilation
// (-DSGB_PREC=0|1|2|3|4). A single register-budget variant: the per-lane arrays of
// the generic path live in local memory whatever the budget.

#include "kin_kernels.cuh"
#include "kin_table.cuh"

#ifndef SGB_PREC
#error "compile with -DSGB_PREC=0, 1, 2, 3 or 4"
#endif

#define SGB_CAT2(a, b) a##b
#define SGB_CAT(a, b) SGB_CAT2(a, b)

namespace sgb {

cudaError_t SGB_CAT(launch_table_p, SGB_PREC)(const Shape &s, const DevArgs &A, cudaStream_t stream) {
    return launch_one<TableOps, RuntimeCoef, SGB_PREC, 1>(s, A, stream);
}

cudaError_t SGB_CAT(occupancy_table_p, SGB_PREC)(uint32_t kind, uint32_t block, size_t smem, int *blocks_per_sm) {
    return occupancy_one<TableOps, RuntimeCoef, SGB_PREC, 1>(kind, 0, block, smem, blocks_per_sm);
}

cudaError_t SGB_CAT(local_table_p, SGB_PREC)(uint32_t kind, size_t *bytes) {
    return local_bytes_one<TableOps, RuntimeCoef, SGB_PREC, 1>(kind, 0, bytes);
}

}   // namespace sgb
