// Straight-line (generated) kernels for the shipped mechanism with Rodas3
// coefficients folded in; one precision per compilation (-DSGB_PREC=0|1|2|3|4).

#include "kin_kernels.cuh"

namespace sgb {
#include "air_ops.cuh"
}

#ifndef SGB_PREC
#error "compile with -DSGB_PREC=0, 1, 2, 3 or 4"
#endif

#define SGB_CAT2(a, b) a##b
#define SGB_CAT(a, b) SGB_CAT2(a, b)

namespace sgb {

cudaError_t SGB_CAT(launch_air_p, SGB_PREC)(const Shape &s, const DevArgs &A, cudaStream_t stream) {
    return launch_one<GenOps<AirOps>, Rodas3Coef, SGB_PREC>(s, A, stream);
}

cudaError_t SGB_CAT(occupancy_air_p, SGB_PREC)(uint32_t kind, uint32_t variant, uint32_t block, int *blocks_per_sm) {
    return occupancy_one<GenOps<AirOps>, Rodas3Coef, SGB_PREC>(kind, variant, block, 0, blocks_per_sm);
}

cudaError_t SGB_CAT(local_air_p, SGB_PREC)(uint32_t kind, uint32_t variant, size_t *bytes) {
    return local_bytes_one<GenOps<AirOps>, Rodas3Coef, SGB_PREC>(kind, variant, bytes);
}

}   // namespace sgb

#if SGB_PREC == 0
namespace sgb {
uint64_t air_ops_signature() { return AirOps::kSignature; }
}
#endif
