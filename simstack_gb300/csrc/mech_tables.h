// Host-side checks and staging of a KinMech for the table-driven kernels,
// shared by every entry point that launches them.
#pragma once
#include <string.h>

#include "../../include/simstack_gpu.h"
#include "kin_table.cuh"
#include "mech.h"

namespace sgb {

// True when the method's coefficients are exactly Rodas3's (the generated
// kernels have them compiled in).
inline bool method_is_rodas3(const KinMethod *m) {
    KinMethod r = method_coefficients(2);
    return m->stages == r.stages && m->order == r.order && memcmp(m->a, r.a, sizeof(r.a)) == 0 &&
           memcmp(m->c, r.c, sizeof(r.c)) == 0 && memcmp(m->m, r.m, sizeof(r.m)) == 0 &&
           memcmp(m->e, r.e, sizeof(r.e)) == 0 && m->gamma0 == r.gamma0 && memcmp(m->new_f, r.new_f, sizeof(r.new_f)) == 0;
}

// The table kernels trust every index: reject records that would read outside them.
inline bool mech_tables_valid(const KinMech *mech, const KinMethod *method) {
    const uint32_t n = mech->species_count, nnz = mech->nnz;
    if (n == 0 || n > KIN_MAX_SPECIES || mech->reaction_count > KIN_MAX_REACTIONS || nnz > KIN_MAX_NNZ ||
        mech->lu_div_count > KIN_MAX_LU_DIV || mech->lu_sub_count > KIN_MAX_LU_SUB || method->stages < 2 ||
        method->stages > KIN_MAX_STAGES)
        return false;
    if (mech->div_begin[n] != mech->lu_div_count || mech->lower_begin[n] > KIN_MAX_NNZ || mech->upper_begin[n] > KIN_MAX_NNZ)
        return false;
    for (uint32_t i = 0; i < n; ++i)
        if (mech->diag[i] >= nnz || mech->div_begin[i] > mech->div_begin[i + 1] ||
            mech->lower_begin[i] > mech->lower_begin[i + 1] || mech->upper_begin[i] > mech->upper_begin[i + 1])
            return false;
    for (uint32_t d = 0; d < mech->lu_div_count; ++d) {
        const KinLuDiv &v = mech->lu_div[d];
        if (v.ik >= nnz || v.kk >= nnz || v.sub_begin > v.sub_end || v.sub_end > mech->lu_sub_count) return false;
    }
    for (uint32_t s = 0; s < mech->lu_sub_count; ++s)
        if (mech->lu_sub[s].ij >= nnz || mech->lu_sub[s].kj >= nnz) return false;
    for (uint32_t e = 0; e < mech->lower_begin[n]; ++e)
        if (mech->lower[e].index >= nnz || mech->lower[e].col >= n) return false;
    for (uint32_t e = 0; e < mech->upper_begin[n]; ++e)
        if (mech->upper[e].index >= nnz || mech->upper[e].col >= n) return false;
    for (uint32_t r = 0; r < mech->reaction_count; ++r) {
        const KinReaction &rx = mech->reactions[r];
        if (rx.reactant_count > KIN_MAX_REACTANTS || rx.net_count > KIN_MAX_NET) return false;
        for (uint32_t p = 0; p < rx.reactant_count; ++p) {
            if (rx.reactant[p] >= n) return false;
            for (uint32_t e = 0; e < rx.net_count; ++e)
                if (rx.jac_index[p][e] >= nnz) return false;
        }
        for (uint32_t e = 0; e < rx.net_count; ++e)
            if (rx.net_species[e] >= n) return false;
    }
    return true;
}

// The staged image (kTableBytes): the KinMech record, then the bitmask of the
// compact slots in the Jacobian's own pattern (slots some reaction scatters
// into, plus the diagonal). The record must have passed mech_tables_valid.
inline void table_image(const KinMech *mech, unsigned char *image) {
    memset(image, 0, kTableBytes);
    memcpy(image, mech, sizeof(KinMech));
    unsigned char *mask = image + kJacMaskOffset;
    for (uint32_t i = 0; i < mech->species_count; ++i) mask[mech->diag[i] >> 3] |= (unsigned char)(1u << (mech->diag[i] & 7));
    for (uint32_t r = 0; r < mech->reaction_count; ++r) {
        const KinReaction &rx = mech->reactions[r];
        for (uint32_t p = 0; p < rx.reactant_count; ++p)
            for (uint32_t e = 0; e < rx.net_count; ++e)
                mask[rx.jac_index[p][e] >> 3] |= (unsigned char)(1u << (rx.jac_index[p][e] & 7));
    }
}

}   // namespace sgb
