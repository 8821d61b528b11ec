// Wide-index mechanism image for the cooperative kernels (one CTA per cell):
// mechanisms beyond the reference's u16 KinMech tables (config-scale: 200
// species, 1,200 reactions, ~32k LU non-zeros, ~1.8M LU updates).
//
// Every array keeps the operation order of the reference's solver
// (src/sim/kinetics/kin_solver.h:40-139) per element:
//   - RHS: f[s] = src[s], then fma(net, rate_r, f[s]) over reactions r ascending;
//   - Jacobian: a[slot] = 0, then fma(-net, d_rp, a[slot]) over (r, p, e) ascending;
//   - LU: the elimination runs pivot by pivot (KIJ) instead of row by row
//     (IKJ), which applies the same updates to every element in the same
//     (ascending pivot) order, so the results are the same bits;
//   - solves: in blocks of 32 columns (a warp solves the diagonal block, then
//     every row outside it takes the block's updates one by one), which gives
//     every x[i] its updates in the reference's order (lower: ascending
//     column; upper: descending column, then the diagonal).
// The LU lives in a dense [n][ld] array (the filled pattern is 78-87% dense
// for a 200-species random mechanism in natural order); the kernels walk it
// densely and test each element against the pattern bitmask, so only
// pattern elements are ever updated, as in the reference.
#pragma once
#include <stdint.h>

namespace sgb {

struct CoopTerm {
    uint32_t index;   // fun: reaction; jac: reaction | reactant position << 24
    float coef;       // net change (fun) or its negation (jac); small integers, exact
};

struct CoopMech {
    uint32_t n, R, ld;        // species, reactions, dense row stride (odd: conflict-free column reads)
    uint32_t nj;              // Jacobian entries reactions scatter into (compact slot order = row-major)
    uint32_t fun_terms, jac_terms;
    uint32_t l_entries, u_entries;
    uint64_t lu_updates;      // sum over pivots of |L(k)| |U(k)|
    uint32_t nnz;             // filled pattern incl. diagonal
    uint32_t bytes;           // image size
    // byte offsets from the image start (each 16-byte aligned)
    uint32_t off_reac;        // uint16[R][4]: reactant count, then up to 3 reactant species
    uint32_t off_fbeg;        // uint32[n+1]
    uint32_t off_fent;        // CoopTerm[fun_terms], per species, reactions ascending
    uint32_t off_jbeg;        // uint32[nj+1]
    uint32_t off_jent;        // CoopTerm[jac_terms], per entry, (r, p, e) ascending
    uint32_t off_jpos;        // uint32[nj]: row * ld + col
    uint32_t off_jrow;        // uint32[n+1]: entries of row i are [jrow[i], jrow[i+1])
    uint32_t off_jcol;        // uint16[nj]
    uint32_t off_lbeg;        // uint32[n+1]
    uint32_t off_lrow;        // uint16[]: rows i > k with (i, k) in the filled pattern, per column k
    uint32_t off_ubeg;        // uint32[n+1]
    uint32_t off_ucol;        // uint16[]: columns j > k with (k, j) in the filled pattern, per row k
    uint32_t off_cbeg;        // uint32[n+1]
    uint32_t off_crow;        // uint16[]: rows i < k with (i, k) in the filled pattern, per column k
    uint32_t off_pat;         // uint32[n][8]: filled pattern, bit j of row i (n <= 256)
    uint32_t off_lcnt;        // uint16[n]: rows below the diagonal in column k
    uint32_t reserved;
};

}   // namespace sgb
