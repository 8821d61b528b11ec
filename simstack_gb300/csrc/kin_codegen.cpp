// Build-time generator: compiles a mechanism with the module's own symbolic
// phase (mech.cpp) and writes straight-line CUDA device code for its solver
// kernels -- the RHS, -J, the W = I/(gamma h) - J elimination and the two
// triangular solves, plus the FP64 iterative-refinement residual of the mixed
// path -- with every array index a compile-time constant.
//
//   kin_codegen <out.cuh>
//
// Each emitted operation is the reference table walk's operation, in the
// same order (src/sim/kinetics/kin_solver.h:40-139; the reference's own
// generator, src/tools/kin_codegen.cpp:32-138, does the same for the CPU), so
// the results are bit-identical to the table walk. One exact rewrite is
// applied: the first contribution to a zeroed Jacobian slot, fma(+-1, d, +0),
// is emitted as an integer sign/zero fix of d (sgb_first_pos / sgb_first_neg),
// which yields the same bits without an FP64 instruction.

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "mech.h"

using namespace sgb;

// acc[s] += c * v with the lazily normalised accumulation (exact scaling for +-1, +-2, +-4).
static void emit_lazy_term(FILE *f, uint32_t s, int c, const char *v) {
    if (c == 1) fprintf(f, "          acc[%u] = df_acc(acc[%u], %s);\n", s, s, v);
    else if (c == -1 || c == 2 || c == -2 || c == 4 || c == -4) fprintf(f, "          acc[%u] = df_acc(acc[%u], df_scale(%s, %d.0f));\n", s, s, v, c);
    else fprintf(f, "          acc[%u] = df_acc(acc[%u], df_mul_u(%s, Df{%d.0f, 0.0f}));\n", s, s, v, c);
}

static void emit_ops(FILE *f, Model &m, const char *name) {
    const Symbolic &S = m.sym;
    const uint32_t n = m.n(), R = m.R();
    KinMech km;
    bool fits = m.to_kinmech(&km);
    uint64_t signature = fits ? fnv1a(&km, sizeof(km)) : 0;

    // J-pattern slots (non-zeros of -J before fill-in), in compact order: the
    // mixed path keeps a copy of them for its FP64 residual.
    std::vector<uint32_t> jslots;
    std::vector<uint32_t> jrow, jcol;
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < n; ++j)
            if (S.jac_pattern[(size_t)i * n + j]) {
                jslots.push_back(S.slot[(size_t)i * n + j]);
                jrow.push_back(i);
                jcol.push_back(j);
            }

    fprintf(f, "struct %s {\n", name);
    fprintf(f, "    static constexpr int N = %u, R = %u, NNZ = %u, NJ = %zu;\n", n, R, S.nnz, jslots.size());
    fprintf(f, "    static constexpr unsigned long long kSignature = 0x%016llxull;\n\n", (unsigned long long)signature);

    // fun: f = src + sum_r net_r k_r prod(y[reactants])
    fprintf(f, "    template <class T>\n    static __device__ __forceinline__ void fun(const T *__restrict__ k, const T *__restrict__ src, const T *__restrict__ y, T *__restrict__ f) {\n");
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        f[%u] = src[%u];\n", s, s);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        fprintf(f, "        { T rate = k[%u]", r);
        for (uint32_t q : rx.reactants) fprintf(f, " * y[%u]", q);
        fprintf(f, ";  // %s\n", rx.equation.c_str());
        for (auto &e : rx.net) fprintf(f, "          f[%u] = sgb_fma((T)%d.0, rate, f[%u]);\n", e.first, e.second, e.first);
        fprintf(f, "        }\n");
    }
    fprintf(f, "    }\n\n");

    // fun in double-float (mixed path): the same terms in the same order as fun,
    // each rate a double-float product, each species a double-float sum.
    fprintf(f, "    static __device__ __forceinline__ void fun_df(const float *__restrict__ khi, const float *__restrict__ klo, const float *__restrict__ shi, const float *__restrict__ slo, const float *__restrict__ yhi, const float *__restrict__ ylo, float *__restrict__ fhi, float *__restrict__ flo) {\n");
    fprintf(f, "        Df acc[%u];\n", n);
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        acc[%u] = Df{shi[%u], slo[%u]};\n", s, s, s);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        fprintf(f, "        { Df rate = Df{khi[%u], klo[%u]};\n", r, r);
        for (uint32_t q : rx.reactants) fprintf(f, "          rate = df_mul(rate, Df{yhi[%u], ylo[%u]});\n", q, q);
        for (auto &e : rx.net) {
            int c = e.second;
            if (c == 1) fprintf(f, "          acc[%u] = df_add(acc[%u], rate);\n", e.first, e.first);
            else if (c == -1 || c == 2 || c == -2 || c == 4 || c == -4)
                fprintf(f, "          acc[%u] = df_add(acc[%u], df_scale(rate, %d.0f));\n", e.first, e.first, c);
            else fprintf(f, "          acc[%u] = df_add(acc[%u], df_mul(rate, Df{%d.0f, 0.0f}));\n", e.first, e.first, c);
        }
        fprintf(f, "        }\n");
    }
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        fhi[%u] = acc[%u].hi; flo[%u] = acc[%u].lo;\n", s, s, s, s);
    fprintf(f, "    }\n\n");

    // mixed variant 2: the refinement residual r = b - ghinv x + J(y) x in lazily normalised
    // double-float, accumulated per species from b - ghinv x through J x's terms reaction by
    // reaction: d rate_r = sum_p k_r (prod_{q != p} y_q) x_p, each term multiplied out from k_r
    // (keeps products of large number densities in FP32 range), then r_s += net_{r,s} d rate_r;
    // out: the FP32 rounding of r, the right-hand side of the correction solve
    fprintf(f, "    static __device__ __forceinline__ void residual_df(const float *__restrict__ khi, const float *__restrict__ klo, const float *__restrict__ yhi, const float *__restrict__ ylo, const float *__restrict__ x, const float *__restrict__ bhi, const float *__restrict__ blo, Df g, float *__restrict__ r) {\n");
    fprintf(f, "        Df acc[%u];\n", n);
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        acc[%u] = df_acc(Df{bhi[%u], blo[%u]}, df_neg(df_mul_fu(g, x[%u])));\n", s, s, s, s);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        if (rx.reactants.empty()) continue;
        fprintf(f, "        { Df drate;\n");
        for (size_t p = 0; p < rx.reactants.size(); ++p) {
            fprintf(f, "          { Df t = Df{khi[%u], klo[%u]};", r, r);
            for (size_t q = 0; q < rx.reactants.size(); ++q)
                if (q != p) fprintf(f, " t = df_mul_u(t, Df{yhi[%u], ylo[%u]});", rx.reactants[q], rx.reactants[q]);
            fprintf(f, " t = df_mul_fu(t, x[%u]);", rx.reactants[p]);
            fprintf(f, p == 0 ? " drate = t; }\n" : " drate = df_acc(drate, t); }\n");
        }
        for (auto &e : rx.net) emit_lazy_term(f, e.first, e.second, "drate");
        fprintf(f, "        }\n");
    }
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        r[%u] = acc[%u].hi + acc[%u].lo;\n", s, s, s);
    fprintf(f, "    }\n\n");

    // fun in lazily normalised double-float (mixed variant 2): fun_df's terms in fun_df's order
    fprintf(f, "    static __device__ __forceinline__ void fun_dfl(const float *__restrict__ khi, const float *__restrict__ klo, const float *__restrict__ shi, const float *__restrict__ slo, const float *__restrict__ yhi, const float *__restrict__ ylo, float *__restrict__ fhi, float *__restrict__ flo) {\n");
    fprintf(f, "        Df acc[%u];\n", n);
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        acc[%u] = Df{shi[%u], slo[%u]};\n", s, s, s);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        fprintf(f, "        { Df rate = Df{khi[%u], klo[%u]};\n", r, r);
        for (uint32_t q : rx.reactants) fprintf(f, "          rate = df_mul_u(rate, Df{yhi[%u], ylo[%u]});\n", q, q);
        for (auto &e : rx.net) emit_lazy_term(f, e.first, e.second, "rate");
        fprintf(f, "        }\n");
    }
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        { const Df v = df_norm(acc[%u]); fhi[%u] = v.hi; flo[%u] = v.lo; }\n", s, s, s);
    fprintf(f, "    }\n\n");

    // mixed path: FP32 RHS increment f(y + d) - f(y) from the exact expansion
    // prod(y_q + d_q) - prod(y_q) = sum_p k d_p prod_{q<p} y_q prod_{q>p} (y_q + d_q)
    fprintf(f, "    static __device__ __forceinline__ void fun_delta(const float *__restrict__ k, const float *__restrict__ y, const float *__restrict__ d, float *__restrict__ df) {\n");
    for (uint32_t s = 0; s < n; ++s) fprintf(f, "        df[%u] = 0.0f;\n", s);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        fprintf(f, "        { float rate = 0.0f;\n");
        for (size_t p = 0; p < rx.reactants.size(); ++p) {
            fprintf(f, "          { float term = k[%u] * d[%u];", r, rx.reactants[p]);
            for (size_t q = 0; q < p; ++q) fprintf(f, " term = term * y[%u];", rx.reactants[q]);
            for (size_t q = p + 1; q < rx.reactants.size(); ++q) fprintf(f, " term = term * (y[%u] + d[%u]);", rx.reactants[q], rx.reactants[q]);
            fprintf(f, " rate = rate + term; }\n");
        }
        for (auto &e : rx.net) fprintf(f, "          df[%u] = fmaf(%d.0f, rate, df[%u]);\n", e.first, e.second, e.first);
        fprintf(f, "        }\n");
    }
    fprintf(f, "    }\n\n");

    // -J into the compact LU storage
    // LU storage element e of a lane lives at a[e * S]: S = 1 for a per-lane array, or the CTA's
    // thread count for shared-memory storage interleaved across the CTA's lanes
    fprintf(f, "    template <class T, int S = 1>\n    static __device__ __forceinline__ void neg_jac(const T *__restrict__ k, const T *__restrict__ y, T *__restrict__ a) {\n");
    std::vector<uint8_t> written(S.nnz, 0);
    std::vector<std::string> body;
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        for (size_t p = 0; p < rx.reactants.size(); ++p) {
            fprintf(f, "        { T d = k[%u]", r);
            for (size_t q = 0; q < rx.reactants.size(); ++q)
                if (q != p) fprintf(f, " * y[%u]", rx.reactants[q]);
            fprintf(f, ";\n");
            for (size_t e = 0; e < rx.net.size(); ++e) {
                int c = -rx.net[e].second;
                uint32_t idx = rx.jac_slot[p][e];
                if (!written[idx] && (c == 1 || c == -1))
                    fprintf(f, "          a[%u * S] = %s(d);\n", idx, c == 1 ? "sgb_first_pos" : "sgb_first_neg");
                else if (!written[idx])
                    fprintf(f, "          a[%u * S] = sgb_fma((T)%d.0, d, (T)0.0);\n", idx, c);
                else
                    fprintf(f, "          a[%u * S] = sgb_fma((T)%d.0, d, a[%u * S]);\n", idx, c, idx);
                written[idx] = 1;
            }
            fprintf(f, "        }\n");
        }
    }
    for (uint32_t i = 0; i < S.nnz; ++i)
        if (!written[i]) fprintf(f, "        a[%u * S] = (T)0.0;\n", i);
    fprintf(f, "    }\n\n");

    // in-place no-pivot LU of I*ghinv - J; the diagonal keeps 1/U(i,i)
    fprintf(f, "    template <class T, int S = 1>\n    static __device__ __forceinline__ void factor(T ghinv, T *__restrict__ a) {\n");
    for (uint32_t i = 0; i < n; ++i) {
        for (uint32_t d = S.div_begin[i]; d < S.div_begin[i + 1]; ++d) {
            const Symbolic::Div &dv = S.divs[d];
            fprintf(f, "        { const T l = a[%u * S] * a[%u * S]; a[%u * S] = l;\n", dv.ik, dv.kk, dv.ik);
            for (uint32_t s = dv.sub_begin; s < dv.sub_end; ++s)
                fprintf(f, "          a[%u * S] = sgb_fma(-l, a[%u * S], a[%u * S]);\n", S.subs[s].ij, S.subs[s].kj, S.subs[s].ij);
            fprintf(f, "        }\n");
        }
        fprintf(f, "        a[%u * S] = (T)1.0 / (a[%u * S] + ghinv);\n", S.diag[i], S.diag[i]);
    }
    fprintf(f, "    }\n\n");

    // forward (unit L, ascending column) and backward (U, descending column)
    fprintf(f, "    template <class T, int S = 1>\n    static __device__ __forceinline__ void solve(const T *__restrict__ a, T *__restrict__ x) {\n");
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t e = S.lower_begin[i]; e < S.lower_begin[i + 1]; ++e)
            fprintf(f, "        x[%u] = sgb_fma(-a[%u * S], x[%u], x[%u]);\n", i, S.lower[e].index, S.lower[e].col, i);
    for (uint32_t ii = n; ii-- > 0;) {
        for (uint32_t e = S.upper_begin[ii]; e < S.upper_begin[ii + 1]; ++e)
            fprintf(f, "        x[%u] = sgb_fma(-a[%u * S], x[%u], x[%u]);\n", ii, S.upper[e].index, S.upper[e].col, ii);
        fprintf(f, "        x[%u] = x[%u] * a[%u * S];\n", ii, ii, S.diag[ii]);
    }
    fprintf(f, "    }\n\n");

    // mixed path: keep -J's pattern entries, widened to FP64 once per step, before the factorisation
    fprintf(f, "    static __device__ __forceinline__ void save_jac(const float *__restrict__ a, double *__restrict__ js) {\n");
    for (size_t q = 0; q < jslots.size(); ++q) fprintf(f, "        js[%zu] = (double)a[%u];\n", q, jslots[q]);
    fprintf(f, "    }\n\n");
    // r = b - W x = b - ghinv x - (-J) x, in FP64 (the -J entries are exact FP32 values)
    fprintf(f, "    static __device__ __forceinline__ void residual(const double *__restrict__ js, double ghinv, const double *__restrict__ b, const double *__restrict__ x, double *__restrict__ r) {\n");
    for (uint32_t i = 0; i < n; ++i) {
        fprintf(f, "        { double acc = sgb_fma(-ghinv, x[%u], b[%u]);\n", i, i);
        for (size_t q = 0; q < jslots.size(); ++q)
            if (jrow[q] == i) fprintf(f, "          acc = sgb_fma(-js[%zu], x[%u], acc);\n", q, jcol[q]);
        fprintf(f, "          r[%u] = acc; }\n", i);
    }
    fprintf(f, "    }\n");
    fprintf(f, "};\n\n");
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: kin_codegen out.cuh\n");
        return 1;
    }
    Model air;
    define_air(&air);
    if (!air.finalize()) {
        fprintf(stderr, "kin_codegen: mechanism error: %s\n", air.error.c_str());
        return 1;
    }
    std::string tmp = std::string(argv[1]) + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) {
        fprintf(stderr, "kin_codegen: cannot write %s\n", tmp.c_str());
        return 1;
    }
    fprintf(f, "// GENERATED by simstack_gb300/csrc/kin_codegen.cpp -- do not edit.\n");
    fprintf(f, "// Straight-line solver kernels for the shipped humid-air mechanism.\n");
    fprintf(f, "#pragma once\n\n");
    emit_ops(f, air, "AirOps");
    fclose(f);
    // replace only when changed, so unchanged builds stay unchanged
    FILE *old = fopen(argv[1], "rb"), *nw = fopen(tmp.c_str(), "rb");
    bool same = old != nullptr;
    if (old) {
        for (;;) {
            int a = fgetc(old), b = fgetc(nw);
            if (a != b) { same = false; break; }
            if (a == EOF) break;
        }
        fclose(old);
    }
    fclose(nw);
    if (same) remove(tmp.c_str());
    else rename(tmp.c_str(), argv[1]);
    return 0;
}
