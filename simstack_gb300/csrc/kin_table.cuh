// Table-driven mechanism ops: any mechanism that fits the reference's KinMech
// capacities (32 species, 96 reactions, 512 non-zeros), walking its index
// tables in the reference's order (src/sim/kinetics/kin_solver.h:40-139).
// The KinMech image is staged once per CTA from global into shared memory with
// a TMA bulk copy (cp.async.bulk + mbarrier); every thread then reads the same
// table entries (broadcast, no bank conflicts).

#pragma once
#include "kin_device.cuh"

namespace sgb {

// Staged image: the KinMech record, then a bitmask of the compact slots that
// belong to the Jacobian's own pattern (before fill-in), used by the mixed
// path's residual.
constexpr uint32_t kJacMaskOffset = (uint32_t)((sizeof(KinMech) + 15) / 16 * 16);
constexpr uint32_t kTableBytes = kJacMaskOffset + KIN_MAX_NNZ / 8;

struct TableOps {
    static constexpr int N = KIN_MAX_SPECIES, R = KIN_MAX_REACTIONS, NNZ = KIN_MAX_NNZ, NJ = KIN_MAX_NNZ;
    static constexpr bool kStridedLu = false;   // shared memory holds the staged tables
    const KinMech *m;

    __device__ __forceinline__ uint32_t n() const { return m->species_count; }
    __device__ __forceinline__ uint32_t r() const { return m->reaction_count; }

    // Stages the tables; every thread of the CTA calls it. False if the bounded
    // wait for the copy ran out (the caller then records the error and returns).
    __device__ bool init(const DevArgs &A, unsigned char *smem) {
        __shared__ __align__(8) uint64_t bar;
        m = (const KinMech *)smem;
        if (threadIdx.x == 0) {
            mbar_init(&bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_arrive_expect_tx(&bar, A.table_bytes);
            tma_bulk_g2s(smem, A.tables, A.table_bytes, &bar);
        }
        const bool ok = mbar_wait(&bar, 0, A.wait_polls);
        // on a timeout the copy may still be in flight into this CTA's shared memory:
        // let it land (a second bounded wait) before the CTA gives up and exits
        if (!ok) mbar_wait(&bar, 0);
        __syncthreads();
        return ok;
    }

    template <class T> __device__ __forceinline__ void fun(const T *k, const T *src, const T *y, T *f) const {
        const uint32_t ns = m->species_count, nr = m->reaction_count;
        for (uint32_t s = 0; s < ns; ++s) f[s] = src[s];
        for (uint32_t r = 0; r < nr; ++r) {
            const KinReaction &rx = m->reactions[r];
            T rate = k[r];
            for (uint32_t p = 0; p < rx.reactant_count; ++p) rate = rate * y[rx.reactant[p]];
            for (uint32_t e = 0; e < rx.net_count; ++e) {
                uint32_t s = rx.net_species[e];
                f[s] = sgb_fma((T)(double)rx.net_coef[e], rate, f[s]);
            }
        }
    }

    template <class T> __device__ __forceinline__ void neg_jac(const T *k, const T *y, T *a) const {
        const uint32_t nz = m->nnz, nr = m->reaction_count;
        for (uint32_t i = 0; i < nz; ++i) a[i] = (T)0.0;
        for (uint32_t r = 0; r < nr; ++r) {
            const KinReaction &rx = m->reactions[r];
            for (uint32_t p = 0; p < rx.reactant_count; ++p) {
                T d = k[r];
                for (uint32_t q = 0; q < rx.reactant_count; ++q)
                    if (q != p) d = d * y[rx.reactant[q]];
                for (uint32_t e = 0; e < rx.net_count; ++e) {
                    uint32_t idx = rx.jac_index[p][e];
                    a[idx] = sgb_fma((T)(-(double)rx.net_coef[e]), d, a[idx]);
                }
            }
        }
    }

    template <class T> __device__ __forceinline__ void factor(T ghinv, T *a) const {
        const uint32_t ns = m->species_count;
        for (uint32_t i = 0; i < ns; ++i) {
            for (uint32_t d = m->div_begin[i]; d < m->div_begin[i + 1]; ++d) {
                const KinLuDiv dv = m->lu_div[d];
                T l = a[dv.ik] * a[dv.kk];
                a[dv.ik] = l;
                for (uint32_t s = dv.sub_begin; s < dv.sub_end; ++s) {
                    const KinLuSub sb = m->lu_sub[s];
                    a[sb.ij] = sgb_fma(-l, a[sb.kj], a[sb.ij]);
                }
            }
            uint32_t ii = m->diag[i];
            a[ii] = (T)1.0 / (a[ii] + ghinv);
        }
    }

    template <class T> __device__ __forceinline__ void solve(const T *a, T *x) const {
        const uint32_t ns = m->species_count;
        for (uint32_t i = 0; i < ns; ++i)
            for (uint32_t e = m->lower_begin[i]; e < m->lower_begin[i + 1]; ++e) {
                const KinRowEntry le = m->lower[e];
                x[i] = sgb_fma(-a[le.index], x[le.col], x[i]);
            }
        for (uint32_t ii = ns; ii-- > 0;) {
            for (uint32_t e = m->upper_begin[ii]; e < m->upper_begin[ii + 1]; ++e) {
                const KinRowEntry ue = m->upper[e];
                x[ii] = sgb_fma(-a[ue.index], x[ue.col], x[ii]);
            }
            x[ii] = x[ii] * a[m->diag[ii]];
        }
    }

    // Double-float RHS in the generated code's order (kin_codegen.cpp, fun_df).
    __device__ __forceinline__ void fun_df(const float *khi, const float *klo, const float *shi, const float *slo, const float *yhi,
                                           const float *ylo, float *fhi, float *flo) const {
        const uint32_t ns = m->species_count, nr = m->reaction_count;
        for (uint32_t s = 0; s < ns; ++s) {
            fhi[s] = shi[s];
            flo[s] = slo[s];
        }
        for (uint32_t r = 0; r < nr; ++r) {
            const KinReaction &rx = m->reactions[r];
            Df rate{khi[r], klo[r]};
            for (uint32_t p = 0; p < rx.reactant_count; ++p) rate = df_mul(rate, Df{yhi[rx.reactant[p]], ylo[rx.reactant[p]]});
            for (uint32_t e = 0; e < rx.net_count; ++e) {
                const uint32_t s = rx.net_species[e];
                const int c = rx.net_coef[e];
                Df term = c == 1 ? rate
                          : (c == -1 || c == 2 || c == -2 || c == 4 || c == -4) ? df_scale(rate, (float)c)
                                                                                 : df_mul(rate, Df{(float)c, 0.0f});
                const Df acc = df_add(Df{fhi[s], flo[s]}, term);
                fhi[s] = acc.hi;
                flo[s] = acc.lo;
            }
        }
    }

    // acc += c * v, lazily normalised (kin_codegen.cpp, emit_lazy_term)
    __device__ __forceinline__ static Df lazy_term(Df acc, Df v, int c) {
        if (c == 1) return df_acc(acc, v);
        if (c == -1 || c == 2 || c == -2 || c == 4 || c == -4) return df_acc(acc, df_scale(v, (float)c));
        return df_acc(acc, df_mul_u(v, Df{(float)c, 0.0f}));
    }

    // f(y) in lazily normalised double-float in the generated code's order (kin_codegen.cpp, fun_dfl).
    __device__ __forceinline__ void fun_dfl(const float *khi, const float *klo, const float *shi, const float *slo, const float *yhi,
                                            const float *ylo, float *fhi, float *flo) const {
        const uint32_t ns = m->species_count, nr = m->reaction_count;
        for (uint32_t s = 0; s < ns; ++s) {
            fhi[s] = shi[s];
            flo[s] = slo[s];
        }
        for (uint32_t r = 0; r < nr; ++r) {
            const KinReaction &rx = m->reactions[r];
            Df rate{khi[r], klo[r]};
            for (uint32_t p = 0; p < rx.reactant_count; ++p) rate = df_mul_u(rate, Df{yhi[rx.reactant[p]], ylo[rx.reactant[p]]});
            for (uint32_t e = 0; e < rx.net_count; ++e) {
                const uint32_t s = rx.net_species[e];
                const Df acc = lazy_term(Df{fhi[s], flo[s]}, rate, rx.net_coef[e]);
                fhi[s] = acc.hi;
                flo[s] = acc.lo;
            }
        }
        for (uint32_t s = 0; s < ns; ++s) {
            const Df v = df_norm(Df{fhi[s], flo[s]});
            fhi[s] = v.hi;
            flo[s] = v.lo;
        }
    }

    // r = b - ghinv x + J(y) x in lazily normalised double-float, out as FP32, in the generated
    // code's order (kin_codegen.cpp, residual_df).
    __device__ __forceinline__ void residual_df(const float *khi, const float *klo, const float *yhi, const float *ylo, const float *x,
                                                const float *bhi, const float *blo, Df g, float *r) const {
        const uint32_t ns = m->species_count, nr = m->reaction_count;
        float ahi[KIN_MAX_SPECIES], alo[KIN_MAX_SPECIES];
        for (uint32_t s = 0; s < ns; ++s) {
            const Df a = df_acc(Df{bhi[s], blo[s]}, df_neg(df_mul_fu(g, x[s])));
            ahi[s] = a.hi;
            alo[s] = a.lo;
        }
        for (uint32_t q = 0; q < nr; ++q) {
            const KinReaction &rx = m->reactions[q];
            if (rx.reactant_count == 0) continue;
            Df drate{0.0f, 0.0f};
            for (uint32_t p = 0; p < rx.reactant_count; ++p) {
                Df t{khi[q], klo[q]};
                for (uint32_t o = 0; o < rx.reactant_count; ++o)
                    if (o != p) t = df_mul_u(t, Df{yhi[rx.reactant[o]], ylo[rx.reactant[o]]});
                t = df_mul_fu(t, x[rx.reactant[p]]);
                drate = p == 0 ? t : df_acc(drate, t);
            }
            for (uint32_t e = 0; e < rx.net_count; ++e) {
                const uint32_t s = rx.net_species[e];
                const Df a = lazy_term(Df{ahi[s], alo[s]}, drate, rx.net_coef[e]);
                ahi[s] = a.hi;
                alo[s] = a.lo;
            }
        }
        for (uint32_t s = 0; s < ns; ++s) r[s] = ahi[s] + alo[s];
    }

    __device__ __forceinline__ bool in_jac(uint32_t slot) const {
        const uint8_t *mask = (const uint8_t *)m + kJacMaskOffset;
        return (mask[slot >> 3] >> (slot & 7)) & 1u;
    }

    // FP32 RHS increment at y + d (kin_codegen.cpp, fun_delta).
    __device__ __forceinline__ void fun_delta(const float *k, const float *y, const float *d, float *df) const {
        const uint32_t ns = m->species_count, nr = m->reaction_count;
        for (uint32_t s = 0; s < ns; ++s) df[s] = 0.0f;
        for (uint32_t r = 0; r < nr; ++r) {
            const KinReaction &rx = m->reactions[r];
            float rate = 0.0f;
            for (uint32_t p = 0; p < rx.reactant_count; ++p) {
                float term = k[r] * d[rx.reactant[p]];
                for (uint32_t q = 0; q < p; ++q) term = term * y[rx.reactant[q]];
                for (uint32_t q = p + 1; q < rx.reactant_count; ++q) term = term * (y[rx.reactant[q]] + d[rx.reactant[q]]);
                rate = rate + term;
            }
            for (uint32_t e = 0; e < rx.net_count; ++e) df[rx.net_species[e]] = fmaf((float)rx.net_coef[e], rate, df[rx.net_species[e]]);
        }
    }

    // Mixed path: keep all of -J (fill-in slots are zero), widened to FP64, before the factorisation.
    __device__ __forceinline__ void save_jac(const float *a, double *js) const {
        const uint32_t nz = m->nnz;
        for (uint32_t i = 0; i < nz; ++i) js[i] = (double)a[i];
    }

    // r = b - ghinv x - (-J) x in FP64, over each row's Jacobian-pattern
    // entries in ascending column order (the generated code's order).
    __device__ __forceinline__ void residual(const double *js, double ghinv, const double *b, const double *x, double *r) const {
        const uint32_t ns = m->species_count;
        for (uint32_t i = 0; i < ns; ++i) {
            double acc = sgb_fma(-ghinv, x[i], b[i]);
            for (uint32_t e = m->lower_begin[i]; e < m->lower_begin[i + 1]; ++e)
                if (in_jac(m->lower[e].index)) acc = sgb_fma(-js[m->lower[e].index], x[m->lower[e].col], acc);
            acc = sgb_fma(-js[m->diag[i]], x[i], acc);
            for (uint32_t e = m->upper_begin[i + 1]; e-- > m->upper_begin[i];)
                if (in_jac(m->upper[e].index)) acc = sgb_fma(-js[m->upper[e].index], x[m->upper[e].col], acc);
            r[i] = acc;
        }
    }
};

}   // namespace sgb
