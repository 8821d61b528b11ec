// Cooperative kernels for large mechanisms: one CTA integrates one cell at a
// time (persistent CTAs take cells from a work queue), its threads splitting
// every phase of the Rosenbrock step -- rates per reaction, RHS per species,
// Jacobian per entry, elimination per (row, column) of each pivot (two pivots
// per pass for an FP64 LU in global memory), solves per row of each column. The step control is the reference's
// (src/sim/kinetics/kin_solver.h:189-345): every thread runs the scalar
// controller on the same values, so its decisions are uniform across the CTA.
//
// Precision 0: FP64 throughout, the same bits as the reference's solver (each
// element sees the reference's operations in the reference's order; see
// coop.h). The dense LU lives in per-CTA global scratch (L2-resident), or in
// shared memory when it fits in 64 KB; the pattern bitmask, vectors and rates
// live in shared memory.
// Precision 2 (mixed): FP64 RHS, Jacobian, residual, state and control; the
// LU and the triangular solves in FP32 with the dense LU in shared memory;
// each stage solve refined with FP64 residual sweeps.

#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "../../include/simstack_gpu.h"
#include "coop.h"
#include "kin_device.cuh"
#include "mech.h"

namespace sgb {

namespace {

constexpr uint32_t kCoopMaxSpecies = 256;   // register cache of a pivot row: 8 columns per lane
constexpr size_t kCoopSmemLuF64Max = 64 * 1024;   // FP64 LUs up to this size live in shared memory (n <= ~90)
constexpr uint32_t kCoopMaxCols = kCoopMaxSpecies / 32;

struct CoopTab {
    const CoopMech *h;
    const uint16_t *reac;
    const uint32_t *fbeg, *jbeg, *jpos, *jrow, *lbeg, *ubeg, *cbeg;
    const CoopTerm *fent, *jent;
    const uint16_t *jcol, *lrow, *ucol, *crow;

    __device__ __forceinline__ void init(const void *image) {
        const unsigned char *b = (const unsigned char *)image;
        h = (const CoopMech *)b;
        reac = (const uint16_t *)(b + h->off_reac);
        fbeg = (const uint32_t *)(b + h->off_fbeg);
        fent = (const CoopTerm *)(b + h->off_fent);
        jbeg = (const uint32_t *)(b + h->off_jbeg);
        jent = (const CoopTerm *)(b + h->off_jent);
        jpos = (const uint32_t *)(b + h->off_jpos);
        jrow = (const uint32_t *)(b + h->off_jrow);
        jcol = (const uint16_t *)(b + h->off_jcol);
        lbeg = (const uint32_t *)(b + h->off_lbeg);
        lrow = (const uint16_t *)(b + h->off_lrow);
        ubeg = (const uint32_t *)(b + h->off_ubeg);
        ucol = (const uint16_t *)(b + h->off_ucol);
        cbeg = (const uint32_t *)(b + h->off_cbeg);
        crow = (const uint16_t *)(b + h->off_crow);
    }
};

// Build-time phase timing (-DSGB_COOP_PROFILE): thread 0 of every CTA adds the
// clock cycles of each phase to g_coop_phase_cycles (rhs, Jacobian, factor,
// solves, refinement residual, total attempt).
#ifdef SGB_COOP_PROFILE
__device__ unsigned long long g_coop_phase_cycles[8];
#define SGB_PHASE(i, stmt)                                                      \
    do {                                                                        \
        const long long _t0 = clock64();                                       \
        stmt;                                                                   \
        if (tid == 0) atomicAdd(&g_coop_phase_cycles[i], (unsigned long long)(clock64() - _t0)); \
    } while (0)
#else
#define SGB_PHASE(i, stmt) stmt
#endif

// Pivots per elimination pass of the FP64 factorisation with its LU in global memory (1, 2 or 4;
// the same bits for any). Measured on 200 species / 1,200 reactions, 1,216 cells x 2 s, 256
// threads x 2 CTAs per SM: 1 -> 6,817 ms, 2 -> 5,805 ms, 4 -> 6,272 ms (the one-warp panel grows).
// The shared-memory LUs (FP64 of small mechanisms, the mixed path's FP32) stay pivot by pivot:
// the mixed kernel measured 2,392 ms pivot by pivot against 2,745 (2) and 2,630 (4).
#ifndef SGB_COOP_PIVOT_BLOCK
#define SGB_COOP_PIVOT_BLOCK 2
#endif

// Shared-memory doubles before the mixed path's FP32 arrays.
__host__ __device__ inline uint32_t coop_smem_doubles(uint32_t n, uint32_t R) { return 11u * n + 2u * R + 8u; }

// Default budget up to which the term lists join shared memory: none. Measured on the 200-species
// FP64 case, staging them (149 KB of shared memory per CTA) made the step 1.31x slower, because the
// smaller L1 then caches less of the global-memory LU; callers may enable it per precision.
constexpr uint32_t kCoopSmemBudget = 0;

// Shared memory of one CTA: doubles, x32 (256 floats), pattern (n x 8 words), lcnt (n u16,
// padded), then the LU (mixed always, n x ld floats; FP64 when it fits kCoopSmemLuF64Max), then
// -- when they fit the budget -- the RHS / Jacobian term lists (image bytes [off_reac, off_lbeg)).
struct CoopSmemLayout {
    size_t lu, lu_bytes, terms, terms_bytes, total;
};
__host__ __device__ inline CoopSmemLayout coop_layout(int prec, const CoopMech &h, uint32_t budget) {
    CoopSmemLayout L;
    L.lu = (size_t)coop_smem_doubles(h.n, h.R) * 8 + kCoopMaxSpecies * 4 + (size_t)h.n * 32 + ((h.n + 7) / 8) * 16;
    const size_t lu64 = (size_t)h.n * h.ld * sizeof(double);
    L.lu_bytes = prec == 2 ? (size_t)h.n * h.ld * 4 : (lu64 <= kCoopSmemLuF64Max ? lu64 : 0);
    L.terms = (L.lu + L.lu_bytes + 15) / 16 * 16;
    const size_t tb = (size_t)h.off_lbeg - h.off_reac;
    L.terms_bytes = L.terms + tb <= budget ? tb : 0;
    L.total = L.terms + L.terms_bytes;
    return L;
}

template <int PREC>
struct CoopCell {
    typedef typename Pick<PREC == 0, double, float>::type Cf;   // LU and solve arithmetic
    static constexpr bool kMixed = PREC == 2;
    typedef RuntimeCoef M;

    CoopTab tb;
    uint32_t n, R, ld, nj, tid, NT, lane, warp, W;
    double *y, *ytmp, *fcn, *src, *qv, *rb, *xv, *K, *kr, *rate, *red;
    float *x32;
    Cf *a;          // dense LU [n][ld]
    bool lu_global;         // eliminate with loads before stores (the LU lives in global scratch: FP64, large)
    const uint32_t *pat;    // shared: filled pattern, 8 words per row
    const uint16_t *lcnt;   // shared: rows below the diagonal per column
    double *js;     // mixed: Jacobian entries (a = -J) in FP64
    // replicated scalar state (kin_solver.h:189-345)
    double t, h, seg_end, applied, duration, period, first, count, steps, rejects, pulses, failed;
    uint32_t iterations, transitions;
    int phase;
    bool pending, reject_last, reject_more;

    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ bool bit(uint32_t i, uint32_t j) const { return (pat[i * 8u + (j >> 5)] >> (j & 31u)) & 1u; }

    __device__ void load(const DevArgs &A, uint32_t cell) {
        const uint32_t p = A.padded;
        for (uint32_t s = tid; s < n; s += NT) {
            y[s] = A.y[(size_t)s * p + cell];
            src[s] = A.src[(size_t)s * p + cell];
        }
        for (uint32_t r = tid; r < R; r += NT) kr[r] = A.k[(size_t)r * p + cell];
        h = A.h[cell];
        period = A.period[cell];
        first = A.pulse_first[cell];
        count = A.pulse_count[cell];
        duration = A.duration;
        steps = rejects = pulses = 0.0;
        failed = A.failed[cell];
        t = 0.0;
        applied = 0.0;
        transitions = 0;
        phase = kPhaseSegStart;
        sync();
    }

    // A parked cell: its scalar state from the record (load() read y, k, src and failed).
    __device__ void restore(const SuspendRec &r) {
        t = r.t;
        h = r.h;
        seg_end = r.seg_end;
        applied = r.applied;
        pending = (r.flags & 1u) != 0;
        reject_last = (r.flags & 2u) != 0;
        reject_more = (r.flags & 4u) != 0;
        iterations = r.iterations;
        transitions = r.transitions;
        phase = kPhaseStepping;
    }

    __device__ void store(const DevArgs &A, uint32_t cell) {
        const uint32_t p = A.padded;
        for (uint32_t s = tid; s < n; s += NT) A.y[(size_t)s * p + cell] = y[s];
        if (tid == 0) {
            A.h[cell] = h;
            A.failed[cell] = failed;
            A.steps[cell] += steps;
            A.rejects[cell] += rejects;
            A.pulses[cell] += pulses;
        }
        sync();
    }

    __device__ void seg_start(const DevArgs &A) {
        pending = applied < count;
        double next_pulse = sgb_fma(applied, period, first);
        seg_end = pending ? vmin(next_pulse, duration) : duration;
        bool active = t < seg_end && !(failed > 0.0);
        reject_last = false;
        reject_more = false;
        h = h > 0.0 ? h : A.ctl.h_start;
        iterations = 0;
        phase = active ? kPhaseStepping : kPhaseSegFinish;
    }

    __device__ void seg_finish(const DevArgs &A, uint32_t cell) {
        bool alive = !(failed > 0.0);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            const uint32_t p = A.padded;
            for (uint32_t s = tid; s < n; s += NT) y[s] = y[s] + A.pulse[(size_t)s * p + cell];
            sync();
            applied = applied + 1.0;
            pulses = pulses + 1.0;
            h = A.ctl.h_start;
        }
        bool done = (t >= duration && applied >= count) || !alive;
        phase = done ? kPhaseDone : kPhaseSegStart;
    }

    // As the lane kernels' settle: transitions until a step attempt is due (true) or the cell is done.
    __device__ bool settle(const DevArgs &A, uint32_t cell) {
        for (;;) {
            if (++transitions > (1u << 24)) {
                failed = 1.0;
                phase = kPhaseDone;
            }
            switch (phase) {
                case kPhaseSegStart: seg_start(A); break;
                case kPhaseSegFinish: seg_finish(A, cell); break;
                case kPhaseStepping:
                    if (++iterations > A.ctl.max_steps) {
                        failed = 1.0;
                        phase = kPhaseSegFinish;
                        break;
                    }
                    return true;
                default: return false;
            }
        }
    }

    // fcn = f(yy): rates per reaction, then each species' terms in reaction order.
    __device__ void rhs(const double *yy) {
        for (uint32_t r = tid; r < R; r += NT) {
            const uint16_t *rc = tb.reac + (size_t)r * 4;
            double v = kr[r];
            for (uint32_t p = 0; p < rc[0]; ++p) v = v * yy[rc[1 + p]];
            rate[r] = v;
        }
        sync();
        for (uint32_t s = tid; s < n; s += NT) {
            double f = src[s];
            for (uint32_t e = tb.fbeg[s]; e < tb.fbeg[s + 1]; ++e) {
                const CoopTerm term = tb.fent[e];
                f = sgb_fma((double)term.coef, rate[term.index], f);
            }
            fcn[s] = f;
        }
        sync();
    }

    // a = -J at yy (zero elsewhere); mixed: the FP64 entries also kept in js.
    __device__ void neg_jac(const double *yy) {
        const uint32_t total = n * ld;
        for (uint32_t q = tid; q < total; q += NT) a[q] = (Cf)0.0;
        sync();
        for (uint32_t e = tid; e < nj; e += NT) {
            double acc = 0.0;
            for (uint32_t q = tb.jbeg[e]; q < tb.jbeg[e + 1]; ++q) {
                const CoopTerm term = tb.jent[q];
                const uint32_t r = term.index & 0xffffffu, p = term.index >> 24;
                const uint16_t *rc = tb.reac + (size_t)r * 4;
                double d = kr[r];
                for (uint32_t o = 0; o < rc[0]; ++o)
                    if (o != p) d = d * yy[rc[1 + o]];
                acc = sgb_fma((double)term.coef, d, acc);
            }
            if constexpr (kMixed) js[e] = acc;
            a[tb.jpos[e]] = (Cf)acc;
        }
        sync();
    }

    // In place: a -> L\U of (I ghinv - J), diagonal holding 1/U(k,k); pivot by
    // pivot (kin_solver.h:97-113 applies the same updates row by row). Rows and
    // columns are walked densely; the pattern bits select the elements the
    // reference updates. The warp that updates row i also forms its multiplier
    // l(i,k) = a[i][k] * (1/U(k,k)) and stores it once the row is done, so a pivot
    // needs one barrier (FP32) or two (FP64: the shared inverse).
    __device__ void factor(Cf ghinv) {
#if SGB_COOP_PIVOT_BLOCK > 1
        if (!kMixed && lu_global) {
            factor_block<SGB_COOP_PIVOT_BLOCK>(ghinv);
            return;
        }
#endif
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t nl = lcnt[k];
            Cf inv;
            if constexpr (kMixed) {
                // FP32: every thread divides (cheap on the FP32 pipe); the inverted diagonal is
                // stored after the pivot's closing barrier, once every thread has read a[k][k]
                if (nl == 0) {   // nothing below the pivot: the next pivot reads none of this pivot's writes
                    if (tid == 0) a[(size_t)k * ld + k] = (Cf)1.0 / (a[(size_t)k * ld + k] + ghinv);
                    continue;
                }
                inv = (Cf)1.0 / (a[(size_t)k * ld + k] + ghinv);
            } else {
                // FP64: 1/U(k,k) once (a division costs many FP64 instructions per warp), shared through red[4]
                Cf *inv_s = (Cf *)(red + 4);
                if (tid == 0) {
                    const Cf v = (Cf)1.0 / (a[(size_t)k * ld + k] + ghinv);
                    a[(size_t)k * ld + k] = v;
                    *inv_s = v;
                }
                if (nl == 0) continue;
                sync();
                inv = *inv_s;
            }
            // pivot row k (final) cached per lane: columns k+1+lane+32c in the pattern
            const uint32_t width = n - 1 - k, chunks = (width + 31) / 32;
            Cf pv[kCoopMaxCols];
            uint32_t live = 0;
#pragma unroll
            for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                const uint32_t j = k + 1 + lane + 32u * c;
                const bool on = c < chunks && j < n && bit(k, j);
                pv[c] = (Cf)0.0;
                if (on) {
                    pv[c] = a[(size_t)k * ld + j];
                    live |= 1u << c;
                }
            }
            if (lu_global) {
                // global-memory LU: the row's elements first, then the updates, so the loads issue
                // back to back instead of each waiting behind the previous element's store
                for (uint32_t i = k + 1 + warp; i < n; i += W) {
                    if (!bit(i, k)) continue;   // same for the whole warp
                    Cf *row = a + (size_t)i * ld;
                    const Cf l = row[k] * inv;
                    Cf v[kCoopMaxCols];
#pragma unroll
                    for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                        const uint32_t j = k + 1 + lane + 32u * c;
                        v[c] = (Cf)0.0;
                        if ((live >> c) & 1u) v[c] = row[j];
                    }
#pragma unroll
                    for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                        const uint32_t j = k + 1 + lane + 32u * c;
                        if ((live >> c) & 1u) row[j] = sgb_fma(-l, pv[c], v[c]);
                    }
                    __syncwarp();   // every lane has read a[i][k]
                    if (lane == 0) row[k] = l;
                }
            } else {
                for (uint32_t i = k + 1 + warp; i < n; i += W) {
                    if (!bit(i, k)) continue;
                    Cf *row = a + (size_t)i * ld;
                    const Cf l = row[k] * inv;
#pragma unroll
                    for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                        const uint32_t j = k + 1 + lane + 32u * c;
                        if ((live >> c) & 1u) row[j] = sgb_fma(-l, pv[c], row[j]);
                    }
                    __syncwarp();
                    if (lane == 0) row[k] = l;
                }
            }
            sync();
            if constexpr (kMixed) {   // every thread has read a[k][k]
                if (tid == 0) a[(size_t)k * ld + k] = inv;
            }
        }
        sync();
    }

    // B pivots per pass (k .. k+B-1). Panel: warp 0 gives each row r of the block the updates of
    // the block's pivots before it, in order, then takes 1/U(r,r), and stages row r's U part in
    // shared memory. Trailing rows i >= k+B, one warp per row: the row's block entries become its
    // multipliers in order (a[i][k+p] takes the updates of pivots k+q, q < p, then the scaling by
    // 1/U(k+p,k+p)), and each a[i][j], j >= k+B, takes the block's pivots' updates in ascending
    // order, loaded once and stored once. Every element receives the operations of the pivot-by-
    // pivot order, in that order, with 1/B of the passes over the trailing rows (the LU of a large
    // mechanism lives in L2) and of the barriers. The staged rows use the stage vectors K (free
    // until the stages begin) and the inverses red[4..7], so B <= 4.
    template <uint32_t B>
    __device__ void factor_block(Cf ghinv) {
        static_assert(B >= 1 && B <= 4 && 32 % B == 0, "block of 1, 2 or 4 pivots");
        static_assert(kCoopMaxCols * B <= 32, "column masks in one word");
        Cf *inv_s = (Cf *)(red + 4);
        Cf *u = (Cf *)K;   // [B][n] staged pivot rows, zero off the pattern
        for (uint32_t k = 0; k < n; k += B) {
            const uint32_t nb = n - k < B ? n - k : B;
            if (warp == 0) {   // the panel
                for (uint32_t r = k; r < k + nb; ++r) {
                    Cf *rr = a + (size_t)r * ld;
                    for (uint32_t q = k; q < r; ++q) {
                        if (!bit(r, q)) continue;   // same for the whole warp
                        const Cf l = rr[q] * inv_s[q - k];
                        const Cf *uq = u + (size_t)(q - k) * n;
                        for (uint32_t j = q + 1 + lane; j < n; j += 32)
                            if (bit(q, j)) rr[j] = sgb_fma(-l, uq[j], rr[j]);
                        __syncwarp();
                        if (lane == 0) rr[q] = l;
                        __syncwarp();
                    }
                    if (lane == 0) {
                        const Cf v = (Cf)1.0 / (rr[r] + ghinv);
                        rr[r] = v;
                        inv_s[r - k] = v;
                    }
                    __syncwarp();
                    Cf *ur = u + (size_t)(r - k) * n;
                    for (uint32_t j = r + 1 + lane; j < n; j += 32) ur[j] = bit(r, j) ? rr[j] : (Cf)0.0;
                    __syncwarp();
                }
            }
            sync();
            const uint32_t j0 = k + nb;
            if (j0 >= n) break;
            const uint32_t bmask = (1u << nb) - 1u;
            // per lane: which block pivots update column j0 + lane + 32c (bits c*B + p)
            uint32_t live = 0;
#pragma unroll
            for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                const uint32_t j = j0 + lane + 32u * c;
                if (j >= n) continue;
#pragma unroll
                for (uint32_t p = 0; p < B; ++p)
                    if (p < nb && bit(k + p, j)) live |= 1u << (c * B + p);
            }
            // inner[p]: block pivots q < p whose row has column k+p
            uint32_t inner = 0;
#pragma unroll
            for (uint32_t p = 1; p < B; ++p)
#pragma unroll
                for (uint32_t q = 0; q < p; ++q)
                    if (p < nb && bit(k + q, k + p)) inner |= 1u << (p * B + q);
            for (uint32_t i = j0 + warp; i < n; i += W) {
                // row i's pattern bits at the block's columns (k is a multiple of B: one word)
                const uint32_t bm = (pat[i * 8u + (k >> 5)] >> (k & 31u)) & bmask;
                if (!bm) continue;   // same for the whole warp
                Cf *row = a + (size_t)i * ld;
                Cf l[B];
#pragma unroll
                for (uint32_t p = 0; p < B; ++p) {
                    l[p] = (Cf)0.0;
                    if ((bm >> p) & 1u) {
                        Cf x = row[k + p];
#pragma unroll
                        for (uint32_t q = 0; q < p; ++q)
                            if (((bm >> q) & 1u) && ((inner >> (p * B + q)) & 1u)) x = sgb_fma(-l[q], u[(size_t)q * n + k + p], x);
                        l[p] = x * inv_s[p];
                    }
                }
                Cf v[kCoopMaxCols];
#pragma unroll
                for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                    const uint32_t j = j0 + lane + 32u * c;
                    v[c] = (Cf)0.0;
                    if ((live >> (c * B)) & bm) v[c] = row[j];
                }
#pragma unroll
                for (uint32_t c = 0; c < kCoopMaxCols; ++c) {
                    const uint32_t j = j0 + lane + 32u * c;
                    const uint32_t m = (live >> (c * B)) & bm;
                    if (!m) continue;
                    Cf x = v[c];
#pragma unroll
                    for (uint32_t p = 0; p < B; ++p)
                        if ((m >> p) & 1u) x = sgb_fma(-l[p], u[(size_t)p * n + j], x);
                    row[j] = x;
                }
                __syncwarp();   // every lane has read the block entries
#pragma unroll
                for (uint32_t p = 0; p < B; ++p)
                    if (lane == p && ((bm >> p) & 1u)) row[k + p] = l[p];
            }
            sync();
        }
        sync();
    }

    // Row elements [k0, min(k0 + kSolveBatch, end)) of a block's pattern columns, loaded together
    // ahead of the FMA chain that uses them (the LU of a large mechanism lives in L2).
    static constexpr uint32_t kSolveBatch = 8;
    __device__ __forceinline__ static void load_batch(Cf (&r)[kSolveBatch], const Cf *row, uint32_t k0, uint32_t end,
                                                      uint32_t w) {
#pragma unroll
        for (uint32_t q = 0; q < kSolveBatch; ++q) {
            r[q] = (Cf)0.0;
            if (k0 + q < end && ((w >> (k0 + q)) & 1u)) r[q] = row[k0 + q];
        }
    }

    // x = (LU)^-1 x in place, in 32-column blocks. Forward (unit L): a warp
    // solves the diagonal block with shuffles, then every row below takes the
    // block's updates in ascending column order. Backward (U, diagonal holding
    // 1/U(k,k)): blocks from the last; rows above take the block's updates in
    // descending column order; a row's diagonal scaling follows its last update.
    template <class V>
    __device__ void solve(V *x) {
        if constexpr (kMixed) solve_plain(x);   // FP32 LU in shared memory: element by element
        else solve_batched(x);                  // FP64 LU, in L2 for large mechanisms: batched loads
    }

    template <class V>
    __device__ void solve_plain(V *x) {
        const uint32_t nb = (n + 31) / 32;
        for (uint32_t b = 0; b < nb; ++b) {
            const uint32_t kb = b * 32;
            const uint32_t kend = kb + 32 < n ? kb + 32 : n;
            if (warp == 0) {
                const uint32_t i = kb + lane;
                V xi = i < n ? x[i] : (V)0.0;
                const Cf *row = a + (size_t)(i < n ? i : 0) * ld;
                // this row's pattern bits for the block's columns, below the diagonal only
                const uint32_t w = i < n ? pat[i * 8u + b] & ((1u << lane) - 1u) : 0u;
                const uint32_t kn = kend - kb;   // columns in this block (32, or fewer in the last)
#pragma unroll 8
                for (uint32_t kk = 0; kk < kn; ++kk) {
                    const V xk = __shfl_sync(0xffffffffu, xi, kk);
                    if ((w >> kk) & 1u) xi = sgb_fma(-(V)row[kb + kk], xk, xi);
                }
                if (i < n) x[i] = xi;
            }
            sync();
            for (uint32_t i = kend + tid; i < n; i += NT) {
                const Cf *row = a + (size_t)i * ld;
                const uint32_t w = pat[i * 8u + b];
                V xi = x[i];
                for (uint32_t k = kb; k < kend; ++k)
                    if ((w >> (k - kb)) & 1u) xi = sgb_fma(-(V)row[k], x[k], xi);
                x[i] = xi;
            }
            sync();
        }
        for (uint32_t b = nb; b-- > 0;) {
            const uint32_t kb = b * 32;
            const uint32_t kend = kb + 32 < n ? kb + 32 : n;
            if (warp == 0) {
                const uint32_t i = kb + lane;
                V xi = i < n ? x[i] : (V)0.0;
                const Cf *row = a + (size_t)(i < n ? i : 0) * ld;
                // this row's pattern bits for the block's columns, above the diagonal only (columns < n)
                const uint32_t w = i < n ? pat[i * 8u + b] & ~((2u << lane) - 1u) : 0u;
                const V d = i < n ? (V)row[i] : (V)0.0;   // 1/U(i,i)
#pragma unroll 8
                for (uint32_t kk = kend - kb; kk-- > 0;) {
                    if (lane == kk) xi = xi * d;   // row kb+kk: all its updates are in
                    const V xk = __shfl_sync(0xffffffffu, xi, kk);
                    if ((w >> kk) & 1u) xi = sgb_fma(-(V)row[kb + kk], xk, xi);
                }
                if (i < n) x[i] = xi;
            }
            sync();
            for (uint32_t i = tid; i < kb; i += NT) {
                const Cf *row = a + (size_t)i * ld;
                const uint32_t w = pat[i * 8u + b];
                V xi = x[i];
                for (uint32_t k = kend; k-- > kb;)
                    if ((w >> (k - kb)) & 1u) xi = sgb_fma(-(V)row[k], x[k], xi);
                x[i] = xi;
            }
            sync();
        }
    }

    // solve_plain's operations in its order, each row's pattern elements of a block loaded
    // kSolveBatch at a time ahead of the FMAs that use them (measured on the 200-species FP64
    // case: 1.05x the whole step; the mixed path's shared-memory LU measured 1.03x slower).
    template <class V>
    __device__ void solve_batched(V *x) {
        const uint32_t nb = (n + 31) / 32;
        for (uint32_t b = 0; b < nb; ++b) {
            const uint32_t kb = b * 32;
            const uint32_t kend = kb + 32 < n ? kb + 32 : n;
            const uint32_t kn = kend - kb;   // columns in this block (32, or fewer in the last)
            if (warp == 0) {
                const uint32_t i = kb + lane;
                V xi = i < n ? x[i] : (V)0.0;
                const Cf *row = a + (size_t)(i < n ? i : 0) * ld + kb;
                // this row's pattern bits for the block's columns, below the diagonal only
                const uint32_t w = i < n ? pat[i * 8u + b] & ((1u << lane) - 1u) : 0u;
                for (uint32_t k0 = 0; k0 < kn; k0 += kSolveBatch) {
                    Cf r[kSolveBatch];
                    load_batch(r, row, k0, kn, w);
#pragma unroll
                    for (uint32_t q = 0; q < kSolveBatch; ++q) {
                        if (k0 + q >= kn) break;
                        const V xk = __shfl_sync(0xffffffffu, xi, k0 + q);
                        if ((w >> (k0 + q)) & 1u) xi = sgb_fma(-(V)r[q], xk, xi);
                    }
                }
                if (i < n) x[i] = xi;
            }
            sync();
            for (uint32_t i = kend + tid; i < n; i += NT) {
                const Cf *row = a + (size_t)i * ld + kb;
                const uint32_t w = pat[i * 8u + b];
                if (!w) continue;
                V xi = x[i];
                for (uint32_t k0 = 0; k0 < kn; k0 += kSolveBatch) {
                    Cf r[kSolveBatch];
                    load_batch(r, row, k0, kn, w);
#pragma unroll
                    for (uint32_t q = 0; q < kSolveBatch; ++q)
                        if (k0 + q < kn && ((w >> (k0 + q)) & 1u)) xi = sgb_fma(-(V)r[q], x[kb + k0 + q], xi);
                }
                x[i] = xi;
            }
            sync();
        }
        for (uint32_t b = nb; b-- > 0;) {
            const uint32_t kb = b * 32;
            const uint32_t kend = kb + 32 < n ? kb + 32 : n;
            const uint32_t kn = kend - kb;
            if (warp == 0) {
                const uint32_t i = kb + lane;
                V xi = i < n ? x[i] : (V)0.0;
                const Cf *row = a + (size_t)(i < n ? i : 0) * ld + kb;
                // this row's pattern bits for the block's columns, above the diagonal only (columns < n)
                const uint32_t w = i < n ? pat[i * 8u + b] & ~((2u << lane) - 1u) : 0u;
                const V d = i < n ? (V)row[lane] : (V)0.0;   // 1/U(i,i)
                // batches from the block's last column down, each in descending order
                for (uint32_t top = kn; top > 0;) {
                    const uint32_t k0 = top > kSolveBatch ? top - kSolveBatch : 0;
                    Cf r[kSolveBatch];
                    load_batch(r, row, k0, top, w);
#pragma unroll
                    for (uint32_t q = kSolveBatch; q-- > 0;) {
                        if (k0 + q >= top) continue;
                        const uint32_t kk = k0 + q;
                        if (lane == kk) xi = xi * d;   // row kb+kk: all its updates are in
                        const V xk = __shfl_sync(0xffffffffu, xi, kk);
                        if ((w >> kk) & 1u) xi = sgb_fma(-(V)r[q], xk, xi);
                    }
                    top = k0;
                }
                if (i < n) x[i] = xi;
            }
            sync();
            for (uint32_t i = tid; i < kb; i += NT) {
                const Cf *row = a + (size_t)i * ld + kb;
                const uint32_t w = pat[i * 8u + b];
                if (!w) continue;
                V xi = x[i];
                for (uint32_t top = kn; top > 0;) {
                    const uint32_t k0 = top > kSolveBatch ? top - kSolveBatch : 0;
                    Cf r[kSolveBatch];
                    load_batch(r, row, k0, top, w);
#pragma unroll
                    for (uint32_t q = kSolveBatch; q-- > 0;)
                        if (k0 + q < top && ((w >> (k0 + q)) & 1u)) xi = sgb_fma(-(V)r[q], x[kb + k0 + q], xi);
                    top = k0;
                }
                x[i] = xi;
            }
            sync();
        }
    }

    // Mixed: out = W^-1 rb by the FP32 LU, then `sweeps` FP64-residual refinement sweeps.
    __device__ void solve_refined(const DevArgs &A, double ghinv, double *out) {
        float *xs = x32;
        for (uint32_t s = tid; s < n; s += NT) xs[s] = (float)rb[s];
        sync();
        SGB_PHASE(3, solve(xs));
        for (uint32_t s = tid; s < n; s += NT) out[s] = (double)xs[s];
        sync();
        for (uint32_t sw = 0; sw < A.ir_sweeps; ++sw) {
            for (uint32_t i = tid; i < n; i += NT) {
                double w = ghinv * out[i];
                for (uint32_t e = tb.jrow[i]; e < tb.jrow[i + 1]; ++e) w = sgb_fma(js[e], out[tb.jcol[e]], w);
                xs[i] = (float)(rb[i] - w);
            }
            sync();
            SGB_PHASE(3, solve(xs));
            for (uint32_t s = tid; s < n; s += NT) out[s] = out[s] + (double)xs[s];
            sync();
        }
    }

    // One pass of kin_integrate's step loop (kin_solver.h:216-311).
    __device__ void attempt(const DevArgs &A) {
        const double h_min = A.ctl.h_min, rtol = A.ctl.rtol, atol = A.ctl.atol;
        const double inv_n = 1.0 / (double)n;
        double remaining = seg_end - t;
        double h_cap = remaining;
        if (A.ctl.h_max > 0.0) h_cap = vmin(h_cap, A.ctl.h_max);
        double h_wanted = vmax(h, h_min);
        bool last = h_wanted >= remaining;
        double hs = last ? remaining : vmin(h_wanted, h_cap);

        if (tid == 0) {   // the step's two divisions once, shared through red[2..3] (rhs synchronises)
            red[2] = 1.0 / (hs * M::gamma0(A));
            red[3] = 1.0 / hs;
        }
        SGB_PHASE(0, rhs(y));
        SGB_PHASE(1, neg_jac(y));
        const double ghinv = red[2];
        SGB_PHASE(2, factor((Cf)ghinv));
        const double hinv = red[3];

        bool fcn_at_y = true;
        const int S = M::stages(A);
        for (int st = 0; st < S; ++st) {
            const int packed = st * (st - 1) / 2;
            double *Ks = K + (size_t)st * n;
            if (st > 0 && M::new_f(A, st)) {
                bool moved = false;
                for (int j = 0; j < st; ++j)
                    if (M::a(A, packed + j) != 0.0) moved = true;
                if (moved || !fcn_at_y) {
                    for (uint32_t s = tid; s < n; s += NT) {
                        double v = y[s];
                        for (int j = 0; j < st; ++j) {
                            const double av = M::a(A, packed + j);
                            if (av == 0.0) continue;
                            v = sgb_fma(av, K[(size_t)j * n + s], v);
                        }
                        ytmp[s] = v;
                    }
                    sync();
                    SGB_PHASE(0, rhs(ytmp));
                    fcn_at_y = !moved;
                }
            }
            for (uint32_t s = tid; s < n; s += NT) {
                double v = fcn[s];
                for (int j = 0; j < st; ++j) {
                    const double c = M::c(A, packed + j);
                    if (c == 0.0) continue;
                    v = sgb_fma(c * hinv, K[(size_t)j * n + s], v);
                }
                if constexpr (kMixed) rb[s] = v;
                else Ks[s] = v;
            }
            sync();
            if constexpr (kMixed) {
                solve_refined(A, ghinv, Ks);
            } else {
                SGB_PHASE(3, solve(Ks));
            }
        }

        // y_new into ytmp and the weighted RMS error (kin_solver.h:263-280)
        for (uint32_t s = tid; s < n; s += NT) {
            double ynew = y[s], yerr = 0.0;
            for (int st = 0; st < S; ++st) {
                const double mc = M::m(A, st), ec = M::e(A, st);
                if (mc != 0.0) ynew = sgb_fma(mc, K[(size_t)st * n + s], ynew);
                if (ec != 0.0) yerr = sgb_fma(ec, K[(size_t)st * n + s], yerr);
            }
            const double scale = sgb_fma(rtol, vmax(vabs(y[s]), vabs(ynew)), atol);
            qv[s] = yerr / scale;
            ytmp[s] = ynew;
        }
        sync();
        if (tid == 0) {   // error norm and step factor once, shared through red[0..1]
            double e = 0.0;
            for (uint32_t s = 0; s < n; ++s) e = sgb_fma(qv[s], qv[s], e);
            e = vsqrt(e * inv_n);
            if (!is_finite_lane(e)) e = 1e10;
            red[0] = e;
            red[1] = step_factor(e, M::order(A));
        }
        sync();
        const double err = red[0];
        double fac = red[1];
        bool ok = err <= 1.0 || hs <= h_min;
        if (A.ctl.fixed_step) {
            ok = true;
            fac = 1.0;
        }
        if (ok) {
            for (uint32_t s = tid; s < n; s += NT) {
                double ynew = ytmp[s];
                if (A.ctl.clamp_negative) ynew = vmax(ynew, 0.0);
                y[s] = ynew;
            }
            t = last ? seg_end : t + hs;
        }
        double h_acc = hs * fac;
        h_acc = reject_last ? vmin(h_acc, hs) : h_acc;
        h_acc = (last && fac >= 1.0) ? vmax(h_acc, h_wanted) : h_acc;
        double h_rej = reject_more ? hs * 0.1 : vmin(hs * fac, hs);
        if (A.ctl.fixed_step) {
            h_acc = h_wanted;
            h_rej = h_wanted;
        }
        h = ok ? h_acc : h_rej;
        reject_more = !ok && reject_last;
        reject_last = !ok;
        steps = steps + (ok ? 1.0 : 0.0);
        rejects = rejects + (ok ? 0.0 : 1.0);
        if (!(t < seg_end && !(failed > 0.0))) phase = kPhaseSegFinish;
        sync();
    }
};

template <int PREC>
__global__ void __launch_bounds__(512, 1) kin_coop_kernel(const __grid_constant__ DevArgs A, double *scratch, uint64_t stride) {
    extern __shared__ __align__(16) double sm[];
    __shared__ uint32_t cell_s;
    CoopCell<PREC> C;
    C.tb.init(A.tables);
    C.n = C.tb.h->n;
    C.R = C.tb.h->R;
    C.ld = C.tb.h->ld;
    C.nj = C.tb.h->nj;
    C.tid = threadIdx.x;
    C.NT = blockDim.x;
    C.lane = threadIdx.x & 31u;
    C.warp = threadIdx.x >> 5;
    C.W = blockDim.x >> 5;
    const uint32_t n = C.n;
    C.y = sm;
    C.ytmp = C.y + n;
    C.fcn = C.ytmp + n;
    C.src = C.fcn + n;
    C.qv = C.src + n;
    C.rb = C.qv + n;
    C.xv = C.rb + n;
    C.K = C.xv + n;   // 4 stage vectors
    C.kr = C.K + 4 * n;
    C.rate = C.kr + C.R;
    C.red = C.rate + C.R;
    C.x32 = (float *)(sm + coop_smem_doubles(n, C.R));
    uint32_t *pat_s = (uint32_t *)(C.x32 + kCoopMaxSpecies);
    uint16_t *lcnt_s = (uint16_t *)(pat_s + (size_t)n * 8);
    {   // stage the pattern once per CTA
        const uint32_t *pg = (const uint32_t *)((const unsigned char *)A.tables + C.tb.h->off_pat);
        const uint16_t *lg = (const uint16_t *)((const unsigned char *)A.tables + C.tb.h->off_lcnt);
        for (uint32_t q = threadIdx.x; q < n * 8; q += blockDim.x) pat_s[q] = pg[q];
        for (uint32_t q = threadIdx.x; q < n; q += blockDim.x) lcnt_s[q] = lg[q];
    }
    C.pat = pat_s;
    C.lcnt = lcnt_s;
    const CoopSmemLayout lay = coop_layout(PREC, *C.tb.h, A.coop_smem_budget);
    unsigned char *smb = (unsigned char *)sm;
    double *g = scratch + (size_t)blockIdx.x * stride;
    if constexpr (PREC == 2) {
        C.a = (typename CoopCell<PREC>::Cf *)(smb + lay.lu);
        C.js = g;
    } else {   // FP64: small LUs in shared memory, large ones in per-CTA global scratch (L2)
        C.a = lay.lu_bytes ? (typename CoopCell<PREC>::Cf *)(smb + lay.lu) : (typename CoopCell<PREC>::Cf *)g;
        C.js = nullptr;
    }
#ifndef SGB_COOP_LOADS_FIRST_SMEM
#define SGB_COOP_LOADS_FIRST_SMEM 0
#endif
    C.lu_global = (PREC == 0 && lay.lu_bytes == 0) || (SGB_COOP_LOADS_FIRST_SMEM && n >= 64);
    if (lay.terms_bytes) {   // the RHS / Jacobian term lists, once per CTA
        const CoopMech *h = C.tb.h;
        const uint4 *src = (const uint4 *)((const unsigned char *)A.tables + h->off_reac);
        uint4 *dst = (uint4 *)(smb + lay.terms);
        for (uint32_t q = threadIdx.x; q < lay.terms_bytes / 16; q += blockDim.x) dst[q] = src[q];
        unsigned char *t = smb + lay.terms - h->off_reac;   // image offset o lives at t + o
        C.tb.reac = (const uint16_t *)(t + h->off_reac);
        C.tb.fbeg = (const uint32_t *)(t + h->off_fbeg);
        C.tb.fent = (const CoopTerm *)(t + h->off_fent);
        C.tb.jbeg = (const uint32_t *)(t + h->off_jbeg);
        C.tb.jent = (const CoopTerm *)(t + h->off_jent);
        C.tb.jpos = (const uint32_t *)(t + h->off_jpos);
        C.tb.jrow = (const uint32_t *)(t + h->off_jrow);
        C.tb.jcol = (const uint16_t *)(t + h->off_jcol);
    }
    __syncthreads();
    const uint32_t parked = A.resume ? min(*(volatile uint32_t *)A.suspend_count, A.suspend_cap) : 0u;
    for (;;) {
        if (threadIdx.x == 0) cell_s = atomicAdd(A.cursor, 1u);
        __syncthreads();
        const uint32_t idx = cell_s;
        __syncthreads();
        uint32_t cell = idx;
        if (A.resume) {   // cells parked by a lane kernel of this launch
            if (idx >= parked) break;
            const SuspendRec r = A.suspend[idx];
            cell = r.cell;
            C.load(A, cell);
            C.restore(r);
        } else {
            if (idx >= A.lanes) break;
            C.load(A, cell);
        }
        while (C.settle(A, cell)) {
            const long long t_attempt = clock64();
            C.attempt(A);
#ifdef SGB_COOP_PROFILE
            if (threadIdx.x == 0) atomicAdd(&g_coop_phase_cycles[5], (unsigned long long)(clock64() - t_attempt));
#else
            (void)t_attempt;
#endif
        }
        C.store(A, cell);
    }
}

// Module state of the cooperative path.
struct CoopModule {
    bool ready = false;
    std::vector<uint8_t> image;
    CoopMech head;
    void *d_image = nullptr;
    uint32_t *d_header = nullptr;   // cursor (+0), error flag (+32 words)
    double *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    KinMethod method;
    KinControl control;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t ir_sweeps = 1;
    float last_ms = 0.0f;
    uint32_t block[3] = {256, 0, 512};    // threads per CTA by precision (0 FP64, 2 mixed)
    uint32_t ctas[3] = {2, 0, 1};         // resident CTAs per SM by precision
    uint32_t smem_budget[3] = {kCoopSmemBudget, 0, kCoopSmemBudget};
    int sms = 0;
};
CoopModule cm;
constexpr uint32_t kCoopMaxCtasPerSm = 2;   // scratch slots per SM

// Dynamic shared memory of a launch (the L1 / shared split is left to the driver: preferring L1
// measured no faster for the global-memory FP64 LU at one CTA per SM, and cost occupancy at two).
cudaError_t set_coop_attributes(void (*fn)(DevArgs, double *, uint64_t), int prec, const CoopMech &h, uint32_t budget) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)coop_layout(prec, h, budget).total);
}

size_t coop_smem_bytes(int prec, const CoopMech &h, uint32_t budget = kCoopSmemBudget) {
    return coop_layout(prec, h, budget).total;
}

size_t coop_scratch_doubles(int prec, const CoopMech &h) {
    size_t d = prec == 2 ? (size_t)h.nj : (size_t)h.n * h.ld;
    return (d + 31) / 32 * 32;   // 256-byte aligned per CTA
}

}   // namespace

size_t coop_smem_bytes_for(int prec, const CoopMech &h) { return coop_smem_bytes(prec, h); }
size_t coop_scratch_doubles_for(int prec, const CoopMech &h) { return coop_scratch_doubles(prec, h); }

// The cooperative kernel on `A` (A.tables the coop image, A.cursor zeroed):
// lanes [0, A.lanes), or with A.resume the cells a lane kernel parked;
// `scratch` holds grid slots of coop_scratch_doubles_for(prec) doubles.
cudaError_t coop_launch(int prec, const DevArgs &A0, const CoopMech &head, double *scratch, uint32_t grid,
                               uint32_t block, cudaStream_t s) {
    void (*fn)(DevArgs, double *, uint64_t) = prec == 0 ? kin_coop_kernel<0> : kin_coop_kernel<2>;
    DevArgs A = A0;
    if (!A.coop_smem_budget) A.coop_smem_budget = kCoopSmemBudget;
    const size_t smem = coop_smem_bytes(prec, head, A.coop_smem_budget);
    cudaError_t ce = set_coop_attributes(fn, prec, head, A.coop_smem_budget);
    if (ce != cudaSuccess) return ce;
    fn<<<grid, block, smem, s>>>(A, scratch, coop_scratch_doubles(prec, head));
    return cudaGetLastError();
}

}   // namespace sgb

using namespace sgb;

namespace sgb {
const Model *model_of(const KinModelHandle *h);
}

SGB_API int32_t gpu_kin_coop_set_mech(const KinModelHandle *model, const KinMethod *method, const KinControl *control) {
    if (!model || !method || !control || method->stages < 2 || method->stages > 4) return (int32_t)cudaErrorInvalidValue;
    const Model *m = model_of(model);
    if (!m || !m->finalized || m->n() > kCoopMaxSpecies) return (int32_t)cudaErrorInvalidValue;
    std::vector<uint8_t> img;
    if (!coop_image(*m, &img)) return (int32_t)cudaErrorInvalidValue;
    CoopMech h;
    memcpy(&h, img.data(), sizeof(h));
    int dev = 0, sms = 0, max_smem = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return (int32_t)e;
    if (coop_smem_bytes(0, h) > (size_t)max_smem) return (int32_t)cudaErrorInvalidValue;
    if (cm.d_image) cudaFree(cm.d_image);
    cm.d_image = nullptr;
    if (!cm.d_header) {
        e = cudaMalloc((void **)&cm.d_header, 256);
        if (e != cudaSuccess) return (int32_t)e;
    }
    e = cudaMalloc(&cm.d_image, img.size());
    if (e == cudaSuccess) e = cudaMemcpy(cm.d_image, img.data(), img.size(), cudaMemcpyHostToDevice);
    // scratch for the larger of the two precisions' needs, one slot per resident CTA (one CTA per SM)
    const size_t per = coop_scratch_doubles(0, h) > coop_scratch_doubles(2, h) ? coop_scratch_doubles(0, h)
                                                                              : coop_scratch_doubles(2, h);
    const size_t need = per * 8 * (size_t)sms * kCoopMaxCtasPerSm;
    if (e == cudaSuccess && need > cm.scratch_bytes) {
        if (cm.d_scratch) cudaFree(cm.d_scratch);
        cm.d_scratch = nullptr;
        cm.scratch_bytes = 0;
        e = cudaMalloc((void **)&cm.d_scratch, need);
        if (e == cudaSuccess) cm.scratch_bytes = need;
    }
    if (e == cudaSuccess && !cm.ev0) e = cudaEventCreate(&cm.ev0);
    if (e == cudaSuccess && !cm.ev1) e = cudaEventCreate(&cm.ev1);
    if (e != cudaSuccess) return (int32_t)e;
    cm.image.swap(img);
    cm.head = h;
    cm.sms = sms;
    cm.method = *method;
    cm.control = *control;
    cm.ready = true;
    return 0;
}

SGB_API int32_t gpu_kin_coop_advance(const GpuKinLaunch *L, float *kernel_ms) {
    if (!cm.ready || !L) return (int32_t)cudaErrorInvalidValue;
    if ((L->precision != 0 && L->precision != 2) || L->padded == 0 || L->lane_count > L->padded)
        return (int32_t)cudaErrorInvalidValue;
    if (!(L->duration >= 0.0) || L->duration > 1.0e300) return (int32_t)cudaErrorInvalidValue;
    if (!L->y || !L->h || !L->steps || !L->rejects || !L->pulses || !L->failed || !L->k || !L->src || !L->pulse ||
        !L->period || !L->pulse_first || !L->pulse_count)
        return (int32_t)cudaErrorInvalidValue;
    const int prec = (int)L->precision;
    int max_smem = 0;
    if (cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0) != cudaSuccess ||
        coop_smem_bytes(prec, cm.head, cm.smem_budget[prec]) > (size_t)max_smem)
        return (int32_t)cudaErrorInvalidValue;   // the mixed path's FP32 LU must fit one CTA's shared memory
    DevArgs A;
    memset(&A, 0, sizeof(A));
    A.y = L->y; A.h = L->h; A.steps = L->steps; A.rejects = L->rejects; A.pulses = L->pulses; A.failed = L->failed;
    A.k = L->k; A.src = L->src; A.pulse = L->pulse; A.period = L->period;
    A.pulse_first = L->pulse_first; A.pulse_count = L->pulse_count;
    A.padded = L->padded;
    A.lanes = L->lane_count ? L->lane_count : L->padded;
    A.duration = L->duration;
    A.ctl = cm.control;
    memcpy(A.ma, cm.method.a, sizeof(A.ma));
    memcpy(A.mc, cm.method.c, sizeof(A.mc));
    memcpy(A.mm, cm.method.m, sizeof(A.mm));
    memcpy(A.me, cm.method.e, sizeof(A.me));
    A.gamma0 = cm.method.gamma0;
    memcpy(A.new_f, cm.method.new_f, sizeof(A.new_f));
    A.stages = cm.method.stages;
    A.order = cm.method.order;
    A.ir_sweeps = cm.ir_sweeps;
    A.cursor = cm.d_header;
    A.error_flag = cm.d_header + 32;
    A.wait_polls = kSpinLimit;
    A.tables = cm.d_image;
    A.table_bytes = cm.head.bytes;
    if (A.lanes == 0 || A.duration == 0.0) {
        if (kernel_ms) *kernel_ms = 0.0f;
        return 0;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int32_t)e;
    void (*fn)(DevArgs, double *, uint64_t) = prec == 0 ? kin_coop_kernel<0> : kin_coop_kernel<2>;
    A.coop_smem_budget = cm.smem_budget[prec];
    const size_t smem = coop_smem_bytes(prec, cm.head, A.coop_smem_budget);
    e = set_coop_attributes(fn, prec, cm.head, A.coop_smem_budget);
    if (e != cudaSuccess) return (int32_t)e;
    int fit = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, (int)cm.block[prec], smem);
    if (e != cudaSuccess) return (int32_t)e;
    const uint32_t per_sm = (uint32_t)(fit < 1 ? 1 : fit) < cm.ctas[prec] ? (uint32_t)(fit < 1 ? 1 : fit) : cm.ctas[prec];
    const uint32_t resident = per_sm * (uint32_t)sms;
    const uint32_t grid = resident < A.lanes ? resident : A.lanes;
    const uint64_t stride = coop_scratch_doubles(prec, cm.head);
    cudaStream_t s = (cudaStream_t)gpu_stream();
    e = cudaMemsetAsync(cm.d_header, 0, 256, s);
    if (e == cudaSuccess) e = cudaEventRecord(cm.ev0, s);
    if (e != cudaSuccess) return (int32_t)e;
    fn<<<grid, cm.block[prec], smem, s>>>(A, cm.d_scratch, stride);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(cm.ev1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(cm.ev1);
    if (e != cudaSuccess) return (int32_t)e;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, cm.ev0, cm.ev1);
    cm.last_ms = ms;
    if (kernel_ms) *kernel_ms = ms;
    return 0;
}

// Counts of the cooperative path's mechanism image: n, R, nnz, Jacobian
// entries, L entries, U entries, LU updates, image bytes.
SGB_API int32_t gpu_kin_coop_info(uint64_t *out8) {
    if (!cm.ready || !out8) return (int32_t)cudaErrorInvalidValue;
    const CoopMech &h = cm.head;
    out8[0] = h.n; out8[1] = h.R; out8[2] = h.nnz; out8[3] = h.nj;
    out8[4] = h.l_entries; out8[5] = h.u_entries; out8[6] = h.lu_updates; out8[7] = h.bytes;
    return 0;
}

// Phase cycle counters of a -DSGB_COOP_PROFILE build (zeros otherwise); reading resets them.
SGB_API int32_t gpu_kin_coop_phase_cycles(uint64_t *out6) {
    if (!out6) return (int32_t)cudaErrorInvalidValue;
    memset(out6, 0, 6 * sizeof(uint64_t));
#ifdef SGB_COOP_PROFILE
    unsigned long long v[8];
    cudaError_t e = cudaMemcpyFromSymbol(v, g_coop_phase_cycles, sizeof(v));
    if (e != cudaSuccess) return (int32_t)e;
    for (int i = 0; i < 6; ++i) out6[i] = v[i];
    memset(v, 0, sizeof(v));
    e = cudaMemcpyToSymbol(g_coop_phase_cycles, v, sizeof(v));
    if (e != cudaSuccess) return (int32_t)e;
#endif
    return 0;
}

SGB_API int32_t gpu_kin_coop_set_smem_budget(uint32_t precision, uint32_t bytes) {
    if ((precision != 0 && precision != 2) || bytes > 227 * 1024) return (int32_t)cudaErrorInvalidValue;
    cm.smem_budget[precision] = bytes;
    return 0;
}

SGB_API int32_t gpu_kin_coop_set_shape(uint32_t precision, uint32_t block, uint32_t ctas_per_sm) {
    if ((precision != 0 && precision != 2) || block < 64 || block > 512 || (block & 31) || ctas_per_sm < 1 ||
        ctas_per_sm > kCoopMaxCtasPerSm)
        return (int32_t)cudaErrorInvalidValue;
    cm.block[precision] = block;
    cm.ctas[precision] = ctas_per_sm;
    return 0;
}

SGB_API int32_t gpu_kin_coop_set_refinement(uint32_t sweeps) {
    if (sweeps > 4) return (int32_t)cudaErrorInvalidValue;
    cm.ir_sweeps = sweeps;
    return 0;
}
