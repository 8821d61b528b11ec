// Device side of the batched Rosenbrock integrator.
//
// One lane = one cell (an independent reactor). A lane's integration over
// [0, duration] is written as a small state machine -- segment start, one
// step attempt, segment end (discharge pulse), done -- so that a kernel can
// run each lane's attempts back to back and refill a lane with a new cell the
// moment its cell finishes (the persistent work-queue kernel), while every
// lane still performs exactly the operation sequence of the reference's
// scalar lane:
//   kin_integrate  src/sim/kinetics/kin_solver.h:189-313 (one attempt = one
//                  pass of its while loop, lines 211-312)
//   kin_advance    kin_solver.h:322-347 (segments between pulses)
//   dbd_advance_group  src/sim/dbd_lanes.h:28-78 (load / store, counters
//                  accumulate, f32 lanes store base + increment)
// Precisions (GpuKinLaunch.precision):
//   0  f64 lanes: every operation the reference's f64 lane performs, built with
//      -fmad=false so FMAs appear only where the reference has lane_fmadd; the
//      result is bit-identical to the reference's CPU path
//   1  f32 lanes, Delta formulation (the reference's f32 / f32x8 lanes)
//   2  mixed: RHS, -J and the LU of W in FP32; each stage solve refined with
//      FP64-residual iterative refinement; state, stage combination, error
//      estimate and step-size control in FP64 (the same controller code as 0)

#pragma once
#include <stdint.h>

#include "../../include/simstack_gpu.h"
#include "ptx.cuh"
#include "tmem.cuh"

namespace sgb {

// ---------------------------------------------------------------------------
// Lane arithmetic with the reference's semantics (src/base/base_lane.h:47-117).

__device__ __forceinline__ double sgb_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float sgb_fma(float a, float b, float c) { return fmaf(a, b, c); }
template <class T> __device__ __forceinline__ T vmin(T a, T b) { return a < b ? a : b; }
template <class T> __device__ __forceinline__ T vmax(T a, T b) { return a > b ? a : b; }
template <class T> __device__ __forceinline__ T vabs(T a) { return a < (T)0 ? -a : a; }
__device__ __forceinline__ double vsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float vsqrt(float a) { return sqrtf(a); }
template <class T> __device__ __forceinline__ bool is_finite_lane(T a) {
    T d = a - a;
    return d == d;
}

// fma(+1, d, +0) and fma(-1, d, +0), exactly, with integer operations: the
// product is exact, and the only case the +0 addend changes is a zero product,
// which becomes +0. (Used for the first term of each Jacobian slot.)
__device__ __forceinline__ double sgb_first_pos(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return __longlong_as_double((long long)((b << 1) == 0 ? 0ull : b));
}
__device__ __forceinline__ double sgb_first_neg(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return __longlong_as_double((long long)((b << 1) == 0 ? 0ull : (b ^ 0x8000000000000000ull)));
}
__device__ __forceinline__ float sgb_first_pos(float d) {
    unsigned b = __float_as_uint(d);
    return __uint_as_float((b << 1) == 0 ? 0u : b);
}
__device__ __forceinline__ float sgb_first_neg(float d) {
    unsigned b = __float_as_uint(d);
    return __uint_as_float((b << 1) == 0 ? 0u : (b ^ 0x80000000u));
}

// Double-float arithmetic: a value is hi + lo, two FP32 numbers (~48-bit
// significand). The mixed path evaluates the RHS this way on the FP32 pipe.
struct Df {
    float hi, lo;
};
__device__ __forceinline__ Df df_from(double d) {
    const float h = (float)d;
    return Df{h, (float)(d - (double)h)};   // d - h is exact in FP64
}
__device__ __forceinline__ double df_to(Df a) { return (double)a.hi + (double)a.lo; }
// df_from of a compile-time constant
__host__ __device__ constexpr Df df_const(double d) { return Df{(float)d, (float)(d - (double)(float)d)}; }
__device__ __forceinline__ Df df_mul(Df a, Df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const float s = p + e;
    return Df{s, e - (s - p)};
}
__device__ __forceinline__ Df df_add(Df a, Df b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e = e + a.lo;
    e = e + b.lo;
    const float t = s + e;
    return Df{t, e - (t - s)};
}
__device__ __forceinline__ Df df_scale(Df a, float c) { return Df{a.hi * c, a.lo * c}; }   // exact for c = +-1, +-2, +-4

// x^(1/3) on [1e-4, 1e4]: x^(1/4) x^(1/16) x^(1/64) from six square roots,
// then two Newton steps; no libm (base_lane.h:123-135).
template <class T> __device__ __forceinline__ T cbrt_clamped(T x) {
    x = vmin(vmax(x, (T)1e-4), (T)1e4);
    T r4 = vsqrt(vsqrt(x));
    T r16 = vsqrt(vsqrt(r4));
    T r64 = vsqrt(vsqrt(r16));
    T g = r4 * r16 * r64;
    const T two = (T)2.0, third = (T)(1.0 / 3.0);
    g = (two * g + x / (g * g)) * third;
    g = (two * g + x / (g * g)) * third;
    return g;
}

// (1/err)^(1/order) * 0.9 clamped to [0.2, 6] (kin_solver.h:169-180).
template <class T> __device__ __forceinline__ T step_factor(T err, uint32_t order) {
    T e = vmin(vmax(err, (T)1e-4), (T)1e4);
    T root;
    if (order == 2) root = vsqrt(e);
    else if (order == 4) root = vsqrt(vsqrt(e));
    else root = cbrt_clamped(e);
    T fac = (T)0.9 / root;
    return vmin(vmax(fac, (T)0.2), (T)6.0);
}

// ---------------------------------------------------------------------------
// Launch arguments (kernel parameter space: uniform, constant-bank reads).

struct DevArgs {
    double *y, *h, *steps, *rejects, *pulses, *failed;
    const double *k, *src, *pulse, *period, *pulse_first, *pulse_count;
    uint32_t padded, lanes;
    double duration;
    KinControl ctl;
    double ma[6], mc[6], mm[4], me[4], gamma0;
    int32_t new_f[4];
    uint32_t stages, order;
    uint32_t ir_sweeps;        // mixed path: refinement sweeps per stage solve (>= 1)
    uint32_t *cursor;          // queue kernel: next unclaimed lane
    uint32_t *error_flag;      // nonzero: a bounded wait ran out (tables not staged)
    uint32_t wait_polls;       // poll limit of the table-staging wait (kSpinLimit unless a caller lowers it)
    const void *tables;        // table-driven ops: KinMech image in global memory
    uint32_t table_bytes;      // bytes to stage (multiple of 16)
    // straggler hand-off (queue and static kernels, precisions 0 and 3): a cell that has
    // taken `budget` step attempts in this launch parks its scalar state in `suspend` and
    // leaves; a cooperative kernel finishes it (0 = never)
    uint32_t budget;
    uint32_t suspend_cap;
    uint32_t *suspend_count;
    struct SuspendRec *suspend;
    uint32_t resume;           // cooperative kernel: take cells from the suspension list
    uint32_t coop_smem_budget; // cooperative kernel: shared-memory bytes the term lists may fill up to
};

// The scalar state of a parked cell (its y, h and counters are in the zone block).
struct SuspendRec {
    double t, h, seg_end, applied;
    uint32_t cell, iterations, transitions, flags;   // flags: pending | reject_last << 1 | reject_more << 2
};

// Method coefficients known at compile time (Rodas3: kin_solver.h:382-391) or
// read from the launch arguments (any method).
struct Rodas3Coef {
    static constexpr int kStages = 4;
    __device__ static constexpr int stages(const DevArgs &) { return 4; }
    __device__ static constexpr uint32_t order(const DevArgs &) { return 3; }
    __device__ static constexpr double a(const DevArgs &, int i) { return i == 1 ? 2.0 : i == 3 ? 2.0 : i == 5 ? 1.0 : 0.0; }
    __device__ static constexpr double c(const DevArgs &, int i) {
        return i == 0 ? 4.0 : i == 1 ? 1.0 : i == 2 ? -1.0 : i == 3 ? 1.0 : i == 4 ? -1.0 : -8.0 / 3.0;
    }
    __device__ static constexpr double m(const DevArgs &, int i) { return i == 0 ? 2.0 : i == 1 ? 0.0 : 1.0; }
    __device__ static constexpr double e(const DevArgs &, int i) { return i == 3 ? 1.0 : 0.0; }
    __device__ static constexpr double gamma0(const DevArgs &) { return 0.5; }
    __device__ static constexpr bool new_f(const DevArgs &, int) { return true; }
    // a and c as double-float constants (the mixed lanes' stage loop indexes them at run time;
    // selecting among constants keeps the FP64 pipe out of it)
    __device__ static Df a_df(const DevArgs &, int i) {
        constexpr Df two = df_const(2.0), one = df_const(1.0), zero = df_const(0.0);
        return i == 1 || i == 3 ? two : i == 5 ? one : zero;
    }
    __device__ static Df c_df(const DevArgs &, int i) {
        constexpr Df c0 = df_const(4.0), c1 = df_const(1.0), c2 = df_const(-1.0), c5 = df_const(-8.0 / 3.0);
        return i == 0 ? c0 : i == 1 || i == 3 ? c1 : i == 2 || i == 4 ? c2 : c5;
    }
};

// Any method of up to KIN_MAX_STAGES stages; the stage count is a runtime bound.
struct RuntimeCoef {
    static constexpr int kStages = KIN_MAX_STAGES;
    __device__ static int stages(const DevArgs &A) { return (int)A.stages; }
    __device__ static uint32_t order(const DevArgs &A) { return A.order; }
    __device__ static double a(const DevArgs &A, int i) { return A.ma[i]; }
    __device__ static double c(const DevArgs &A, int i) { return A.mc[i]; }
    __device__ static double m(const DevArgs &A, int i) { return A.mm[i]; }
    __device__ static double e(const DevArgs &A, int i) { return A.me[i]; }
    __device__ static double gamma0(const DevArgs &A) { return A.gamma0; }
    __device__ static bool new_f(const DevArgs &A, int i) { return A.new_f[i] != 0; }
    __device__ static Df a_df(const DevArgs &A, int i) { return df_from(A.ma[i]); }
    __device__ static Df c_df(const DevArgs &A, int i) { return df_from(A.mc[i]); }
};

template <bool B, class X, class Y> struct Pick { typedef X type; };
template <class X, class Y> struct Pick<false, X, Y> { typedef Y type; };

enum : int { kPhaseSegStart = 0, kPhaseStepping = 1, kPhaseSegFinish = 2, kPhaseDone = 3 };

// ---------------------------------------------------------------------------
// One lane. Ops provides the mechanism kernels (generated straight-line code
// or the table walk); M the method coefficients; PREC the precision.

template <class Ops, class M, int PREC>
struct Lane {
    typedef typename Pick<PREC == 1, float, double>::type T;    // time, step size, state, stage vectors
    typedef typename Pick<PREC == 0, double, float>::type Cf;   // RHS / Jacobian / LU arithmetic
    static constexpr bool kDelta = PREC == 1;
    static constexpr bool kMixed = PREC == 2;
    static constexpr int N = Ops::N, R = Ops::R, NNZ = Ops::NNZ, S = M::kStages;

    Ops ops;
    // cell data
    T y[N];
    T base[kDelta ? N : 1];
    Cf k[kMixed ? 1 : R], src[kMixed ? 1 : N];
    float khi[kMixed ? R : 1], klo[kMixed ? R : 1], shi[kMixed ? N : 1], slo[kMixed ? N : 1];   // mixed: double-float k, src
    T t, h, seg_end, applied, duration, period, first, count;
    T steps, rejects, pulses, failed;
    uint32_t iterations, transitions, attempts;
    int phase;
    bool pending, reject_last, reject_more;
    // per-attempt scratch
    Cf lu[NNZ];
    Cf fcn[kMixed ? 1 : N];
    Cf ceval[kDelta ? N : 1];                  // delta: base + increment
    float yhi[kMixed ? N : 1], ylo[kMixed ? N : 1], fhi[kMixed ? N : 1], flo[kMixed ? N : 1];   // mixed: double-float point, RHS
    T ytmp[N];
    T K[S][N];
    double js[kMixed ? Ops::NJ : 1];           // mixed: -J pattern entries (FP64) before the factorisation
    double f0[kMixed ? N : 1];                 // mixed: f(y) at the step start
    float d32[kMixed ? N : 1], df32[kMixed ? N : 1];   // mixed: stage increment and its RHS increment
    double rb[kMixed ? N : 1];                 // mixed: stage right-hand side b
    double rr[kMixed ? N : 1];                 // mixed: residual
    float x32[kMixed ? N : 1];

    static constexpr size_t kSmemBytes = 0;
    __device__ __forceinline__ void bind(unsigned char *) {}
    __device__ __forceinline__ uint32_t n() const { return ops.n(); }

    // dbd_lanes.h:28-58: storage is f64; f32 lanes round on load.
    __device__ __forceinline__ void load(const DevArgs &A, uint32_t i) {
        const uint32_t p = A.padded, nn = n(), rr_ = ops.r();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            double v = A.y[(size_t)s * p + i];
            if (kDelta) {
                base[s] = (T)v;
                y[s] = (T)0.0;
            } else {
                y[s] = (T)v;
            }
            if constexpr (kMixed) {
                const Df v = df_from(A.src[(size_t)s * p + i]);
                shi[s] = v.hi;
                slo[s] = v.lo;
            } else {
                src[s] = (Cf)A.src[(size_t)s * p + i];
            }
        }
        for (int r = 0; r < R; ++r) {
            if (r >= (int)rr_) break;
            if constexpr (kMixed) {
                const Df v = df_from(A.k[(size_t)r * p + i]);
                khi[r] = v.hi;
                klo[r] = v.lo;
            } else {
                k[r] = (Cf)A.k[(size_t)r * p + i];
            }
        }
        h = (T)A.h[i];
        period = (T)A.period[i];
        first = (T)A.pulse_first[i];
        count = (T)A.pulse_count[i];
        duration = (T)A.duration;
        steps = rejects = pulses = (T)0.0;
        failed = (T)A.failed[i];
        t = (T)0.0;
        applied = (T)0.0;
        transitions = 0;
        attempts = 0;
        phase = kPhaseSegStart;
    }

    // Straggler hand-off: park the scalar state; false if the list is full (the lane keeps the cell).
    __device__ __forceinline__ bool park(const DevArgs &A, uint32_t cell) {
        const uint32_t slot = atomicAdd(A.suspend_count, 1u);
        if (slot >= A.suspend_cap) return false;
        SuspendRec r;
        r.t = (double)t;
        r.h = (double)h;
        r.seg_end = (double)seg_end;
        r.applied = (double)applied;
        r.cell = cell;
        r.iterations = iterations;
        r.transitions = transitions;
        r.flags = (pending ? 1u : 0u) | (reject_last ? 2u : 0u) | (reject_more ? 4u : 0u);
        A.suspend[slot] = r;
        phase = kPhaseDone;
        return true;
    }

    // dbd_lanes.h:60-77: f32 lanes add their increment to the f64 storage.
    __device__ __forceinline__ void store(const DevArgs &A, uint32_t i) {
        const uint32_t p = A.padded, nn = n();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            double *dst = A.y + (size_t)s * p + i;
            if (kDelta) {
                double v = *dst + (double)y[s];
                if (A.ctl.clamp_negative) v = v > 0.0 ? v : 0.0;
                *dst = v;
            } else {
                *dst = (double)y[s];
            }
        }
        A.h[i] = (double)h;
        A.failed[i] = (double)failed;
        A.steps[i] += (double)steps;
        A.rejects[i] += (double)rejects;
        A.pulses[i] += (double)pulses;
    }

    // kin_advance segment start + kin_integrate prologue (kin_solver.h:204-208, 330-334).
    __device__ __forceinline__ void seg_start(const DevArgs &A) {
        const T zero = (T)0.0;
        pending = applied < count;
        T next_pulse = sgb_fma(applied, period, first);
        seg_end = pending ? vmin(next_pulse, duration) : duration;
        bool active = t < seg_end && !(failed > zero);
        reject_last = false;
        reject_more = false;
        h = h > zero ? h : (T)A.ctl.h_start;
        iterations = 0;
        phase = active ? kPhaseStepping : kPhaseSegFinish;
    }

    // kin_advance after one segment (kin_solver.h:336-345).
    __device__ __forceinline__ void seg_finish(const DevArgs &A, uint32_t cell) {
        const T zero = (T)0.0, one = (T)1.0;
        bool alive = !(failed > zero);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            const uint32_t p = A.padded, nn = n();
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                y[s] = y[s] + (T)A.pulse[(size_t)s * p + cell];
            }
            applied = applied + one;
            pulses = pulses + one;
            h = (T)A.ctl.h_start;
        }
        bool done = (t >= duration && applied >= count) || !alive;
        phase = done ? kPhaseDone : kPhaseSegStart;
    }

    // Runs the cheap transitions until the lane needs a step attempt (true)
    // or has finished its cell (false). The transition guard (2^24 segment
    // transitions per cell, far above any real pulse schedule) ends cells whose
    // schedule cannot terminate (a non-finite pulse count), marking them failed.
    __device__ __forceinline__ bool settle(const DevArgs &A, uint32_t cell) {
        for (;;) {
            if (++transitions > (1u << 24)) {
                failed = (T)1.0;
                phase = kPhaseDone;
            }
            switch (phase) {
                case kPhaseSegStart: seg_start(A); break;
                case kPhaseSegFinish: seg_finish(A, cell); break;
                case kPhaseStepping:
                    if constexpr (PREC == 0) {
                        if (A.budget && attempts >= A.budget && park(A, cell)) return false;
                        ++attempts;
                    }
                    if (++iterations > A.ctl.max_steps) {   // kin_solver.h:212-215
                        failed = (T)1.0;
                        phase = kPhaseSegFinish;
                        break;
                    }
                    return true;
                default: return false;
            }
        }
    }

    __device__ __forceinline__ void eval_point(const T *yy, const Cf *&at) {
        const uint32_t nn = n();
        if constexpr (kDelta) {
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                ceval[s] = base[s] + yy[s];
            }
            at = ceval;
        } else {
            at = (const Cf *)yy;
        }
    }

    // Mixed path: the RHS at yy (FP64) in double-float on the FP32 pipe.
    __device__ __forceinline__ void rhs_df(const double *yy) {
        const uint32_t nn = n();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            const Df v = df_from(yy[s]);
            yhi[s] = v.hi;
            ylo[s] = v.lo;
        }
        ops.fun_df(khi, klo, shi, slo, yhi, ylo, fhi, flo);
    }

    // Mixed path: x = W^-1 b with the FP32 LU, then `sweeps` refinement
    // sweeps x += W^-1 (b - W x), residual in FP64. b in rb, result in x.
    __device__ __forceinline__ void solve_refined(const DevArgs &A, double ghinv, double *x) {
        const uint32_t nn = n();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            x32[s] = (float)rb[s];
        }
        ops.solve(lu, x32);
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            x[s] = (double)x32[s];
        }
        for (uint32_t sw = 0; sw < A.ir_sweeps; ++sw) {
            ops.residual(js, ghinv, rb, x, rr);
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                x32[s] = (float)rr[s];
            }
            ops.solve(lu, x32);
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                x[s] = x[s] + (double)x32[s];
            }
        }
    }

    // One pass of kin_integrate's step loop (kin_solver.h:216-311) for an active lane.
    // kSync: called by every thread of the CTA together (the CTA-synchronous
    // kernel); barriers between the phases keep the CTA's warps on the same
    // stretch of straight-line code. commit = false: the lane has no cell this
    // round; it computes on its last state and keeps none of the results.
    template <bool kSync = false>
    __device__ __forceinline__ void attempt(const DevArgs &A, bool commit = true) {
        const T zero = (T)0.0, one = (T)1.0;
        const uint32_t nn = n();
        const T h_min = (T)A.ctl.h_min, rtol = (T)A.ctl.rtol, atol = (T)A.ctl.atol;
        const T inv_n = (T)(1.0 / (double)nn);

        T remaining = seg_end - t;
        T h_cap = remaining;
        if (A.ctl.h_max > 0.0) h_cap = vmin(h_cap, (T)A.ctl.h_max);
        T h_wanted = vmax(h, h_min);
        bool last = h_wanted >= remaining;
        T hs = last ? remaining : vmin(h_wanted, h_cap);

        const Cf *at = nullptr;
        if constexpr (kMixed) {
            rhs_df(y);
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                f0[s] = df_to(Df{fhi[s], flo[s]});
            }
            ops.neg_jac(khi, yhi, lu);   // FP32 Jacobian at the FP32 rounding of y
            ops.save_jac(lu, js);
        } else {
            eval_point(y, at);
            ops.fun(k, src, at, fcn);
            ops.neg_jac(k, at, lu);
        }
        if constexpr (kSync) __syncthreads();
        T ghinv = one / (hs * (T)M::gamma0(A));
        if constexpr (kMixed) ops.factor((float)ghinv, lu);
        else ops.factor((Cf)ghinv, lu);
        if constexpr (kSync) __syncthreads();
        T hinv = one / hs;

        bool fcn_at_y = true;   // fcn (plain paths) holds f at the step-start point
        bool last_moved = false;   // mixed: the last stage RHS was f(y) + df32 (else f(y))
#pragma unroll(kMixed ? 1 : S)
        for (int st = 0; st < S; ++st) {
            if (st >= M::stages(A)) break;
            const int packed = st * (st - 1) / 2;
            if (st > 0 && M::new_f(A, st)) {
                // stage point Y = y + sum_j a_j K_j; when no a_j is nonzero Y is y
                // itself (Rodas3 stage 2) and f(Y) = f(y) is reused, bit for bit
                bool moved = false;
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    ytmp[s] = y[s];
                }
#pragma unroll
                for (int j = 0; j < st; ++j) {
                    double a = M::a(A, packed + j);
                    if (a == 0.0) continue;
                    moved = true;
                    T av = (T)a;
                    for (int s = 0; s < N; ++s) {
                        if (s >= (int)nn) break;
                        ytmp[s] = sgb_fma(av, K[j][s], ytmp[s]);
                    }
                }
                if constexpr (kMixed) {
                    if (moved) {
                        for (int s = 0; s < N; ++s) {
                            if (s >= (int)nn) break;
                            d32[s] = (float)(ytmp[s] - y[s]);
                        }
                        ops.fun_delta(khi, yhi, d32, df32);
                    }
                    last_moved = moved;
                } else if (moved || !fcn_at_y) {
                    eval_point(ytmp, at);
                    ops.fun(k, src, at, fcn);
                    fcn_at_y = !moved;
                }
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    if constexpr (kMixed) K[st][s] = moved ? f0[s] + (double)df32[s] : f0[s];
                    else K[st][s] = (T)fcn[s];
                }
            } else {   // no new evaluation: the last stage RHS again
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    if constexpr (kMixed) K[st][s] = last_moved ? f0[s] + (double)df32[s] : f0[s];
                    else K[st][s] = (T)fcn[s];
                }
            }
#pragma unroll
            for (int j = 0; j < st; ++j) {
                double c = M::c(A, packed + j);
                if (c == 0.0) continue;
                T hc = (T)c * hinv;
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    K[st][s] = sgb_fma(hc, K[j][s], K[st][s]);
                }
            }
            if constexpr (kMixed) {
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    rb[s] = K[st][s];
                }
                solve_refined(A, ghinv, K[st]);
            } else {
                ops.solve(lu, K[st]);
            }
            if constexpr (kSync) __syncthreads();
        }

        // y_new into ytmp and the weighted RMS error (kin_solver.h:263-280)
        T err = zero;
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            T ynew = y[s], yerr = zero;
            bool first_e = true;
#pragma unroll
            for (int st = 0; st < S; ++st) {
                if (st >= M::stages(A)) break;
                const double mc = M::m(A, st), ec = M::e(A, st);
                if (mc != 0.0) ynew = sgb_fma((T)mc, K[st][s], ynew);
                if (ec != 0.0) {
                    yerr = (first_e && ec == 1.0) ? sgb_first_pos(K[st][s]) : sgb_fma((T)ec, K[st][s], yerr);
                    first_e = false;
                }
            }
            T scale;
            if (kDelta) scale = sgb_fma(rtol, vmax(vabs(base[s] + y[s]), vabs(base[s] + ynew)), atol);
            else scale = sgb_fma(rtol, vmax(vabs(y[s]), vabs(ynew)), atol);
            T q = yerr / scale;
            err = sgb_fma(q, q, err);
            ytmp[s] = ynew;
        }
        err = vsqrt(err * inv_n);
        if (!is_finite_lane(err)) err = (T)1e10;

        T fac = step_factor(err, M::order(A));
        bool ok = err <= one || hs <= h_min;
        if (A.ctl.fixed_step) {
            ok = true;
            fac = one;
        }
        if (!commit) return;
        if (ok) {
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                T ynew = ytmp[s];
                if (A.ctl.clamp_negative) ynew = kDelta ? vmax(ynew, -base[s]) : vmax(ynew, zero);
                y[s] = ynew;
            }
            t = last ? seg_end : t + hs;
        }
        T h_acc = hs * fac;
        h_acc = reject_last ? vmin(h_acc, hs) : h_acc;
        h_acc = (last && fac >= one) ? vmax(h_acc, h_wanted) : h_acc;
        T h_rej = reject_more ? hs * (T)0.1 : vmin(hs * fac, hs);
        if (A.ctl.fixed_step) {
            h_acc = h_wanted;
            h_rej = h_wanted;
        }
        h = ok ? h_acc : h_rej;
        reject_more = !ok && reject_last;
        reject_last = !ok;
        steps = steps + (ok ? one : zero);
        rejects = rejects + (ok ? zero : one);
        if (!(t < seg_end && !(failed > zero))) phase = kPhaseSegFinish;
    }
};

// ---------------------------------------------------------------------------
// Mixed path, double-float state: the whole step on the FP32 pipe. The state
// y and the RHS at the step start are double-float (hi + lo, ~48-bit
// significand); the Jacobian, LU, stage vectors K and solves are FP32; the
// stage right-hand sides f(y) + [f(Y) - f(y)] + sum c/h K_j are accumulated in
// double-float before rounding to FP32, so the cancellation between f(y) and
// the stage terms costs no FP32 accuracy; y_new = y + sum m K in
// double-float. Only the scalar controller (t, h) stays FP64. FP64 arithmetic
// is 1/74 of FP32 on this GPU and conversions between the two run at the FP64
// rate, so this path issues almost no FP64 work per species.

__device__ __forceinline__ Df df_add_f(Df a, float b) {   // a + b, b a float (two-sum of the high parts)
    const float s = a.hi + b;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b - bb);
    e = e + a.lo;
    const float t = s + e;
    return Df{t, e - (t - s)};
}
__device__ __forceinline__ Df df_prod_f(float a, float b) {   // exact product of two floats
    const float p = a * b;
    return Df{p, fmaf(a, b, -p)};
}

// kLuStride > 0: the LU lives in shared memory, interleaved across the CTA's
// lanes (element e of lane t at [e * kLuStride + t]: consecutive lanes hit
// consecutive banks), instead of in the lane's registers / local memory.
template <class Ops, class M, int kLuStride = 0>
struct LaneDf {
    static constexpr int N = Ops::N, R = Ops::R, NNZ = Ops::NNZ, S = M::kStages;
    static constexpr size_t kSmemBytes = kLuStride ? (size_t)NNZ * kLuStride * sizeof(float) : 0;

    Ops ops;
    float yhi[N], ylo[N];
    float khi[R], klo[R], shi[N], slo[N];
    double t, h, seg_end, applied, duration, period, first, count;
    double steps, rejects, pulses, failed;
    uint32_t iterations, transitions, attempts;
    int phase;
    bool pending, reject_last, reject_more;
    float lu_r[kLuStride ? 1 : NNZ];
    float *lu_s;
    float fhi[N], flo[N];
    float K[S][N];
    float d32[N], df32[N];
    float nhi[N], nlo[N];

    __device__ __forceinline__ void bind(unsigned char *smem) {
        if constexpr (kLuStride > 0) lu_s = (float *)smem + threadIdx.x;
    }
    __device__ __forceinline__ uint32_t n() const { return ops.n(); }

    __device__ __forceinline__ void load(const DevArgs &A, uint32_t i) {
        const uint32_t p = A.padded, nn = n(), rr_ = ops.r();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            Df v = df_from(A.y[(size_t)s * p + i]);
            yhi[s] = v.hi;
            ylo[s] = v.lo;
            v = df_from(A.src[(size_t)s * p + i]);
            shi[s] = v.hi;
            slo[s] = v.lo;
        }
        for (int r = 0; r < R; ++r) {
            if (r >= (int)rr_) break;
            const Df v = df_from(A.k[(size_t)r * p + i]);
            khi[r] = v.hi;
            klo[r] = v.lo;
        }
        h = A.h[i];
        period = A.period[i];
        first = A.pulse_first[i];
        count = A.pulse_count[i];
        duration = A.duration;
        steps = rejects = pulses = 0.0;
        failed = A.failed[i];
        t = 0.0;
        applied = 0.0;
        transitions = 0;
        attempts = 0;
        phase = kPhaseSegStart;
    }

    // Straggler hand-off (see Lane::park); y goes to the zone block as hi + lo, exact in FP64.
    __device__ __forceinline__ bool park(const DevArgs &A, uint32_t cell) {
        const uint32_t slot = atomicAdd(A.suspend_count, 1u);
        if (slot >= A.suspend_cap) return false;
        SuspendRec r;
        r.t = t;
        r.h = h;
        r.seg_end = seg_end;
        r.applied = applied;
        r.cell = cell;
        r.iterations = iterations;
        r.transitions = transitions;
        r.flags = (pending ? 1u : 0u) | (reject_last ? 2u : 0u) | (reject_more ? 4u : 0u);
        A.suspend[slot] = r;
        phase = kPhaseDone;
        return true;
    }

    __device__ __forceinline__ void store(const DevArgs &A, uint32_t i) {
        const uint32_t p = A.padded, nn = n();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            A.y[(size_t)s * p + i] = df_to(Df{yhi[s], ylo[s]});
        }
        A.h[i] = h;
        A.failed[i] = failed;
        A.steps[i] += steps;
        A.rejects[i] += rejects;
        A.pulses[i] += pulses;
    }

    __device__ __forceinline__ void seg_start(const DevArgs &A) {
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

    __device__ __forceinline__ void seg_finish(const DevArgs &A, uint32_t cell) {
        bool alive = !(failed > 0.0);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            const uint32_t p = A.padded, nn = n();
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                const Df v = df_add(Df{yhi[s], ylo[s]}, df_from(A.pulse[(size_t)s * p + cell]));
                yhi[s] = v.hi;
                ylo[s] = v.lo;
            }
            applied = applied + 1.0;
            pulses = pulses + 1.0;
            h = A.ctl.h_start;
        }
        bool done = (t >= duration && applied >= count) || !alive;
        phase = done ? kPhaseDone : kPhaseSegStart;
    }

    __device__ __forceinline__ bool settle(const DevArgs &A, uint32_t cell) {
        for (;;) {
            if (++transitions > (1u << 24)) {
                failed = 1.0;
                phase = kPhaseDone;
            }
            switch (phase) {
                case kPhaseSegStart: seg_start(A); break;
                case kPhaseSegFinish: seg_finish(A, cell); break;
                case kPhaseStepping:
                    if (A.budget && attempts >= A.budget && park(A, cell)) return false;
                    ++attempts;
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

    template <bool kSync = false>
    __device__ __forceinline__ void attempt(const DevArgs &A, bool commit = true) {
        const uint32_t nn = n();
        const float rtol = (float)A.ctl.rtol, atol = (float)A.ctl.atol;
        const float inv_n = 1.0f / (float)nn;

        const double remaining = seg_end - t;
        double h_cap = remaining;
        if (A.ctl.h_max > 0.0) h_cap = vmin(h_cap, A.ctl.h_max);
        const double h_wanted = vmax(h, A.ctl.h_min);
        const bool last = h_wanted >= remaining;
        const double hs = last ? remaining : vmin(h_wanted, h_cap);
        const float hs32 = (float)hs;

        ops.fun_df(khi, klo, shi, slo, yhi, ylo, fhi, flo);
        const float g32 = 1.0f / (hs32 * (float)M::gamma0(A));
        if constexpr (kLuStride > 0) {
            ops.template neg_jac<kLuStride>(khi, yhi, lu_s);
            if constexpr (kSync) __syncthreads();
            ops.template factor<kLuStride>(g32, lu_s);
        } else {
            ops.neg_jac(khi, yhi, lu_r);
            if constexpr (kSync) __syncthreads();
            ops.factor(g32, lu_r);
        }
        if constexpr (kSync) __syncthreads();
        const float hinv = 1.0f / hs32;

        bool last_moved = false;
#pragma unroll 1
        for (int st = 0; st < S; ++st) {
            if (st >= M::stages(A)) break;
            const int packed = st * (st - 1) / 2;
            if (st > 0 && M::new_f(A, st)) {
                bool moved = false;
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    d32[s] = 0.0f;
                }
#pragma unroll
                for (int j = 0; j < st; ++j) {
                    const float av = (float)M::a(A, packed + j);
                    if (av == 0.0f) continue;
                    moved = true;
                    for (int s = 0; s < N; ++s) {
                        if (s >= (int)nn) break;
                        d32[s] = fmaf(av, K[j][s], d32[s]);
                    }
                }
                if (moved) ops.fun_delta(khi, yhi, d32, df32);
                last_moved = moved;
            }
            // b = f(y) [+ f(Y) - f(y)] + sum_j c_j / h K_j in double-float, rounded once
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                Df b{fhi[s], flo[s]};
                if (last_moved) b = df_add_f(b, df32[s]);
#pragma unroll
                for (int j = 0; j < st; ++j) {
                    const float c = (float)M::c(A, packed + j);
                    if (c == 0.0f) continue;
                    b = df_add(b, df_prod_f(c * hinv, K[j][s]));
                }
                K[st][s] = b.hi + b.lo;
            }
            if constexpr (kLuStride > 0) ops.template solve<kLuStride>(lu_s, K[st]);
            else ops.solve(lu_r, K[st]);
            if constexpr (kSync) __syncthreads();
        }

        // y_new (double-float) and the weighted RMS error (FP32)
        float err32 = 0.0f;
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            Df yn{yhi[s], ylo[s]};
            float yerr = 0.0f;
#pragma unroll
            for (int st = 0; st < S; ++st) {
                if (st >= M::stages(A)) break;
                const float mc = (float)M::m(A, st), ec = (float)M::e(A, st);
                if (mc != 0.0f) yn = df_add(yn, df_prod_f(mc, K[st][s]));
                if (ec != 0.0f) yerr = fmaf(ec, K[st][s], yerr);
            }
            const float scale = fmaf(rtol, fmaxf(fabsf(yhi[s]), fabsf(yn.hi)), atol);
            const float q = yerr / scale;
            err32 = fmaf(q, q, err32);
            nhi[s] = yn.hi;
            nlo[s] = yn.lo;
        }
        err32 = sqrtf(err32 * inv_n);
        if (!is_finite_lane(err32)) err32 = 1e10f;
        float fac32 = step_factor(err32, M::order(A));
        bool ok = err32 <= 1.0f || hs <= A.ctl.h_min;
        if (A.ctl.fixed_step) {
            ok = true;
            fac32 = 1.0f;
        }
        if (!commit) return;
        if (ok) {
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                float hi = nhi[s], lo = nlo[s];
                if (A.ctl.clamp_negative && (hi < 0.0f || (hi == 0.0f && lo < 0.0f))) {
                    hi = 0.0f;
                    lo = 0.0f;
                }
                yhi[s] = hi;
                ylo[s] = lo;
            }
            t = last ? seg_end : t + hs;
        }
        const double fac = (double)fac32;
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
    }
};



// ---------------------------------------------------------------------------
// Mixed path, double-float state with refined stages (mixed variant 2): every
// per-species quantity -- y, f at each stage point, the stage right-hand sides
// b, the stage vectors K, y_new and the error norm -- is a double-float on the
// FP32 pipe; -J, the LU of W and the triangular solves are FP32 and precondition
// one refinement sweep per stage, whose residual r = b - ghinv x + J x is formed
// in double-float with J x evaluated reaction by reaction at y (no stored
// Jacobian). Only t, h and a few scalars per step are FP64. Its results track
// the FP64 path to ~1e-8 (4,096 cells of the shipped mechanism, 1 s) where an FP32 solve alone
// leaves ~1e-3 on species near atol.

__device__ __forceinline__ Df df_mul_f(Df a, float b) {   // double-float times float
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    const float s = p + e;
    return Df{s, e - (s - p)};
}
__device__ __forceinline__ Df df_neg(Df a) { return Df{-a.hi, -a.lo}; }
__device__ __forceinline__ Df df_abs(Df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? df_neg(a) : a; }
__device__ __forceinline__ bool df_less(Df a, Df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ Df df_two_sum(float a, float b) {   // exact a + b, normalised
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return Df{s, e};
}
// Lazily normalised double-float arithmetic for the long sums: df_acc adds a pair to an
// accumulator whose hi holds the rounded running sum and whose lo collects the low parts and
// every two-sum rounding error (8 FP32 operations instead of df_add's 11); the products skip
// their final renormalisation (|lo| stays within a few ulp of hi); a sum is normalised once,
// with a two-sum, when it is complete.
__device__ __forceinline__ Df df_acc(Df a, Df t) {
    const float s = a.hi + t.hi;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (t.hi - bb);
    return Df{s, a.lo + (t.lo + e)};
}
__device__ __forceinline__ Df df_mul_u(Df a, Df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return Df{p, e};
}
__device__ __forceinline__ Df df_mul_fu(Df a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return Df{p, e};
}
__device__ __forceinline__ Df df_norm(Df a) { return df_two_sum(a.hi, a.lo); }

// times a method coefficient: exact for +-1, +-2, +-4, +-1/2, else a double-float product
__device__ __forceinline__ Df df_times_coef(Df a, double c) {
    if (c == 1.0) return a;
    if (c == -1.0 || c == 2.0 || c == -2.0 || c == 4.0 || c == -4.0 || c == 0.5 || c == -0.5) return df_scale(a, (float)c);
    return df_mul(a, df_from(c));
}
__device__ __forceinline__ Df df_times_coef_u(Df a, double c) {
    if (c == 1.0) return a;
    if (c == -1.0 || c == 2.0 || c == -2.0 || c == 4.0 || c == -4.0 || c == 0.5 || c == -0.5) return df_scale(a, (float)c);
    return df_mul_u(a, df_from(c));
}
// df_times_coef_u with the coefficient already split (c = df_from of the FP64 value): the same
// branches and results, decided by FP32 compares
__device__ __forceinline__ Df df_times_coef_df_u(Df a, Df c) {
    if (c.lo == 0.0f) {
        if (c.hi == 1.0f) return a;
        if (c.hi == -1.0f || c.hi == 2.0f || c.hi == -2.0f || c.hi == 4.0f || c.hi == -4.0f || c.hi == 0.5f || c.hi == -0.5f)
            return df_scale(a, c.hi);
    }
    return df_mul_u(a, c);
}

// The mixed lanes' step-size factor (kin_solver.h:169-180's formula): for order 3 the cube
// root comes from the FP32 chain of cbrt_clamped, then one division-free Newton step in FP64
// for w = e^(-1/3) (w <- w (4 - e w^3) / 3, relative error ~2e-14 from FP32's ~1e-7), and
// fac = 0.9 w -- a few FP64 operations instead of the six FP64 square roots and three FP64
// divisions of the FP64 lanes. Orders 2 and 4 as step_factor.
__device__ __forceinline__ double step_factor_mixed(double err, uint32_t order) {
    if (order != 3) return step_factor(err, order);
    const double e = vmin(vmax(err, 1e-4), 1e4);
    const float g = cbrt_clamped((float)e);
    double w = (double)(1.0f / g);
    const double w3 = w * w * w;
    w = w * (4.0 - e * w3) * (1.0 / 3.0);
    const double fac = 0.9 * w;
    return vmin(vmax(fac, 0.2), 6.0);
}

// kLuStride > 0: the FP32 LU lives in shared memory, interleaved across the CTA's lanes
// (element e of lane t at [e * kLuStride + t]), which frees registers for the double-float vectors.
// kTmemCols > 0: the stage vectors K live in tensor memory -- the CTA allocates kTmemCols columns,
// warp w uses lane quarter w % 4 and columns 256 (w / 4) + [0, 256), stage st at column 64 st:
// K hi then K lo, 2N <= 64 floats -- instead of local memory (they are indexed by the stage).
// Build-time switches of the CTA-synchronous kernel's barriers inside a refined step: after -J
// and the factorisation (phase), and after every stage (stage). They keep the CTA's warps on the
// same stretch of code; no data is shared between lanes, so results do not depend on them.
// Measured on 1,048,576 cells x 10 s (256 threads, stage vectors in TMEM): stage barriers only
// 558 ms, both 568 ms, none 678 ms (the instruction fetch is shared by fewer warps).
#ifndef SGB_IR_PHASE_BARRIERS
#define SGB_IR_PHASE_BARRIERS 0
#endif
#ifndef SGB_IR_STAGE_BARRIERS
#define SGB_IR_STAGE_BARRIERS 1
#endif

template <class Ops, class M, int kLuStride = 0, int kTmemCols = 0>
struct LaneIr {
    static constexpr bool kPhaseBarriers = SGB_IR_PHASE_BARRIERS != 0, kStageBarriers = SGB_IR_STAGE_BARRIERS != 0;
    static constexpr int N = Ops::N, R = Ops::R, NNZ = Ops::NNZ, S = M::kStages;
    static constexpr size_t kSmemBytes = kLuStride ? (size_t)NNZ * kLuStride * sizeof(float) : 0;
    static constexpr bool kTmemK = kTmemCols > 0;
    static constexpr uint32_t kTmemAlloc = (uint32_t)kTmemCols;
    static_assert(!kTmemK || (2 * N <= 64 && S * 64 <= 256), "stage vectors must fit 64 TMEM columns each, 4 stages");

    Ops ops;
    float yhi[N], ylo[N];
    float khi[R], klo[R], shi[N], slo[N];
    double t, h, seg_end, applied, duration, period, first, count;
    double steps, rejects, pulses, failed;
    uint32_t iterations, transitions, attempts;
    int phase;
    bool pending, reject_last, reject_more;
    float lu_r[kLuStride ? 1 : NNZ];
    float *lu_s;
    float Yhi[N], Ylo[N], fhi[N], flo[N], bhi[N], blo[N];
    float Khi[kTmemK ? 1 : S][N], Klo[kTmemK ? 1 : S][N];
    float x[N], x2[N];
    uint32_t tmem_k;   // this thread's TMEM address of stage slot 0

    __device__ __forceinline__ void bind(unsigned char *smem) {
        if constexpr (kLuStride > 0) lu_s = (float *)smem + threadIdx.x;
    }
    __device__ __forceinline__ void bind_tmem(uint32_t base) { tmem_k = tmem_lane_addr(base, 256u * ((threadIdx.x >> 5) >> 2)); }

    // stage vector st <-> kh, kl (TMEM slot or the local arrays)
    __device__ __forceinline__ void k_store(int st, const float *kh, const float *kl) {
        if constexpr (kTmemK) {
            float v[2 * N];
#pragma unroll
            for (int s = 0; s < N; ++s) {
                v[s] = kh[s];
                v[N + s] = kl[s];
            }
            const uint32_t a = tmem_k + 64u * (uint32_t)st;
            __syncwarp();
#pragma unroll
            for (int c = 0; c + 32 <= 2 * N; c += 32) tmem_st32(a + c, v + c);
#pragma unroll
            for (int c = (2 * N / 32) * 32; c < 2 * N; c += 2) tmem_st2(a + c, v[c], v[c + 1]);
        } else {
#pragma unroll
            for (int s = 0; s < N; ++s) {
                Khi[st][s] = kh[s];
                Klo[st][s] = kl[s];
            }
        }
    }
    __device__ __forceinline__ void k_load(int st, float *kh, float *kl) {
        if constexpr (kTmemK) {
            float v[2 * N];
            const uint32_t a = tmem_k + 64u * (uint32_t)st;
            __syncwarp();
#pragma unroll
            for (int c = 0; c + 32 <= 2 * N; c += 32) tmem_ld32(a + c, v + c);
#pragma unroll
            for (int c = (2 * N / 32) * 32; c < 2 * N; c += 2) tmem_ld2(a + c, v[c], v[c + 1]);
#pragma unroll
            for (int s = 0; s < N; ++s) {
                kh[s] = v[s];
                kl[s] = v[N + s];
            }
        } else {
#pragma unroll
            for (int s = 0; s < N; ++s) {
                kh[s] = Khi[st][s];
                kl[s] = Klo[st][s];
            }
        }
    }
    __device__ __forceinline__ void lu_solve(float *v) {
        if constexpr (kLuStride > 0) ops.template solve<kLuStride>(lu_s, v);
        else ops.solve(lu_r, v);
    }
    __device__ __forceinline__ uint32_t n() const { return ops.n(); }

    __device__ __forceinline__ void load(const DevArgs &A, uint32_t i) {
        const uint32_t p = A.padded, nn = n(), rr_ = ops.r();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            Df v = df_from(A.y[(size_t)s * p + i]);
            yhi[s] = v.hi;
            ylo[s] = v.lo;
            v = df_from(A.src[(size_t)s * p + i]);
            shi[s] = v.hi;
            slo[s] = v.lo;
        }
        for (int r = 0; r < R; ++r) {
            if (r >= (int)rr_) break;
            const Df v = df_from(A.k[(size_t)r * p + i]);
            khi[r] = v.hi;
            klo[r] = v.lo;
        }
        h = A.h[i];
        period = A.period[i];
        first = A.pulse_first[i];
        count = A.pulse_count[i];
        duration = A.duration;
        steps = rejects = pulses = 0.0;
        failed = A.failed[i];
        t = 0.0;
        applied = 0.0;
        transitions = 0;
        attempts = 0;
        phase = kPhaseSegStart;
    }

    __device__ __forceinline__ void store(const DevArgs &A, uint32_t i) {
        const uint32_t p = A.padded, nn = n();
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            A.y[(size_t)s * p + i] = df_to(Df{yhi[s], ylo[s]});
        }
        A.h[i] = h;
        A.failed[i] = failed;
        A.steps[i] += steps;
        A.rejects[i] += rejects;
        A.pulses[i] += pulses;
    }

    __device__ __forceinline__ void seg_start(const DevArgs &A) {
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

    __device__ __forceinline__ void seg_finish(const DevArgs &A, uint32_t cell) {
        bool alive = !(failed > 0.0);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            const uint32_t p = A.padded, nn = n();
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                const Df v = df_add(Df{yhi[s], ylo[s]}, df_from(A.pulse[(size_t)s * p + cell]));
                yhi[s] = v.hi;
                ylo[s] = v.lo;
            }
            applied = applied + 1.0;
            pulses = pulses + 1.0;
            h = A.ctl.h_start;
        }
        bool done = (t >= duration && applied >= count) || !alive;
        phase = done ? kPhaseDone : kPhaseSegStart;
    }

    __device__ __forceinline__ bool settle(const DevArgs &A, uint32_t cell) {
        for (;;) {
            if (++transitions > (1u << 24)) {
                failed = 1.0;
                phase = kPhaseDone;
            }
            switch (phase) {
                case kPhaseSegStart: seg_start(A); break;
                case kPhaseSegFinish: seg_finish(A, cell); break;
                case kPhaseStepping:
                    ++attempts;
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

    template <bool kSync = false>
    __device__ __forceinline__ void attempt(const DevArgs &A, bool commit = true) {
        const uint32_t nn = n();
        const double remaining = seg_end - t;
        double h_cap = remaining;
        if (A.ctl.h_max > 0.0) h_cap = vmin(h_cap, A.ctl.h_max);
        const double h_wanted = vmax(h, A.ctl.h_min);
        const bool last = h_wanted >= remaining;
        const double hs = last ? remaining : vmin(h_wanted, h_cap);
        const double hinv = 1.0 / hs;
        // 1 / (gamma h): for gamma = 1/2 the same bits as 2 (1 / h), one FP64 division saved
        const double ghinv = M::gamma0(A) == 0.5 ? 2.0 * hinv : 1.0 / (hs * M::gamma0(A));
        const Df gd = df_from(ghinv), hd = df_from(hinv);

        // FP32 -J at the FP32 rounding of y, factorised
        if constexpr (kLuStride > 0) {
            ops.template neg_jac<kLuStride>(khi, yhi, lu_s);
            if constexpr (kSync && kPhaseBarriers) __syncthreads();
            ops.template factor<kLuStride>((float)ghinv, lu_s);
        } else {
            ops.neg_jac(khi, yhi, lu_r);
            if constexpr (kSync && kPhaseBarriers) __syncthreads();
            ops.factor((float)ghinv, lu_r);
        }
        if constexpr (kSync && kPhaseBarriers) __syncthreads();

        bool f_at_y = false;   // f (fhi, flo) holds f(y)
#pragma unroll 1
        for (int st = 0; st < S; ++st) {
            if (st >= M::stages(A)) break;
            const int packed = st * (st - 1) / 2;
            if (st == 0 || M::new_f(A, st)) {
                // stage point Y = y + sum_j a_j K_j; f(y) is reused when the point is y
                bool moved = false;
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    Yhi[s] = yhi[s];
                    Ylo[s] = ylo[s];
                }
#pragma unroll 1   // one copy of the body: the smaller step code is faster (1,048,576 cells x 10 s: 509.5 vs 520.7 ms)
                for (int j = 0; j < S - 1; ++j) {
                    if (j >= st) break;
                    const Df a = M::a_df(A, packed + j);
                    if (a.hi == 0.0f) continue;
                    moved = true;
                    float kh[N], kl[N];
                    k_load(j, kh, kl);
                    for (int s = 0; s < N; ++s) {
                        if (s >= (int)nn) break;
                        const Df v = df_acc(Df{Yhi[s], Ylo[s]}, df_times_coef_df_u(Df{kh[s], kl[s]}, a));
                        Yhi[s] = v.hi;
                        Ylo[s] = v.lo;
                    }
                }
                if (moved) {
                    for (int s = 0; s < N; ++s) {
                        if (s >= (int)nn) break;
                        const Df v = df_norm(Df{Yhi[s], Ylo[s]});
                        Yhi[s] = v.hi;
                        Ylo[s] = v.lo;
                    }
                }
                if (moved || !f_at_y) {
                    ops.fun_dfl(khi, klo, shi, slo, Yhi, Ylo, fhi, flo);
                    f_at_y = !moved;
                }
            }
            // b = f + sum_j (c_j / h) K_j in double-float
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                bhi[s] = fhi[s];
                blo[s] = flo[s];
            }
#pragma unroll 1   // as above
            for (int j = 0; j < S - 1; ++j) {
                if (j >= st) break;
                const Df c = M::c_df(A, packed + j);
                if (c.hi == 0.0f) continue;
                const Df ch = df_mul(c, hd);   // c / h in double-float
                float kh[N], kl[N];
                k_load(j, kh, kl);
                for (int s = 0; s < N; ++s) {
                    if (s >= (int)nn) break;
                    const Df v = df_acc(Df{bhi[s], blo[s]}, df_mul_u(ch, Df{kh[s], kl[s]}));
                    bhi[s] = v.hi;
                    blo[s] = v.lo;
                }
            }
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                const Df v = df_norm(Df{bhi[s], blo[s]});
                bhi[s] = v.hi;
                blo[s] = v.lo;
                x[s] = v.hi;
            }
            lu_solve(x);
            // one refinement sweep: r = b - ghinv x + J x (double-float), x2 = W32^-1 r
            ops.residual_df(khi, klo, yhi, ylo, x, bhi, blo, gd, x2);
            lu_solve(x2);
            {
                float kh[N], kl[N];
                for (int s = 0; s < N; ++s) {
                    const Df v = df_two_sum(x[s], x2[s]);
                    kh[s] = v.hi;
                    kl[s] = v.lo;
                }
                k_store(st, kh, kl);
            }
            if constexpr (kSync && kStageBarriers) __syncthreads();
        }

        // y_new (accumulated in Y) and the error estimate (in b), stage vector by stage vector:
        // per species the same operations in the same order as a species-by-species loop
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            Yhi[s] = yhi[s];
            Ylo[s] = ylo[s];
        }
        bool first_e = true;
#pragma unroll
        for (int st = 0; st < S; ++st) {
            if (st >= M::stages(A)) break;
            const double mc = M::m(A, st), ec = M::e(A, st);
            if (mc == 0.0 && ec == 0.0) continue;
            float kh[N], kl[N];
            k_load(st, kh, kl);
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                const Df kv{kh[s], kl[s]};
                if (mc != 0.0) {
                    const Df v = df_acc(Df{Yhi[s], Ylo[s]}, df_times_coef_u(kv, mc));
                    Yhi[s] = v.hi;
                    Ylo[s] = v.lo;
                }
                if (ec != 0.0) {
                    const Df v = first_e ? df_times_coef_u(kv, ec) : df_acc(Df{bhi[s], blo[s]}, df_times_coef_u(kv, ec));
                    bhi[s] = v.hi;
                    blo[s] = v.lo;
                }
            }
            if (ec != 0.0) first_e = false;
        }
        const Df rtol = df_from(A.ctl.rtol), atol = df_from(A.ctl.atol);
        Df err2{0.0f, 0.0f};
        for (int s = 0; s < N; ++s) {
            if (s >= (int)nn) break;
            const Df yn = df_norm(Df{Yhi[s], Ylo[s]});
            const Df ye = first_e ? Df{0.0f, 0.0f} : df_norm(Df{bhi[s], blo[s]});
            const Df ay = df_abs(Df{yhi[s], ylo[s]}), an = df_abs(yn);
            const Df scale = df_add(df_mul(rtol, df_less(ay, an) ? an : ay), atol);
            const float inv = 1.0f / scale.hi;
            const float q1 = ye.hi * inv;
            const float q2 = df_add(ye, df_neg(df_mul_f(scale, q1))).hi * inv;
            const Df q = df_two_sum(q1, q2);
            err2 = df_add(err2, df_mul(q, q));
            Yhi[s] = yn.hi;   // y_new, kept in the stage-point buffer
            Ylo[s] = yn.lo;
        }
        double err = sqrt(df_to(err2) * (1.0 / (double)nn));
        if (!is_finite_lane(err)) err = 1e10;
        double fac = step_factor_mixed(err, M::order(A));
        bool ok = err <= 1.0 || hs <= A.ctl.h_min;
        if (A.ctl.fixed_step) {
            ok = true;
            fac = 1.0;
        }
        if (!commit) return;
        if (ok) {
            for (int s = 0; s < N; ++s) {
                if (s >= (int)nn) break;
                float hi = Yhi[s], lo = Ylo[s];
                if (A.ctl.clamp_negative && (hi < 0.0f || (hi == 0.0f && lo < 0.0f))) {
                    hi = 0.0f;
                    lo = 0.0f;
                }
                yhi[s] = hi;
                ylo[s] = lo;
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
    }
};

// ---------------------------------------------------------------------------
// Generated straight-line ops (kin_codegen.cpp) as an Ops object.

// SGB_OPS_QUALIFIER: __forceinline__ (default) inlines every op at every call
// site; building with -DSGB_NOINLINE_OPS keeps one copy of each op's body
// (smaller code, more calls) -- a build-time variant for the instruction-cache
// experiments.
#ifdef SGB_NOINLINE_OPS
#define SGB_OPS_QUALIFIER __noinline__
#else
#define SGB_OPS_QUALIFIER __forceinline__
#endif

template <class G>
struct GenOps {
    static constexpr int N = G::N, R = G::R, NNZ = G::NNZ, NJ = G::NJ;
    static constexpr bool kStridedLu = true;   // the LU ops take a storage stride (shared-memory LU)
    __device__ __forceinline__ uint32_t n() const { return (uint32_t)N; }
    __device__ __forceinline__ uint32_t r() const { return (uint32_t)R; }
    __device__ __forceinline__ bool init(const DevArgs &, unsigned char *) { return true; }
    template <class T> __device__ SGB_OPS_QUALIFIER void fun(const T *k, const T *src, const T *y, T *f) const { G::fun(k, src, y, f); }
    template <int S = 1, class T> __device__ SGB_OPS_QUALIFIER void neg_jac(const T *k, const T *y, T *a) const {
        G::template neg_jac<T, S>(k, y, a);
    }
    template <int S = 1, class T> __device__ SGB_OPS_QUALIFIER void factor(T ghinv, T *a) const { G::template factor<T, S>(ghinv, a); }
    template <int S = 1, class T> __device__ SGB_OPS_QUALIFIER void solve(const T *a, T *x) const { G::template solve<T, S>(a, x); }
    __device__ SGB_OPS_QUALIFIER void fun_df(const float *khi, const float *klo, const float *shi, const float *slo, const float *yhi,
                                             const float *ylo, float *fhi, float *flo) const {
        G::fun_df(khi, klo, shi, slo, yhi, ylo, fhi, flo);
    }
    __device__ SGB_OPS_QUALIFIER void fun_delta(const float *k, const float *y, const float *d, float *df) const { G::fun_delta(k, y, d, df); }
    __device__ SGB_OPS_QUALIFIER void fun_dfl(const float *khi, const float *klo, const float *shi, const float *slo, const float *yhi,
                                              const float *ylo, float *fhi, float *flo) const {
        G::fun_dfl(khi, klo, shi, slo, yhi, ylo, fhi, flo);
    }
    __device__ SGB_OPS_QUALIFIER void residual_df(const float *khi, const float *klo, const float *yhi, const float *ylo, const float *x,
                                                  const float *bhi, const float *blo, Df g, float *r) const {
        G::residual_df(khi, klo, yhi, ylo, x, bhi, blo, g, r);
    }
    __device__ SGB_OPS_QUALIFIER void save_jac(const float *a, double *js) const { G::save_jac(a, js); }
    __device__ SGB_OPS_QUALIFIER void residual(const double *js, double ghinv, const double *b, const double *x, double *r) const {
        G::residual(js, ghinv, b, x, r);
    }
};

}   // namespace sgb
