// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// The reference's builder and table-walk solver compiled with larger
// KIN_MAX_* capacities (oracle/Makefile), for synthetic mechanisms that still
// fit its u16 tables. The tests use it to pin the oracle's wide-index
// restatement beyond the shipped mechanism. Built only where the reference
// sources exist.

#define BASE_DEBUG_H
#define TIMED_BLOCK(name)
#define TIMED_FUNCTION()
struct DebugTable;

#include <stdio.h>
#include <stdlib.h>
#include <math.h>

#include "sim_platform.h"
#include "sim/kinetics/kin_build.cpp"
#include "sim/dbd_lanes.h"

#define REF_API extern "C" __attribute__((visibility("default")))

REF_API void *ref_big_new(void) { return calloc(1, sizeof(KinModel)); }
REF_API void ref_big_free(void *h) { free(h); }
REF_API u32 ref_big_add_species(void *h, const char *name, s32 abstract_species) {
    return kin_add_species((KinModel *)h, name, abstract_species);
}
REF_API u32 ref_big_add_reaction(void *h, const char *equation, s32 kind, const f64 *p, s32 ref) {
    KinRateLaw l;
    if (kind == 0) l = kin_arr(p[0], p[1], p[2]);
    else if (kind == 1) l = kin_m(p[0], p[1], p[2]);
    else if (kind == 2) l = kin_troe(p[0], p[1], p[2], p[3], p[4]);
    else l = kin_eq_reverse((u32)ref, p[0], p[1]);
    return kin_add_reaction((KinModel *)h, equation, l);
}
REF_API void ref_big_finalize(void *h) { kin_mech_finalize((KinModel *)h); }
REF_API const char *ref_big_error(void *h) { return ((KinModel *)h)->error ? ((KinModel *)h)->error_text : ""; }
REF_API void ref_big_counts(void *h, u64 *c) {
    KinMech *m = &((KinModel *)h)->mech;
    c[0] = m->species_count; c[1] = m->reaction_count; c[2] = m->nnz; c[3] = m->lu_div_count; c[4] = m->lu_sub_count;
    c[5] = m->lower_begin[m->species_count]; c[6] = m->upper_begin[m->species_count]; c[7] = ((KinModel *)h)->error;
}
REF_API void ref_big_lu_ops(void *h, u32 *pivots4, u32 *updates2) {
    KinMech *m = &((KinModel *)h)->mech;
    for (u32 d = 0; d < m->lu_div_count; ++d) {
        pivots4[4 * d] = m->lu_div[d].ik; pivots4[4 * d + 1] = m->lu_div[d].kk;
        pivots4[4 * d + 2] = m->lu_div[d].sub_begin; pivots4[4 * d + 3] = m->lu_div[d].sub_end;
    }
    for (u32 s = 0; s < m->lu_sub_count; ++s) { updates2[2 * s] = m->lu_sub[s].ij; updates2[2 * s + 1] = m->lu_sub[s].kj; }
}
REF_API void ref_big_rate_constants(void *h, f64 T, f64 M, f64 *k) { kin_eval_rate_constants((KinModel *)h, T, M, k); }

struct RefControl {
    f64 rtol, atol, h_min, h_max, h_start;
    u32 max_steps;
    s32 fixed_step, clamp_negative;
};
struct RefLaneArrays {
    f64 *y, *h, *steps, *rejects, *pulses, *failed;
    const f64 *k, *src, *pulse, *period, *pulse_first, *pulse_count;
    u32 padded;
};

// Lanes [first, end): variant 0 = f64x4 table walk, 1 = f64 scalar table walk.
REF_API s32 ref_big_advance(void *h, s32 method_id, const RefControl *rc, const RefLaneArrays *a, u32 first, u32 end,
                            f64 duration, s32 variant) {
    KinModel *model = (KinModel *)h;
    KinMethod method = kin_method((KinMethodId)method_id);
    KinControl ctl = {};
    ctl.rtol = rc->rtol; ctl.atol = rc->atol; ctl.h_min = rc->h_min; ctl.h_max = rc->h_max; ctl.h_start = rc->h_start;
    ctl.max_steps = rc->max_steps; ctl.fixed_step = rc->fixed_step; ctl.clamp_negative = rc->clamp_negative;
    DbdLaneArrays la;
    la.y = a->y; la.h = a->h; la.steps = a->steps; la.rejects = a->rejects; la.pulses = a->pulses; la.failed = a->failed;
    la.k = a->k; la.src = a->src; la.pulse = a->pulse; la.period = a->period;
    la.pulse_first = a->pulse_first; la.pulse_count = a->pulse_count; la.padded = a->padded;
    if (variant == 0) {
        if (first % 4 || end % 4) return -1;
        for (u32 i = first; i < end; i += 4) dbd_advance_group<f64x4>(&model->mech, &method, &ctl, la, i, duration);
    } else {
        for (u32 i = first; i < end; ++i) dbd_advance_group<f64>(&model->mech, &method, &ctl, la, i, duration);
    }
    return 0;
}
