// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// Thin C ABI over the reference's NFT channel system (sim/nft.cpp), compiled from
// the reference sources by include path (nothing copied) into oracle/_ref/. It
// includes the reference's test translation unit (tests/test_kinetics.cpp, main
// renamed) for its window driver nft_run<V> (test_kinetics.cpp:503-511).
//
// What the tests use it for:
//   - nft_run<f32x8> / nft_run<f32>: the reference's whole-system windows;
//   - the same windows split at the transport (prepare / transport / finish):
//     nft_group_window's steps (nft.cpp:1142-1152) with the transport of every
//     group run after the other groups' plants, so that a GPU transport can take
//     its place between the two halves (groups are independent within a window);
//   - nft_transport<f32x8> (nft.cpp:1028-1106) on caller arrays, for fixtures;
//   - the layout of the group arrays (nft.cpp:134-203), for the ABI test.
// The reference's transport runs under NftFlushDenormals (nft.cpp:1130-1136):
// FTZ/DAZ on x86-64 hosts, IEEE elsewhere (the struct is empty there).

#define main reference_test_kinetics_main
#include "tests/test_kinetics.cpp"
#undef main

#include <stddef.h>

#define REF_API extern "C" __attribute__((visibility("default")))

struct RefNft {
    NftSystem *s;
    u8 *memory;
    f32 shift[NftF_Count];
    b32 rebase;
    NftEnv env;
};

static const u64 kNftMemory = 256ull << 20;

REF_API void *ref_nft_create(u32 rails, f32 rail_length_m, u32 plants_per_rail) {
    RefNft *h = (RefNft *)calloc(1, sizeof(RefNft));
    h->memory = (u8 *)calloc(1, kNftMemory);
    Arena arena = arena_make(h->memory, kNftMemory);
    NftParams p = nft_default_params();
    p.rails = rails;
    if (rail_length_m > 0.0f) p.rail_length_m = rail_length_m;
    if (plants_per_rail) p.plants_per_rail = plants_per_rail;
    h->s = push_struct(&arena, NftSystem);
    nft_init(h->s, &arena, p);
    return h;
}

REF_API void ref_nft_destroy(void *hv) {
    RefNft *h = (RefNft *)hv;
    free(h->memory);
    free(h);
}

// rails, groups, cells, sites, site_offset, site_stride, substeps, lanes per group
REF_API void ref_nft_info(void *hv, u32 *out) {
    NftSystem *s = ((RefNft *)hv)->s;
    out[0] = s->rails; out[1] = s->groups; out[2] = s->cells; out[3] = s->sites;
    out[4] = s->site_offset; out[5] = s->site_stride; out[6] = s->substeps; out[7] = NFT_LANES;
}

// The reference's own window driver (test_kinetics.cpp:503-511).
REF_API void ref_nft_run(void *hv, u32 windows, u32 scalar_lanes) {
    NftSystem *s = ((RefNft *)hv)->s;
    if (scalar_lanes) nft_run<f32>(s, windows);
    else nft_run<f32x8>(s, windows);
}

// One window split at the transport: nft_window_begin, then per group the steps of
// nft_group_window before its transport (rebase, root-mat cells when due, plants).
REF_API void ref_nft_window_prepare(void *hv) {
    RefNft *h = (RefNft *)hv;
    NftSystem *s = h->s;
    h->env = nft_window_begin(s, h->shift, &h->rebase);
    for (u32 g = 0; g < s->groups; ++g) {
        NftGroup *grp = s->group + g;
        NftFlushDenormals ftz;
        if (h->rebase)
            for (u32 lane = 0; lane < NFT_LANES; lane += LaneTraits<f32x8>::width) nft_rebase<f32x8>(grp, lane, s->cells, h->shift);
        if (nft_cells_due(s, g)) nft_group_cells(s, g, s->ref, 1);
        for (u32 lane = 0; lane < NFT_LANES; lane += LaneTraits<f32x8>::width)
            nft_plants<f32x8>(grp, lane, s->sites, s->site_offset, s->site_stride, (f32)s->window_s, (f32)s->dt_sub, &h->env, s->ref);
    }
}

// The reference's transport of every group (nft_group_window's last step).
REF_API void ref_nft_window_transport(void *hv) {
    RefNft *h = (RefNft *)hv;
    NftSystem *s = h->s;
    for (u32 g = 0; g < s->groups; ++g) {
        NftFlushDenormals ftz;
        for (u32 lane = 0; lane < NFT_LANES; lane += LaneTraits<f32x8>::width)
            nft_transport<f32x8>(s->group + g, lane, s->cells, s->sites, s->site_offset, s->site_stride, s->ref, &h->env, s->substeps);
    }
}

REF_API void ref_nft_window_finish(void *hv) { nft_window_end(((RefNft *)hv)->s); }

// This window's transport inputs: ref[NftF_Count]; env = T_amb, radiant, e0, es_slope;
// returns the substeps per window (re-derived whenever the hydraulics are re-solved).
REF_API u32 ref_nft_window_inputs(void *hv, f32 *ref, f32 *env) {
    RefNft *h = (RefNft *)hv;
    for (u32 k = 0; k < NftF_Count; ++k) ref[k] = h->s->ref[k];
    env[0] = h->env.T_amb; env[1] = h->env.radiant; env[2] = h->env.e0; env[3] = h->env.es_slope;
    return h->s->substeps;
}

// Host addresses of group g's arrays: rows, hot, cold, sites, out_sum, lp.evap_kg.
REF_API void ref_nft_group_arrays(void *hv, u32 g, void **out) {
    NftGroup *grp = ((RefNft *)hv)->s->group + g;
    out[0] = grp->rows; out[1] = grp->hot; out[2] = grp->cold; out[3] = grp->sites;
    out[4] = grp->out_sum; out[5] = grp->lp.evap_kg;
}

static u64 fnv_bytes(u64 h, const void *p, u64 n) {
    const u8 *b = (const u8 *)p;
    for (u64 i = 0; i < n; ++i) { h ^= b[i]; h *= 0x100000001b3ull; }
    return h;
}

// FNV-1a over what the reference's f32x8-vs-f32 test compares (test_kinetics.cpp:528-534):
// the reservoir record and every group's rows, sites, hot and cold arrays.
REF_API u64 ref_nft_digest(void *hv) {
    NftSystem *s = ((RefNft *)hv)->s;
    u64 h = fnv_bytes(0xcbf29ce484222325ull, &s->res, sizeof(s->res));
    for (u32 g = 0; g < s->groups; ++g) {
        h = fnv_bytes(h, s->group[g].rows, sizeof(NftRow) * s->cells);
        h = fnv_bytes(h, s->group[g].sites, sizeof(NftSiteRow) * s->sites);
        h = fnv_bytes(h, s->group[g].hot, sizeof(NftCellHot) * s->cells);
        h = fnv_bytes(h, s->group[g].cold, sizeof(NftCellCold) * s->cells);
    }
    return h;
}

// Sizes and byte offsets of the group arrays (nft.cpp:134-203).
REF_API void ref_nft_layout(u64 *out) {
    out[0] = NFT_LANES; out[1] = NftF_Count;
    out[2] = sizeof(NftRow); out[3] = sizeof(NftCellHot); out[4] = sizeof(NftCellCold); out[5] = sizeof(NftSiteRow);
    out[6] = offsetof(NftCellHot, c); out[7] = offsetof(NftCellHot, kT); out[8] = offsetof(NftCellHot, bT);
    out[9] = offsetof(NftCellHot, ko);
    out[10] = offsetof(NftCellCold, kw); out[11] = offsetof(NftCellCold, kr); out[12] = offsetof(NftCellCold, ge);
    out[13] = offsetof(NftCellCold, ev);
    out[14] = offsetof(NftSiteRow, drop); out[15] = offsetof(NftSiteRow, removed);
}

// nft_transport<f32x8> (nft.cpp:1028-1106) of one group over caller arrays (32-byte
// aligned, the reference's layouts). out_sum [NftF_Count][8] and evap_kg[8] receive the
// group's outputs. ieee = 0: under the reference's denormal mode for this host
// (NftFlushDenormals: FTZ/DAZ on x86-64); ieee = 1: without it, as the reference runs on
// hosts where that struct is empty.
REF_API void ref_nft_transport_arrays(f32 *rows, f32 *hot, f32 *cold, f32 *sites, f32 *out_sum, f32 *evap_kg, u32 cells,
                                      u32 sites_count, u32 site_offset, u32 site_stride, const f32 *ref, const f32 *env4,
                                      u32 substeps, u32 ieee) {
    NftGroup *grp = (NftGroup *)aligned_alloc(64, (sizeof(NftGroup) + 63) & ~(size_t)63);
    memset(grp, 0, sizeof(NftGroup));
    grp->rows = (NftRow *)rows;
    grp->hot = (NftCellHot *)hot;
    grp->cold = (NftCellCold *)cold;
    grp->sites = (NftSiteRow *)sites;
    NftEnv env = {};
    env.T_amb = env4[0]; env.radiant = env4[1]; env.e0 = env4[2]; env.es_slope = env4[3];
    if (ieee) {
        for (u32 lane = 0; lane < NFT_LANES; lane += LaneTraits<f32x8>::width)
            nft_transport<f32x8>(grp, lane, cells, sites_count, site_offset, site_stride, ref, &env, substeps);
    } else {
        NftFlushDenormals ftz;
        for (u32 lane = 0; lane < NFT_LANES; lane += LaneTraits<f32x8>::width)
            nft_transport<f32x8>(grp, lane, cells, sites_count, site_offset, site_stride, ref, &env, substeps);
    }
    memcpy(out_sum, grp->out_sum, sizeof(grp->out_sum));
    memcpy(evap_kg, grp->lp.evap_kg, sizeof(grp->lp.evap_kg));
    free(grp);
}
