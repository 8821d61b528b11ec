// Host side of the cooperative kernels: the wide-index mechanism image
// (coop.h) built from a finalized Model's symbolic phase or from a
// reference-layout KinMech (the same pattern, slots and scatter lists).
#include <string.h>

#include "coop.h"
#include "mech.h"

namespace sgb {

namespace {
uint32_t align16(size_t v) { return (uint32_t)((v + 15) / 16 * 16); }

// What the image needs, from either source (a Model or a reference-layout KinMech).
struct Desc {
    uint32_t n = 0, R = 0, nnz = 0;
    std::vector<std::vector<uint32_t>> reactants;                   // per reaction, equation order
    std::vector<std::vector<std::pair<uint32_t, int32_t>>> net;     // per reaction, (species, change)
    std::vector<std::vector<std::vector<uint32_t>>> jac_slot;       // [r][p][e] -> compact slot
    std::vector<uint8_t> pattern;                                   // n x n after fill-in
    std::vector<uint32_t> slot;                                     // n x n -> compact slot or ~0u
};

bool build_image(const Desc &d, std::vector<uint8_t> *out);

}   // namespace

bool coop_image(const Model &m, std::vector<uint8_t> *out) {
    if (!m.finalized) return false;
    Desc d;
    d.n = m.n();
    d.R = m.R();
    d.nnz = m.sym.nnz;
    for (const Reaction &rx : m.reactions) {
        d.reactants.push_back(rx.reactants);
        d.net.push_back(rx.net);
        d.jac_slot.push_back(rx.jac_slot);
    }
    d.pattern = m.sym.pattern;
    d.slot = m.sym.slot;
    return build_image(d, out);
}

bool coop_image(const KinMech &k, std::vector<uint8_t> *out) {
    Desc d;
    d.n = k.species_count;
    d.R = k.reaction_count;
    d.nnz = k.nnz;
    const uint32_t n = d.n;
    if (n == 0 || n > KIN_MAX_SPECIES || d.R > KIN_MAX_REACTIONS) return false;
    d.pattern.assign((size_t)n * n, 0);
    d.slot.assign((size_t)n * n, ~0u);
    auto put = [&](uint32_t i, uint32_t j, uint32_t s) {
        d.pattern[(size_t)i * n + j] = 1;
        d.slot[(size_t)i * n + j] = s;
    };
    for (uint32_t i = 0; i < n; ++i) {
        put(i, i, k.diag[i]);
        for (uint32_t e = k.lower_begin[i]; e < k.lower_begin[i + 1]; ++e) put(i, k.lower[e].col, k.lower[e].index);
        for (uint32_t e = k.upper_begin[i]; e < k.upper_begin[i + 1]; ++e) put(i, k.upper[e].col, k.upper[e].index);
    }
    for (uint32_t r = 0; r < d.R; ++r) {
        const KinReaction &rx = k.reactions[r];
        std::vector<uint32_t> re;
        for (uint32_t p = 0; p < rx.reactant_count; ++p) re.push_back(rx.reactant[p]);
        std::vector<std::pair<uint32_t, int32_t>> nt;
        for (uint32_t e = 0; e < rx.net_count; ++e) nt.push_back({rx.net_species[e], (int32_t)rx.net_coef[e]});
        std::vector<std::vector<uint32_t>> js(rx.reactant_count, std::vector<uint32_t>(rx.net_count));
        for (uint32_t p = 0; p < rx.reactant_count; ++p)
            for (uint32_t e = 0; e < rx.net_count; ++e) js[p][e] = rx.jac_index[p][e];
        d.reactants.push_back(re);
        d.net.push_back(nt);
        d.jac_slot.push_back(js);
    }
    return build_image(d, out);
}

namespace {

bool build_image(const Desc &d, std::vector<uint8_t> *out) {
    const uint32_t n = d.n, R = d.R;
    if (n == 0 || n > 256) return false;   // pattern rows are 256-bit masks
    auto pat_at = [&](uint32_t i, uint32_t j) { return d.pattern[(size_t)i * n + j] != 0; };

    CoopMech h;
    memset(&h, 0, sizeof(h));
    h.n = n;
    h.R = R;
    h.ld = n | 1u;
    h.nnz = d.nnz;

    std::vector<uint16_t> reac((size_t)R * 4, 0);
    for (uint32_t r = 0; r < R; ++r) {
        if (d.reactants[r].size() > 3) return false;
        reac[(size_t)r * 4] = (uint16_t)d.reactants[r].size();
        for (size_t p = 0; p < d.reactants[r].size(); ++p) reac[(size_t)r * 4 + 1 + p] = (uint16_t)d.reactants[r][p];
    }
    // RHS terms per species, reactions ascending
    std::vector<std::vector<CoopTerm>> fs(n);
    for (uint32_t r = 0; r < R; ++r)
        for (auto &e : d.net[r]) fs[e.first].push_back({r, (float)e.second});
    std::vector<uint32_t> fbeg(n + 1, 0);
    std::vector<CoopTerm> fent;
    for (uint32_t s = 0; s < n; ++s) {
        fbeg[s] = (uint32_t)fent.size();
        fent.insert(fent.end(), fs[s].begin(), fs[s].end());
    }
    fbeg[n] = (uint32_t)fent.size();
    // Jacobian terms per compact slot, (r, p, e) ascending; entries = slots some reaction scatters into
    std::vector<std::vector<CoopTerm>> js(d.nnz);
    for (uint32_t r = 0; r < R; ++r)
        for (size_t p = 0; p < d.reactants[r].size(); ++p)
            for (size_t e = 0; e < d.net[r].size(); ++e) {
                const uint32_t sl = d.jac_slot[r][p][e];
                if (sl >= d.nnz) return false;
                js[sl].push_back({r | ((uint32_t)p << 24), (float)(-d.net[r][e].second)});
            }
    std::vector<uint32_t> slot_row(d.nnz), slot_col(d.nnz);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < n; ++j) {
            uint32_t s = d.slot[(size_t)i * n + j];
            if (s != ~0u) {
                slot_row[s] = i;
                slot_col[s] = j;
            }
        }
    std::vector<uint32_t> jbeg, jpos, jrow(n + 1, 0);
    std::vector<uint16_t> jcol;
    std::vector<CoopTerm> jent;
    for (uint32_t s = 0; s < d.nnz; ++s) {   // slots are row-major, so entries come out sorted by row
        if (js[s].empty()) continue;
        jbeg.push_back((uint32_t)jent.size());
        jent.insert(jent.end(), js[s].begin(), js[s].end());
        jpos.push_back(slot_row[s] * h.ld + slot_col[s]);
        jcol.push_back((uint16_t)slot_col[s]);
        jrow[slot_row[s] + 1]++;
    }
    h.nj = (uint32_t)jpos.size();
    jbeg.push_back((uint32_t)jent.size());
    for (uint32_t i = 0; i < n; ++i) jrow[i + 1] += jrow[i];
    // elimination lists
    std::vector<uint32_t> lbeg(n + 1), ubeg(n + 1), cbeg(n + 1);
    std::vector<uint16_t> lrow, ucol, crow;
    for (uint32_t k = 0; k < n; ++k) {
        lbeg[k] = (uint32_t)lrow.size();
        ubeg[k] = (uint32_t)ucol.size();
        cbeg[k] = (uint32_t)crow.size();
        for (uint32_t i = k + 1; i < n; ++i)
            if (pat_at(i, k)) lrow.push_back((uint16_t)i);
        for (uint32_t j = k + 1; j < n; ++j)
            if (pat_at(k, j)) ucol.push_back((uint16_t)j);
        for (uint32_t i = 0; i < k; ++i)
            if (pat_at(i, k)) crow.push_back((uint16_t)i);
        h.lu_updates += (uint64_t)(lrow.size() - lbeg[k]) * (ucol.size() - ubeg[k]);
    }
    lbeg[n] = (uint32_t)lrow.size();
    ubeg[n] = (uint32_t)ucol.size();
    cbeg[n] = (uint32_t)crow.size();
    std::vector<uint32_t> pat((size_t)n * 8, 0u);
    std::vector<uint16_t> lcnt(n, 0);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < n; ++j)
            if (pat_at(i, j)) {
                pat[(size_t)i * 8 + (j >> 5)] |= 1u << (j & 31);
                if (i > j) lcnt[j]++;
            }
    h.fun_terms = (uint32_t)fent.size();
    h.jac_terms = (uint32_t)jent.size();
    h.l_entries = (uint32_t)lrow.size();
    h.u_entries = (uint32_t)ucol.size();

    // layout
    size_t off = align16(sizeof(CoopMech));
    auto place = [&](uint32_t *field, size_t bytes) {
        *field = (uint32_t)off;
        off = align16(off + bytes);
    };
    place(&h.off_reac, reac.size() * 2);
    place(&h.off_fbeg, fbeg.size() * 4);
    place(&h.off_fent, fent.size() * sizeof(CoopTerm));
    place(&h.off_jbeg, jbeg.size() * 4);
    place(&h.off_jent, jent.size() * sizeof(CoopTerm));
    place(&h.off_jpos, jpos.size() * 4);
    place(&h.off_jrow, jrow.size() * 4);
    place(&h.off_jcol, jcol.size() * 2);
    place(&h.off_lbeg, lbeg.size() * 4);
    place(&h.off_lrow, lrow.size() * 2);
    place(&h.off_ubeg, ubeg.size() * 4);
    place(&h.off_ucol, ucol.size() * 2);
    place(&h.off_cbeg, cbeg.size() * 4);
    place(&h.off_crow, crow.size() * 2);
    place(&h.off_pat, pat.size() * 4);
    place(&h.off_lcnt, lcnt.size() * 2);
    if (off > 0xffffffffu) return false;
    h.bytes = (uint32_t)off;
    out->assign(off, 0);
    uint8_t *b = out->data();
    memcpy(b, &h, sizeof(h));
    auto put = [&](uint32_t o, const void *src, size_t bytes) {
        if (bytes) memcpy(b + o, src, bytes);
    };
    put(h.off_reac, reac.data(), reac.size() * 2);
    put(h.off_fbeg, fbeg.data(), fbeg.size() * 4);
    put(h.off_fent, fent.data(), fent.size() * sizeof(CoopTerm));
    put(h.off_jbeg, jbeg.data(), jbeg.size() * 4);
    put(h.off_jent, jent.data(), jent.size() * sizeof(CoopTerm));
    put(h.off_jpos, jpos.data(), jpos.size() * 4);
    put(h.off_jrow, jrow.data(), jrow.size() * 4);
    put(h.off_jcol, jcol.data(), jcol.size() * 2);
    put(h.off_lbeg, lbeg.data(), lbeg.size() * 4);
    put(h.off_lrow, lrow.data(), lrow.size() * 2);
    put(h.off_ubeg, ubeg.data(), ubeg.size() * 4);
    put(h.off_ucol, ucol.data(), ucol.size() * 2);
    put(h.off_cbeg, cbeg.data(), cbeg.size() * 4);
    put(h.off_crow, crow.data(), crow.size() * 2);
    put(h.off_pat, pat.data(), pat.size() * 4);
    put(h.off_lcnt, lcnt.data(), lcnt.size() * 2);
    return true;
}

}   // namespace

}   // namespace sgb
