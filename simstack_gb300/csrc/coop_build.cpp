// Host side of the cooperative kernels: the wide-index mechanism image
// (coop.h) built from a finalized Model's symbolic phase.
#include <string.h>

#include "coop.h"
#include "mech.h"

namespace sgb {

namespace {
uint32_t align16(size_t v) { return (uint32_t)((v + 15) / 16 * 16); }
}   // namespace

bool coop_image(const Model &m, std::vector<uint8_t> *out) {
    if (!m.finalized) return false;
    const Symbolic &S = m.sym;
    const uint32_t n = m.n(), R = m.R();
    if (n == 0 || n > 256) return false;   // pattern rows are 256-bit masks
    auto pat_at = [&](uint32_t i, uint32_t j) { return S.pattern[(size_t)i * n + j] != 0; };

    CoopMech h;
    memset(&h, 0, sizeof(h));
    h.n = n;
    h.R = R;
    h.ld = n | 1u;
    h.nnz = S.nnz;

    std::vector<uint16_t> reac((size_t)R * 4, 0);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        if (rx.reactants.size() > 3) return false;
        reac[(size_t)r * 4] = (uint16_t)rx.reactants.size();
        for (size_t p = 0; p < rx.reactants.size(); ++p) reac[(size_t)r * 4 + 1 + p] = (uint16_t)rx.reactants[p];
    }
    // RHS terms per species, reactions ascending
    std::vector<std::vector<CoopTerm>> fs(n);
    for (uint32_t r = 0; r < R; ++r)
        for (auto &e : m.reactions[r].net) fs[e.first].push_back({r, (float)e.second});
    std::vector<uint32_t> fbeg(n + 1, 0);
    std::vector<CoopTerm> fent;
    for (uint32_t s = 0; s < n; ++s) {
        fbeg[s] = (uint32_t)fent.size();
        fent.insert(fent.end(), fs[s].begin(), fs[s].end());
    }
    fbeg[n] = (uint32_t)fent.size();
    // Jacobian terms per compact slot, (r, p, e) ascending; entries = slots some reaction scatters into
    std::vector<std::vector<CoopTerm>> js(S.nnz);
    for (uint32_t r = 0; r < R; ++r) {
        const Reaction &rx = m.reactions[r];
        for (size_t p = 0; p < rx.reactants.size(); ++p)
            for (size_t e = 0; e < rx.net.size(); ++e)
                js[rx.jac_slot[p][e]].push_back({r | ((uint32_t)p << 24), (float)(-rx.net[e].second)});
    }
    std::vector<uint32_t> slot_row(S.nnz), slot_col(S.nnz);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < n; ++j) {
            uint32_t s = S.slot[(size_t)i * n + j];
            if (s != ~0u) {
                slot_row[s] = i;
                slot_col[s] = j;
            }
        }
    std::vector<uint32_t> jbeg, jpos, jrow(n + 1, 0);
    std::vector<uint16_t> jcol;
    std::vector<CoopTerm> jent;
    for (uint32_t s = 0; s < S.nnz; ++s) {   // slots are row-major, so entries come out sorted by row
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

}   // namespace sgb
