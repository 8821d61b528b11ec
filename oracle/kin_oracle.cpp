// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// CPU oracle for SimStack's batched Rosenbrock stiff-chemistry path. Only the
// tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py load
// this library, and only to check (or time beside) the GPU module. Nothing in
// simstack_gb300/ links or calls it.
//
// It restates, for scalar lanes (one cell at a time), the reference's
//   - mechanism builder and symbolic sparse-LU phase
//       src/sim/kinetics/kin_build.cpp:78-223 (kin_add_species,
//       kin_add_reaction, kin_mech_finalize)
//   - rate laws             kin_build.cpp:226-244 (kin_eval_rate_constants)
//   - RHS / -J / LU / solve src/sim/kinetics/kin_solver.h:40-139
//   - adaptive Rosenbrock   kin_solver.h:169-313 (kin_step_factor, kin_integrate)
//   - pulse segments        kin_solver.h:322-347 (kin_advance)
//   - lane-group load/store src/sim/dbd_lanes.h:28-78 (dbd_advance_group)
//   - method coefficients   kin_solver.h:352-395 (kin_method)
//   - cube root             src/base/base_lane.h:123-135 (lane_cbrt_clamped)
//   - shipped mechanism     src/sim/kinetics/air_mech.cpp:30-103 (air_mech_define)
//   - discharge source      air_mech.cpp:184-276 (air_branch, air_source_delta)
//   - plug-flow / upwind    src/sim/nft.cpp:1070-1079 (x_j += c (x_{j-1} - x_j))
// with 32-bit indices, so mechanisms larger than the reference's u16 tables
// (the 200-species synthetic mechanism) run through the same operation order.
//
// Every floating-point operation is performed in the reference's order and
// with fused multiply-adds exactly where the reference calls lane_fmadd /
// lane_fnmadd; the file must be compiled with -ffp-contract=off so the
// compiler adds no others. Under that rule the scalar lanes here produce the
// same bits as the reference's f64 / f64x4 (and f32 / f32x8) lanes; the tests
// pin that against the reference compiled from its own sources.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace oracle {

typedef uint8_t u8;
typedef uint16_t u16;
typedef uint32_t u32;
typedef uint64_t u64;
typedef int32_t s32;

enum { kMaxReactants = 3, kMaxNet = 6, kElements = 3 };

enum RateKind { kArrhenius = 0, kThirdBody = 1, kTroe = 2, kEqReverse = 3 };

struct RateLaw {
    s32 kind;
    double A, n, E, A_inf, n_inf, fc;
    s32 ref;
    double keq_A, keq_B;
};

struct Reaction {
    u32 reactant_count;
    u32 reactant[kMaxReactants];
    u32 net_count;
    u32 net_species[kMaxNet];
    s32 net_coef[kMaxNet];
    u32 jac_index[kMaxReactants][kMaxNet];
};

struct LuPivot {   // one elimination: l = a[ik] * a[kk], then a[ij] -= l * a[kj] for sub ops [sub_begin, sub_end)
    u32 ik, kk, sub_begin, sub_end;
};
struct LuUpdate {
    u32 ij, kj;
};
struct RowEntry {
    u32 index, col;
};

struct Mechanism {
    std::vector<std::string> names;
    std::vector<std::vector<u8>> elements;
    std::vector<Reaction> reactions;
    std::vector<RateLaw> laws;
    std::vector<std::string> equations;
    // symbolic phase
    u32 nnz = 0;
    std::vector<u32> diag, pivot_begin, lower_begin, upper_begin;
    std::vector<LuPivot> pivots;
    std::vector<LuUpdate> updates;
    std::vector<RowEntry> lower, upper;
    std::vector<u8> pattern;       // n*n, after fill-in
    std::vector<u8> jac_pattern;   // n*n, J + diagonal before fill-in
    std::vector<u32> slot;         // n*n -> compact index (or ~0u)
    bool failed = false;
    std::string error;
    u32 n() const { return (u32)names.size(); }
    u32 R() const { return (u32)reactions.size(); }
};

static void fail(Mechanism *m, const char *what, const char *detail) {
    if (m->failed) return;
    m->failed = true;
    m->error = std::string(what) + ": " + detail;
}

// Element counts of a formula over N, O, H ("HNO3", "N2(A)"): kin_build.cpp:62-76.
static bool parse_formula(const char *name, u8 *counts) {
    static const char symbols[kElements] = {'N', 'O', 'H'};
    for (int e = 0; e < kElements; ++e) counts[e] = 0;
    for (const char *p = name; *p && *p != '(';) {
        int element = -1;
        for (int e = 0; e < kElements; ++e)
            if (*p == symbols[e]) element = e;
        if (element < 0) return false;
        ++p;
        u32 count = 0;
        while (*p >= '0' && *p <= '9') count = count * 10 + (u32)(*p++ - '0');
        counts[element] = (u8)(counts[element] + (count ? count : 1));
    }
    return true;
}

static u32 add_species(Mechanism *m, const char *name, bool abstract_species) {
    std::vector<u8> counts(kElements, 0);
    if (!abstract_species && !parse_formula(name, counts.data())) fail(m, "species formula must use N, O, H", name);
    m->names.push_back(name);
    m->elements.push_back(counts);
    return m->n() - 1;
}

static int find_species(const Mechanism *m, const char *name) {
    for (u32 s = 0; s < m->n(); ++s)
        if (m->names[s] == name) return (int)s;
    return -1;
}

// "O + O2 + M -> O3 + M": kin_build.cpp:100-148. Reactants in equation
// order; net species in species-index order with non-zero net change.
static u32 add_reaction(Mechanism *m, const char *equation, const RateLaw &law) {
    Reaction rx;
    memset(&rx, 0, sizeof(rx));
    u32 r = m->R();
    m->laws.push_back(law);
    m->equations.push_back(equation);
    std::vector<int> net(m->n(), 0);
    int balance[kElements] = {0, 0, 0};
    bool products = false;
    const char *p = equation;
    while (*p) {
        while (*p == ' ' || *p == '+') ++p;
        if (!*p) break;
        if (p[0] == '-' && p[1] == '>') {
            products = true;
            p += 2;
            continue;
        }
        char token[16];
        u32 len = 0;
        while (*p && *p != ' ' && *p != '+' && !(p[0] == '-' && p[1] == '>') && len < sizeof(token) - 1) token[len++] = *p++;
        token[len] = 0;
        if (strcmp(token, "M") == 0) continue;
        int s = find_species(m, token);
        if (s < 0) {
            fail(m, "unknown species in reaction", equation);
            m->reactions.push_back(rx);
            return r;
        }
        if (!products) {
            if (rx.reactant_count >= kMaxReactants) {
                fail(m, "too many reactants", equation);
                m->reactions.push_back(rx);
                return r;
            }
            rx.reactant[rx.reactant_count++] = (u32)s;
            net[s] -= 1;
            for (int e = 0; e < kElements; ++e) balance[e] -= m->elements[s][e];
        } else {
            net[s] += 1;
            for (int e = 0; e < kElements; ++e) balance[e] += m->elements[s][e];
        }
    }
    if (!products || rx.reactant_count == 0) fail(m, "reaction needs reactants and '->'", equation);
    for (int e = 0; e < kElements; ++e)
        if (balance[e] != 0) fail(m, "element balance violated", equation);
    if (law.kind == kEqReverse && (u32)law.ref >= r) fail(m, "reverse reaction must follow its forward reaction", equation);
    for (u32 s = 0; s < m->n(); ++s) {
        if (net[s] == 0) continue;
        if (rx.net_count >= kMaxNet) {
            fail(m, "too many net species", equation);
            break;
        }
        rx.net_species[rx.net_count] = s;
        rx.net_coef[rx.net_count] = net[s];
        ++rx.net_count;
    }
    m->reactions.push_back(rx);
    return r;
}

// Symbolic phase, kin_build.cpp:152-223: pattern = J + diagonal, IKJ fill-in
// of the no-pivot LU, row-major compact numbering, elimination op lists, and
// triangular-solve lists (lower ascending column, upper DESCENDING column).
static void finalize(Mechanism *m) {
    const u32 n = m->n();
    std::vector<u8> &pat = m->pattern;
    pat.assign((size_t)n * n, 0);
    for (u32 i = 0; i < n; ++i) pat[(size_t)i * n + i] = 1;
    for (const Reaction &rx : m->reactions)
        for (u32 p = 0; p < rx.reactant_count; ++p)
            for (u32 e = 0; e < rx.net_count; ++e) pat[(size_t)rx.net_species[e] * n + rx.reactant[p]] = 1;
    m->jac_pattern = pat;
    for (u32 i = 1; i < n; ++i)
        for (u32 k = 0; k < i; ++k)
            if (pat[(size_t)i * n + k])
                for (u32 j = k + 1; j < n; ++j)
                    if (pat[(size_t)k * n + j]) pat[(size_t)i * n + j] = 1;

    std::vector<u32> index((size_t)n * n, 0xFFFFFFFFu);
    m->nnz = 0;
    for (u32 i = 0; i < n; ++i)
        for (u32 j = 0; j < n; ++j)
            if (pat[(size_t)i * n + j]) index[(size_t)i * n + j] = m->nnz++;
    m->slot = index;
    m->diag.resize(n);
    for (u32 i = 0; i < n; ++i) m->diag[i] = index[(size_t)i * n + i];

    m->pivots.clear();
    m->updates.clear();
    m->pivot_begin.assign(n + 1, 0);
    for (u32 i = 0; i < n; ++i) {
        m->pivot_begin[i] = (u32)m->pivots.size();
        for (u32 k = 0; k < i; ++k) {
            if (!pat[(size_t)i * n + k]) continue;
            LuPivot d;
            d.ik = index[(size_t)i * n + k];
            d.kk = index[(size_t)k * n + k];
            d.sub_begin = (u32)m->updates.size();
            for (u32 j = k + 1; j < n; ++j) {
                if (!pat[(size_t)k * n + j]) continue;
                m->updates.push_back({index[(size_t)i * n + j], index[(size_t)k * n + j]});
            }
            d.sub_end = (u32)m->updates.size();
            m->pivots.push_back(d);
        }
    }
    m->pivot_begin[n] = (u32)m->pivots.size();

    m->lower.clear();
    m->upper.clear();
    m->lower_begin.assign(n + 1, 0);
    m->upper_begin.assign(n + 1, 0);
    for (u32 i = 0; i < n; ++i) {
        m->lower_begin[i] = (u32)m->lower.size();
        m->upper_begin[i] = (u32)m->upper.size();
        for (u32 j = 0; j < i; ++j)
            if (pat[(size_t)i * n + j]) m->lower.push_back({index[(size_t)i * n + j], j});
        for (u32 j = n; j-- > i + 1;)
            if (pat[(size_t)i * n + j]) m->upper.push_back({index[(size_t)i * n + j], j});
    }
    m->lower_begin[n] = (u32)m->lower.size();
    m->upper_begin[n] = (u32)m->upper.size();

    for (Reaction &rx : m->reactions)
        for (u32 p = 0; p < rx.reactant_count; ++p)
            for (u32 e = 0; e < rx.net_count; ++e) rx.jac_index[p][e] = index[(size_t)rx.net_species[e] * n + rx.reactant[p]];
}

// kin_build.cpp:226-244; the operand order of each product is the reference's.
static void rate_constants(const Mechanism *m, double T, double M, double *k) {
    double t300 = T / 300.0;
    for (u32 r = 0; r < m->R(); ++r) {
        const RateLaw &l = m->laws[r];
        switch (l.kind) {
            case kArrhenius: k[r] = l.A * pow(t300, l.n) * exp(-l.E / T); break;
            case kThirdBody: k[r] = l.A * pow(t300, l.n) * exp(-l.E / T) * M; break;
            case kTroe: {
                double k0m = l.A * pow(t300, l.n) * M;
                double kinf = l.A_inf * pow(t300, l.n_inf);
                double ratio = k0m / kinf;
                double lg = log10(ratio);
                k[r] = (k0m / (1.0 + ratio)) * pow(l.fc, 1.0 / (1.0 + lg * lg));
            } break;
            case kEqReverse: k[r] = k[l.ref] / (l.keq_A * exp(l.keq_B / T)); break;
            default: k[r] = 0.0; break;
        }
    }
}

static RateLaw law_arr(double A, double n = 0.0, double E = 0.0) {
    RateLaw l = {};
    l.kind = kArrhenius; l.A = A; l.n = n; l.E = E;
    return l;
}
static RateLaw law_m(double A, double n = 0.0, double E = 0.0) {
    RateLaw l = {};
    l.kind = kThirdBody; l.A = A; l.n = n; l.E = E;
    return l;
}
static RateLaw law_troe(double A0, double n0, double A_inf, double n_inf, double fc = 0.6) {
    RateLaw l = {};
    l.kind = kTroe; l.A = A0; l.n = n0; l.A_inf = A_inf; l.n_inf = n_inf; l.fc = fc;
    return l;
}
static RateLaw law_eq_reverse(u32 forward, double keq_A, double keq_B) {
    RateLaw l = {};
    l.kind = kEqReverse; l.ref = (s32)forward; l.keq_A = keq_A; l.keq_B = keq_B;
    return l;
}

// The shipped humid-air mechanism (air_mech.cpp:30-103): species order, equations and
// rate data are the reference's table, restated because the symbolic phase and the
// mechanism signature depend on them.
static void define_air(Mechanism *m) {
    static const char *species[] = {"O",  "O3",  "N",  "NO", "NO2", "NO3", "N2O5", "N2O", "HNO2",
                                    "HNO3", "OH", "HO2", "H2O2", "H", "N2", "O2", "H2O"};
    for (const char *s : species) add_species(m, s, false);
    add_reaction(m, "O + O2 + M -> O3 + M", law_m(6.0e-34, -2.4));
    add_reaction(m, "O + O3 -> O2 + O2", law_arr(8.0e-12, 0.0, 2060.0));
    add_reaction(m, "O + O + M -> O2 + M", law_m(5.2e-35, 0.0, -900.0));
    add_reaction(m, "O + NO + M -> NO2 + M", law_troe(9.0e-32, -1.5, 3.0e-11, 0.0));
    add_reaction(m, "O + NO2 -> NO + O2", law_arr(5.1e-12, 0.0, -210.0));
    add_reaction(m, "O + NO2 + M -> NO3 + M", law_troe(2.5e-31, -1.8, 2.2e-11, -0.7));
    add_reaction(m, "O3 + NO -> NO2 + O2", law_arr(3.0e-12, 0.0, 1500.0));
    add_reaction(m, "O3 + NO2 -> NO3 + O2", law_arr(1.2e-13, 0.0, 2450.0));
    add_reaction(m, "NO3 + NO -> NO2 + NO2", law_arr(1.5e-11, 0.0, -170.0));
    u32 r_n2o5 = add_reaction(m, "NO2 + NO3 + M -> N2O5 + M", law_troe(2.0e-30, -4.4, 1.4e-12, -0.7));
    add_reaction(m, "N2O5 + M -> NO2 + NO3 + M", law_eq_reverse(r_n2o5, 2.7e-27, 11000.0));
    add_reaction(m, "NO + NO + O2 -> NO2 + NO2", law_arr(3.3e-39, 0.0, -530.0));
    add_reaction(m, "N2O5 + H2O -> HNO3 + HNO3", law_arr(2.5e-22));
    add_reaction(m, "N + NO -> N2 + O", law_arr(2.1e-11, 0.0, -100.0));
    add_reaction(m, "N + O2 -> NO + O", law_arr(1.5e-11, 0.0, 3600.0));
    add_reaction(m, "N + NO2 -> N2O + O", law_arr(0.434 * 5.8e-12, 0.0, -220.0));
    add_reaction(m, "N + NO2 -> NO + NO", law_arr(0.333 * 5.8e-12, 0.0, -220.0));
    add_reaction(m, "N + NO2 -> N2 + O + O", law_arr(0.132 * 5.8e-12, 0.0, -220.0));
    add_reaction(m, "N + NO2 -> N2 + O2", law_arr(0.101 * 5.8e-12, 0.0, -220.0));
    add_reaction(m, "N + O + M -> NO + M", law_m(5.5e-33, 0.0, -155.0));
    add_reaction(m, "N + N + M -> N2 + M", law_m(8.3e-34, 0.0, -500.0));
    add_reaction(m, "N + OH -> NO + H", law_arr(4.7e-11));
    add_reaction(m, "OH + OH + M -> H2O2 + M", law_troe(6.9e-31, -1.0, 2.6e-11, 0.0));
    add_reaction(m, "OH + OH -> H2O + O", law_arr(1.8e-12));
    add_reaction(m, "OH + O -> H + O2", law_arr(1.8e-11, 0.0, -180.0));
    add_reaction(m, "OH + O3 -> HO2 + O2", law_arr(1.7e-12, 0.0, 940.0));
    add_reaction(m, "OH + HO2 -> H2O + O2", law_arr(4.8e-11, 0.0, -250.0));
    add_reaction(m, "OH + H2O2 -> HO2 + H2O", law_arr(1.8e-12));
    add_reaction(m, "HO2 + HO2 -> H2O2 + O2", law_arr(3.0e-13, 0.0, -460.0));
    add_reaction(m, "HO2 + O -> OH + O2", law_arr(3.0e-11, 0.0, -200.0));
    add_reaction(m, "HO2 + O3 -> OH + O2 + O2", law_arr(1.0e-14, 0.0, 490.0));
    add_reaction(m, "H + O2 + M -> HO2 + M", law_troe(4.4e-32, -1.3, 7.5e-11, 0.2));
    add_reaction(m, "H + O3 -> OH + O2", law_arr(1.4e-10, 0.0, 470.0));
    add_reaction(m, "H + HO2 -> OH + OH", law_arr(7.2e-11));
    add_reaction(m, "O + H2O2 -> OH + HO2", law_arr(1.4e-12, 0.0, 2000.0));
    add_reaction(m, "OH + NO + M -> HNO2 + M", law_troe(7.0e-31, -2.6, 3.6e-11, -0.1));
    add_reaction(m, "OH + NO2 + M -> HNO3 + M", law_troe(1.8e-30, -3.0, 2.8e-11, 0.0));
    add_reaction(m, "OH + HNO2 -> NO2 + H2O", law_arr(1.8e-11, 0.0, 390.0));
    add_reaction(m, "OH + HNO3 -> NO3 + H2O", law_arr(1.5e-13));
    add_reaction(m, "HO2 + NO -> OH + NO2", law_arr(3.3e-12, 0.0, -270.0));
    add_reaction(m, "H + NO2 -> OH + NO", law_arr(4.0e-10, 0.0, 340.0));
    add_reaction(m, "OH + NO3 -> HO2 + NO2", law_arr(2.2e-11));
    add_reaction(m, "HO2 + NO3 -> OH + NO2 + O2", law_arr(3.5e-12));
    add_reaction(m, "O3 + M -> O2 + O + M", law_m(7.2e-10, 0.0, 11400.0));
}

// ---------------------------------------------------------------------------
// Reference-layout KinMech bytes (src/sim/kinetics/kin_mech.h:42-87 at the
// default capacities), so the oracle's symbolic phase can be compared with the
// reference's byte for byte and by its FNV-1a signature.

enum { kRefMaxSpecies = 32, kRefMaxReactions = 96, kRefMaxNnz = 512, kRefMaxLuDiv = 512, kRefMaxLuSub = 4096 };
struct RefReaction {
    u8 reactant[3];
    u8 reactant_count;
    u8 net_count;
    u8 net_species[6];
    int8_t net_coef[6];
    u16 jac_index[3][6];
};
struct RefLuDiv { u16 ik, kk, sub_begin, sub_end; };
struct RefLuSub { u16 ij, kj; };
struct RefRowEntry { u16 index; u8 col; u8 pad; };
struct RefKinMech {
    u32 species_count;
    u32 reaction_count;
    RefReaction reactions[kRefMaxReactions];
    u32 nnz;
    u16 diag[kRefMaxSpecies];
    u32 lu_div_count, lu_sub_count;
    u16 div_begin[kRefMaxSpecies + 1];
    RefLuDiv lu_div[kRefMaxLuDiv];
    RefLuSub lu_sub[kRefMaxLuSub];
    u16 lower_begin[kRefMaxSpecies + 1];
    u16 upper_begin[kRefMaxSpecies + 1];
    RefRowEntry lower[kRefMaxNnz];
    RefRowEntry upper[kRefMaxNnz];
};
static_assert(sizeof(RefKinMech) == 30044, "reference KinMech layout");

static bool export_ref_layout(const Mechanism *m, RefKinMech *out) {
    memset(out, 0, sizeof(*out));
    if (m->n() > kRefMaxSpecies || m->R() > kRefMaxReactions || m->nnz > kRefMaxNnz || m->pivots.size() > kRefMaxLuDiv ||
        m->updates.size() > kRefMaxLuSub)
        return false;
    out->species_count = m->n();
    out->reaction_count = m->R();
    for (u32 r = 0; r < m->R(); ++r) {
        const Reaction &rx = m->reactions[r];
        RefReaction &o = out->reactions[r];
        for (u32 p = 0; p < 3; ++p) o.reactant[p] = p < rx.reactant_count ? (u8)rx.reactant[p] : 0xFF;
        o.reactant_count = (u8)rx.reactant_count;
        o.net_count = (u8)rx.net_count;
        for (u32 e = 0; e < rx.net_count; ++e) {
            o.net_species[e] = (u8)rx.net_species[e];
            o.net_coef[e] = (int8_t)rx.net_coef[e];
        }
        for (u32 p = 0; p < rx.reactant_count; ++p)
            for (u32 e = 0; e < rx.net_count; ++e) o.jac_index[p][e] = (u16)rx.jac_index[p][e];
    }
    out->nnz = m->nnz;
    for (u32 i = 0; i < m->n(); ++i) out->diag[i] = (u16)m->diag[i];
    out->lu_div_count = (u32)m->pivots.size();
    out->lu_sub_count = (u32)m->updates.size();
    for (u32 i = 0; i <= m->n(); ++i) {
        out->div_begin[i] = (u16)m->pivot_begin[i];
        out->lower_begin[i] = (u16)m->lower_begin[i];
        out->upper_begin[i] = (u16)m->upper_begin[i];
    }
    for (size_t d = 0; d < m->pivots.size(); ++d)
        out->lu_div[d] = {(u16)m->pivots[d].ik, (u16)m->pivots[d].kk, (u16)m->pivots[d].sub_begin, (u16)m->pivots[d].sub_end};
    for (size_t s = 0; s < m->updates.size(); ++s) out->lu_sub[s] = {(u16)m->updates[s].ij, (u16)m->updates[s].kj};
    for (size_t e = 0; e < m->lower.size(); ++e) out->lower[e] = {(u16)m->lower[e].index, (u8)m->lower[e].col, 0};
    for (size_t e = 0; e < m->upper.size(); ++e) out->upper[e] = {(u16)m->upper[e].index, (u8)m->upper[e].col, 0};
    return true;
}

static u64 fnv1a(const void *data, u64 size) {
    const u8 *p = (const u8 *)data;
    u64 h = 14695981039346656037ull;
    for (u64 i = 0; i < size; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

// ---------------------------------------------------------------------------
// Method coefficients: kin_solver.h:352-395 (KPP Rosenbrock family, Sandu et
// al., Atmos. Env. 1997). a and c packed strictly-lower: (i,j) at i(i-1)/2+j.

struct Method {
    u32 stages, order;
    double a[6], c[6], m[4], e[4], gamma0;
    int new_f[4];
};

static Method method_coefficients(int id) {
    Method r;
    memset(&r, 0, sizeof(r));
    if (id == 0) {   // Ros2
        double g = 1.0 + 1.0 / 1.4142135623730950488;
        r.stages = 2; r.order = 2;
        r.a[0] = 1.0 / g;
        r.c[0] = -2.0 / g;
        r.m[0] = 3.0 / (2.0 * g); r.m[1] = 1.0 / (2.0 * g);
        r.e[0] = 1.0 / (2.0 * g); r.e[1] = 1.0 / (2.0 * g);
        r.gamma0 = g;
        r.new_f[0] = r.new_f[1] = 1;
    } else if (id == 1) {   // Ros3
        r.stages = 3; r.order = 3;
        r.a[0] = 1.0; r.a[1] = 1.0; r.a[2] = 0.0;
        r.c[0] = -0.10156171083877702091975600115545e+01;
        r.c[1] = 0.40759956452537699824805835358067e+01;
        r.c[2] = 0.92076794298330791242156818474003e+01;
        r.m[0] = 0.1e+01;
        r.m[1] = 0.61697947043828245592553615689730e+01;
        r.m[2] = -0.42772256543218573326238373806514e+00;
        r.e[0] = 0.5e+00;
        r.e[1] = -0.29079558716805469821718236208017e+01;
        r.e[2] = 0.22354069897811569627360909276199e+00;
        r.gamma0 = 0.43586652150845899941601945119356;
        r.new_f[0] = 1; r.new_f[1] = 1; r.new_f[2] = 0;
    } else if (id == 2) {   // Rodas3
        r.stages = 4; r.order = 3;
        r.a[0] = 0.0; r.a[1] = 2.0; r.a[2] = 0.0; r.a[3] = 2.0; r.a[4] = 0.0; r.a[5] = 1.0;
        r.c[0] = 4.0; r.c[1] = 1.0; r.c[2] = -1.0; r.c[3] = 1.0; r.c[4] = -1.0; r.c[5] = -8.0 / 3.0;
        r.m[0] = 2.0; r.m[1] = 0.0; r.m[2] = 1.0; r.m[3] = 1.0;
        r.e[0] = 0.0; r.e[1] = 0.0; r.e[2] = 0.0; r.e[3] = 1.0;
        r.gamma0 = 0.5;
        r.new_f[0] = r.new_f[1] = r.new_f[2] = r.new_f[3] = 1;
    }
    return r;
}

// Tolerances and limits (kin_mech.h:112-120), passed in by value from Python.
struct Control {
    double rtol, atol, h_min, h_max, h_start;
    u32 max_steps;
    s32 fixed_step;
    s32 clamp_negative;
};

// ---------------------------------------------------------------------------
// Scalar-lane arithmetic. T = double (f64 lanes) or float (f32 lanes). Each
// helper is the reference lane operation of the same name (base_lane.h:47-117).

static inline double fmadd(double a, double b, double c) { return std::fma(a, b, c); }
static inline float fmadd(float a, float b, float c) { return std::fma(a, b, c); }
template <class T> static inline T fnmadd(T a, T b, T c) { return fmadd(-a, b, c); }
template <class T> static inline T vmin(T a, T b) { return a < b ? a : b; }
template <class T> static inline T vmax(T a, T b) { return a > b ? a : b; }
template <class T> static inline T vabs(T a) { return a < (T)0 ? -a : a; }
static inline double vsqrt(double a) { return std::sqrt(a); }
static inline float vsqrt(float a) { return std::sqrt(a); }
template <class T> static inline bool finite(T a) { T d = a - a; return d == d; }

// x^(1/3) on [1e-4, 1e4] from six square roots and two Newton steps (base_lane.h:123-135).
template <class T> static inline T cbrt_clamped(T x) {
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

template <class T> static inline T step_factor(T err, u32 order) {
    T e = vmin(vmax(err, (T)1e-4), (T)1e4);
    T root;
    if (order == 2) root = vsqrt(e);
    else if (order == 4) root = vsqrt(vsqrt(e));
    else root = cbrt_clamped(e);
    T fac = (T)0.9 / root;
    return vmin(vmax(fac, (T)0.2), (T)6.0);
}

// The mixed lanes' step-size factor (the GPU's step_factor_mixed): order 3 from the FP32
// cube-root chain, one division-free FP64 Newton step for e^(-1/3), fac = 0.9 w.
static inline double step_factor_mixed(double err, u32 order) {
    if (order != 3) return step_factor(err, order);
    const double e = vmin(vmax(err, 1e-4), 1e4);
    const float g = cbrt_clamped((float)e);
    double w = (double)(1.0f / g);
    const double w3 = w * w * w;
    w = w * (4.0 - e * w3) * (1.0 / 3.0);
    const double fac = 0.9 * w;
    return vmin(vmax(fac, 0.2), 6.0);
}

template <class T> static void eval_fun(const Mechanism &m, const T *k, const T *src, const T *y, T *f) {
    const u32 n = m.n();
    for (u32 s = 0; s < n; ++s) f[s] = src[s];
    for (const Reaction &rx : m.reactions) {
        size_t r = &rx - m.reactions.data();
        T rate = k[r];
        for (u32 p = 0; p < rx.reactant_count; ++p) rate = rate * y[rx.reactant[p]];
        for (u32 e = 0; e < rx.net_count; ++e) {
            u32 s = rx.net_species[e];
            f[s] = fmadd((T)(double)rx.net_coef[e], rate, f[s]);
        }
    }
}

// a = -J over the compact pattern (fill-in stays zero).
template <class T> static void eval_neg_jac(const Mechanism &m, const T *k, const T *y, T *a) {
    for (u32 i = 0; i < m.nnz; ++i) a[i] = (T)0.0;
    for (const Reaction &rx : m.reactions) {
        size_t r = &rx - m.reactions.data();
        for (u32 p = 0; p < rx.reactant_count; ++p) {
            T d = k[r];
            for (u32 q = 0; q < rx.reactant_count; ++q)
                if (q != p) d = d * y[rx.reactant[q]];
            for (u32 e = 0; e < rx.net_count; ++e) {
                u32 idx = rx.jac_index[p][e];
                a[idx] = fmadd((T)(-(double)rx.net_coef[e]), d, a[idx]);
            }
        }
    }
}

template <class T> static void eval_jac(const Mechanism &m, const T *k, const T *y, T *jac) {
    for (u32 i = 0; i < m.nnz; ++i) jac[i] = (T)0.0;
    for (const Reaction &rx : m.reactions) {
        size_t r = &rx - m.reactions.data();
        for (u32 p = 0; p < rx.reactant_count; ++p) {
            T d = k[r];
            for (u32 q = 0; q < rx.reactant_count; ++q)
                if (q != p) d = d * y[rx.reactant[q]];
            for (u32 e = 0; e < rx.net_count; ++e) {
                u32 idx = rx.jac_index[p][e];
                jac[idx] = fmadd((T)(double)rx.net_coef[e], d, jac[idx]);
            }
        }
    }
}

// In place: a = -J -> L\U of (I ghinv - J); the diagonal keeps 1/U(i,i).
template <class T> static void factor(const Mechanism &m, T ghinv, T *a) {
    for (u32 i = 0; i < m.n(); ++i) {
        for (u32 d = m.pivot_begin[i]; d < m.pivot_begin[i + 1]; ++d) {
            const LuPivot &pv = m.pivots[d];
            T l = a[pv.ik] * a[pv.kk];
            a[pv.ik] = l;
            for (u32 s = pv.sub_begin; s < pv.sub_end; ++s) {
                const LuUpdate &u = m.updates[s];
                a[u.ij] = fnmadd(l, a[u.kj], a[u.ij]);
            }
        }
        u32 ii = m.diag[i];
        a[ii] = (T)1.0 / (a[ii] + ghinv);
    }
}

template <class T> static void solve(const Mechanism &m, const T *a, T *x) {
    const u32 n = m.n();
    for (u32 i = 0; i < n; ++i)
        for (u32 e = m.lower_begin[i]; e < m.lower_begin[i + 1]; ++e) x[i] = fnmadd(a[m.lower[e].index], x[m.lower[e].col], x[i]);
    for (u32 ii = n; ii-- > 0;) {
        for (u32 e = m.upper_begin[ii]; e < m.upper_begin[ii + 1]; ++e)
            x[ii] = fnmadd(a[m.upper[e].index], x[m.upper[e].col], x[ii]);
        x[ii] = x[ii] * a[m.diag[ii]];
    }
}

template <class T> struct Stats {
    T steps, rejects, pulses, failed;
};

// Per-cell scratch reused across calls (sized once per mechanism).
template <class T> struct Work {
    std::vector<T> lu, fcn, ytmp, yeval, kst;
    void size(const Mechanism &m) {
        lu.resize(m.nnz ? m.nnz : 1);
        fcn.resize(m.n());
        ytmp.resize(m.n());
        yeval.resize(m.n());
        kst.resize((size_t)4 * m.n());
    }
};

// kin_solver.h:189-313 for one scalar lane. Delta: y is an increment over base.
template <class T, bool Delta>
static void integrate(const Mechanism &m, const Method &me, const Control &ctl, const T *k, const T *src, T *y, T &t,
                      T t_end, T &h, Stats<T> &st, const T *base, Work<T> &w) {
    const u32 n = m.n();
    const T zero = (T)0.0, one = (T)1.0;
    const T h_min = (T)ctl.h_min, rtol = (T)ctl.rtol, atol = (T)ctl.atol;
    const T inv_n = (T)(1.0 / (double)n);
    T *lu = w.lu.data(), *fcn = w.fcn.data(), *ytmp = w.ytmp.data(), *yeval = w.yeval.data();
    T *K[4] = {w.kst.data(), w.kst.data() + n, w.kst.data() + 2 * n, w.kst.data() + 3 * n};

    bool active = t < t_end && !(st.failed > zero);
    bool reject_last = false, reject_more = false;
    h = h > zero ? h : (T)ctl.h_start;
    u32 iterations = 0;
    while (active) {
        if (++iterations > ctl.max_steps) {
            st.failed = one;
            break;
        }
        T remaining = t_end - t;
        T h_cap = remaining;
        if (ctl.h_max > 0.0) h_cap = vmin(h_cap, (T)ctl.h_max);
        T h_wanted = vmax(h, h_min);
        bool last = h_wanted >= remaining;
        T hs = last ? remaining : vmin(h_wanted, h_cap);

        const T *yfun = y;
        if (Delta) {
            for (u32 s = 0; s < n; ++s) yeval[s] = base[s] + y[s];
            yfun = yeval;
        }
        eval_fun(m, k, src, yfun, fcn);
        eval_neg_jac(m, k, yfun, lu);
        T ghinv = one / (hs * (T)me.gamma0);
        factor(m, ghinv, lu);
        T hinv = one / hs;

        for (u32 stg = 0; stg < me.stages; ++stg) {
            u32 packed = stg * (stg - 1) / 2;
            if (stg > 0 && me.new_f[stg]) {
                for (u32 s = 0; s < n; ++s) ytmp[s] = y[s];
                for (u32 j = 0; j < stg; ++j) {
                    double a = me.a[packed + j];
                    if (a == 0.0) continue;
                    T av = (T)a;
                    for (u32 s = 0; s < n; ++s) ytmp[s] = fmadd(av, K[j][s], ytmp[s]);
                }
                if (Delta) {
                    for (u32 s = 0; s < n; ++s) yeval[s] = base[s] + ytmp[s];
                    eval_fun(m, k, src, yeval, fcn);
                } else {
                    eval_fun(m, k, src, ytmp, fcn);
                }
            }
            for (u32 s = 0; s < n; ++s) K[stg][s] = fcn[s];
            for (u32 j = 0; j < stg; ++j) {
                double c = me.c[packed + j];
                if (c == 0.0) continue;
                T hc = (T)c * hinv;
                for (u32 s = 0; s < n; ++s) K[stg][s] = fmadd(hc, K[j][s], K[stg][s]);
            }
            solve(m, lu, K[stg]);
        }

        T err = zero;
        for (u32 s = 0; s < n; ++s) {
            T ynew = y[s], yerr = zero;
            for (u32 stg = 0; stg < me.stages; ++stg) {
                if (me.m[stg] != 0.0) ynew = fmadd((T)me.m[stg], K[stg][s], ynew);
                if (me.e[stg] != 0.0) yerr = fmadd((T)me.e[stg], K[stg][s], yerr);
            }
            T scale;
            if (Delta) scale = fmadd(rtol, vmax(vabs(base[s] + y[s]), vabs(base[s] + ynew)), atol);
            else scale = fmadd(rtol, vmax(vabs(y[s]), vabs(ynew)), atol);
            T q = yerr / scale;
            err = fmadd(q, q, err);
            ytmp[s] = ynew;
        }
        err = vsqrt(err * inv_n);
        if (!finite(err)) err = (T)1e10;

        T fac = step_factor(err, me.order);
        bool ok = err <= one || hs <= h_min;
        if (ctl.fixed_step) {
            ok = true;
            fac = one;
        }
        bool accept = ok, reject = !ok;
        if (accept) {
            for (u32 s = 0; s < n; ++s) {
                T ynew = ytmp[s];
                if (ctl.clamp_negative) ynew = Delta ? vmax(ynew, -base[s]) : vmax(ynew, zero);
                y[s] = ynew;
            }
            t = last ? t_end : t + hs;
        }
        T h_acc = hs * fac;
        h_acc = reject_last ? vmin(h_acc, hs) : h_acc;
        h_acc = (last && fac >= one) ? vmax(h_acc, h_wanted) : h_acc;
        T h_rej = reject_more ? hs * (T)0.1 : vmin(hs * fac, hs);
        if (ctl.fixed_step) {
            h_acc = h_wanted;
            h_rej = h_wanted;
        }
        h = accept ? h_acc : h_rej;
        reject_more = reject && reject_last;
        reject_last = reject;
        st.steps = st.steps + (accept ? one : zero);
        st.rejects = st.rejects + (reject ? one : zero);
        active = t < t_end && !(st.failed > zero);
    }
}

// kin_solver.h:322-347 for one scalar lane: segments between discharge pulses.
template <class T, bool Delta>
static void advance(const Mechanism &m, const Method &me, const Control &ctl, const T *k, const T *src, const T *pulse,
                    T period, T first_pulse, T pulse_count, T *y, T duration, T &h, Stats<T> &st, const T *base,
                    Work<T> &w) {
    const u32 n = m.n();
    const T zero = (T)0.0, one = (T)1.0;
    T t = zero, applied = zero;
    for (;;) {
        bool pending = applied < pulse_count;
        T next_pulse = fmadd(applied, period, first_pulse);
        T seg_end = pending ? vmin(next_pulse, duration) : duration;
        integrate<T, Delta>(m, me, ctl, k, src, y, t, seg_end, h, st, base, w);
        bool alive = !(st.failed > zero);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            for (u32 s = 0; s < n; ++s) y[s] = y[s] + pulse[s];
            applied = applied + one;
            st.pulses = st.pulses + one;
            h = (T)ctl.h_start;
        }
        bool done = (t >= duration && applied >= pulse_count) || !alive;
        if (done) break;
    }
}

// The DbdZones SoA block of one launch (src/sim/dbd_lanes.h:13-19 / gpu_api.h:30-37).
struct LaneArrays {
    double *y, *h, *steps, *rejects, *pulses, *failed;
    const double *k, *src, *pulse, *period, *pulse_first, *pulse_count;
    u32 padded;
};

// dbd_lanes.h:28-78 for one lane i: load (f64 storage, converted to T), advance, store.
template <class T, bool Delta>
static void advance_lane(const Mechanism &m, const Method &me, const Control &ctl, const LaneArrays &a, u32 i,
                         double duration, Work<T> &w, std::vector<T> &buf) {
    const u32 n = m.n(), R = m.R(), p = a.padded;
    buf.resize((size_t)4 * n + R);
    T *y = buf.data(), *src = y + n, *pls = src + n, *base = pls + n, *k = base + n;
    for (u32 s = 0; s < n; ++s) {
        if (Delta) {
            base[s] = (T)a.y[(size_t)s * p + i];
            y[s] = (T)0.0;
        } else {
            y[s] = (T)a.y[(size_t)s * p + i];
        }
        src[s] = (T)a.src[(size_t)s * p + i];
        pls[s] = (T)a.pulse[(size_t)s * p + i];
    }
    for (u32 r = 0; r < R; ++r) k[r] = (T)a.k[(size_t)r * p + i];
    T h = (T)a.h[i];
    T per = (T)a.period[i], first = (T)a.pulse_first[i], count = (T)a.pulse_count[i];
    Stats<T> st;
    st.steps = st.rejects = st.pulses = (T)0.0;
    st.failed = (T)a.failed[i];
    advance<T, Delta>(m, me, ctl, k, src, pls, per, first, count, y, (T)duration, h, st, Delta ? base : nullptr, w);
    for (u32 s = 0; s < n; ++s) {
        double *dst = a.y + (size_t)s * p + i;
        if (Delta) {
            *dst += (double)y[s];
            if (ctl.clamp_negative) *dst = *dst > 0.0 ? *dst : 0.0;
        } else {
            *dst = (double)y[s];
        }
    }
    a.h[i] = (double)h;
    a.failed[i] = (double)st.failed;
    a.steps[i] += (double)st.steps;
    a.rejects[i] += (double)st.rejects;
    a.pulses[i] += (double)st.pulses;
}

template <class T, bool Delta>
static void advance_range(const Mechanism *m, const Method *me, const Control *ctl, const LaneArrays *a, u32 begin,
                          u32 end, double duration) {
    Work<T> w;
    w.size(*m);
    std::vector<T> buf;
    for (u32 i = begin; i < end; ++i) advance_lane<T, Delta>(*m, *me, *ctl, *a, i, duration, w, buf);
}

// ---------------------------------------------------------------------------
// Model of this module's MIXED-precision attempt (not a reference algorithm:
// the reference has no mixed path), in the GPU kernel's operation order so
// the tests can compare the GPU's mixed kernel with it bit for bit:
//   RHS      f(y) once per step in double-float (hi + lo FP32 pairs); at the
//            other stage points Y = y + d, f(y) + df with df in FP32 from the
//            exact increment expansion (eval_fun_delta32)
//   -J, LU   FP32 at the FP32 rounding of the point
//   solve    FP32 LU solve, then `sweeps` refinement sweeps with the FP64
//            residual r = b - ghinv x - (-J) x over the Jacobian pattern
//   state, stage combination, error estimate, controller: FP64, the same
//            controller code as the FP64 lane above.

struct Df2 {
    float hi, lo;
};
static inline Df2 df_from(double d) {
    float h = (float)d;
    return Df2{h, (float)(d - (double)h)};
}
static inline double df_to(Df2 a) { return (double)a.hi + (double)a.lo; }
static inline Df2 df_mul(Df2 a, Df2 b) {
    float p = a.hi * b.hi;
    float e = std::fma(a.hi, b.hi, -p);
    e = std::fma(a.hi, b.lo, e);
    e = std::fma(a.lo, b.hi, e);
    float s = p + e;
    return Df2{s, e - (s - p)};
}
static inline Df2 df_add(Df2 a, Df2 b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e = e + a.lo;
    e = e + b.lo;
    float t = s + e;
    return Df2{t, e - (t - s)};
}
static inline Df2 df_scale(Df2 a, float c) { return Df2{a.hi * c, a.lo * c}; }

static void eval_fun_df(const Mechanism &m, const Df2 *k, const Df2 *src, const Df2 *y, Df2 *f) {
    for (u32 s = 0; s < m.n(); ++s) f[s] = src[s];
    for (u32 r = 0; r < m.R(); ++r) {
        const Reaction &rx = m.reactions[r];
        Df2 rate = k[r];
        for (u32 p = 0; p < rx.reactant_count; ++p) rate = df_mul(rate, y[rx.reactant[p]]);
        for (u32 e = 0; e < rx.net_count; ++e) {
            const int c = rx.net_coef[e];
            Df2 term = c == 1 ? rate
                       : (c == -1 || c == 2 || c == -2 || c == 4 || c == -4) ? df_scale(rate, (float)c)
                                                                              : df_mul(rate, Df2{(float)c, 0.0f});
            f[rx.net_species[e]] = df_add(f[rx.net_species[e]], term);
        }
    }
}

struct MixedWork {
    std::vector<float> a, js, k32, x32;
    std::vector<Df2> kd, sd, yd, fd;
    std::vector<double> ytmp, kst, b, r;
    void size(const Mechanism &m) {
        a.resize(m.nnz ? m.nnz : 1);
        js.resize(m.nnz ? m.nnz : 1);
        k32.resize(m.R() ? m.R() : 1);
        x32.resize(m.n());
        kd.resize(m.R() ? m.R() : 1);
        sd.resize(m.n()); yd.resize(m.n()); fd.resize(m.n());
        ytmp.resize(m.n()); kst.resize((size_t)4 * m.n()); b.resize(m.n()); r.resize(m.n());
    }
};

// r = b - ghinv x - (-J) x over each row's Jacobian-pattern entries, ascending column.
static void residual64(const Mechanism &m, const float *js, double ghinv, const double *b, const double *x, double *r) {
    const u32 n = m.n();
    for (u32 i = 0; i < n; ++i) {
        double acc = std::fma(-ghinv, x[i], b[i]);
        for (u32 j = 0; j < n; ++j)
            if (m.jac_pattern[(size_t)i * n + j]) acc = std::fma(-(double)js[m.slot[(size_t)i * n + j]], x[j], acc);
        r[i] = acc;
    }
}

// Stage RHS in increment form: f(y + d) = f(y) + df with df evaluated in FP32
// from the exact expansion prod(y_q + d_q) - prod(y_q) =
// sum_p (prod_{q<p} y_q) d_p (prod_{q>p} (y_q + d_q)), per reaction.
static void eval_fun_delta32(const Mechanism &m, const float *k, const float *y, const float *d, float *df) {
    for (u32 s = 0; s < m.n(); ++s) df[s] = 0.0f;
    for (u32 r = 0; r < m.R(); ++r) {
        const Reaction &rx = m.reactions[r];
        float rate = 0.0f;
        for (u32 p = 0; p < rx.reactant_count; ++p) {
            float term = k[r] * d[rx.reactant[p]];   // k first: keeps products of large densities in FP32 range
            for (u32 q = 0; q < p; ++q) term = term * y[rx.reactant[q]];
            for (u32 q = p + 1; q < rx.reactant_count; ++q) term = term * (y[rx.reactant[q]] + d[rx.reactant[q]]);
            rate = rate + term;
        }
        for (u32 e = 0; e < rx.net_count; ++e) df[rx.net_species[e]] = std::fma((float)rx.net_coef[e], rate, df[rx.net_species[e]]);
    }
}

static void integrate_mixed(const Mechanism &m, const Method &me, const Control &ctl, u32 sweeps, double *y, double &t,
                            double t_end, double &h, Stats<double> &st, MixedWork &w) {
    std::vector<double> f0(m.n());
    std::vector<float> d32(m.n()), df32(m.n());
    std::vector<double> fcur(m.n());
    const u32 n = m.n();
    const double zero = 0.0, one = 1.0, h_min = ctl.h_min, rtol = ctl.rtol, atol = ctl.atol;
    const double inv_n = 1.0 / (double)n;
    float *a = w.a.data(), *js = w.js.data(), *x32 = w.x32.data();
    double *ytmp = w.ytmp.data(), *b = w.b.data(), *rr = w.r.data();
    double *K[4] = {w.kst.data(), w.kst.data() + n, w.kst.data() + 2 * n, w.kst.data() + 3 * n};
    std::vector<float> yhi(n);

    auto rhs = [&](const double *yy) {
        for (u32 s = 0; s < n; ++s) w.yd[s] = df_from(yy[s]);
        eval_fun_df(m, w.kd.data(), w.sd.data(), w.yd.data(), w.fd.data());
    };

    bool active = t < t_end && !(st.failed > zero);
    bool reject_last = false, reject_more = false;
    h = h > zero ? h : ctl.h_start;
    u32 iterations = 0;
    while (active) {
        if (++iterations > ctl.max_steps) { st.failed = one; break; }
        double remaining = t_end - t;
        double h_cap = remaining;
        if (ctl.h_max > 0.0) h_cap = vmin(h_cap, ctl.h_max);
        double h_wanted = vmax(h, h_min);
        bool last = h_wanted >= remaining;
        double hs = last ? remaining : vmin(h_wanted, h_cap);

        rhs(y);
        for (u32 s = 0; s < n; ++s) f0[s] = df_to(w.fd[s]);
        for (u32 s = 0; s < n; ++s) fcur[s] = f0[s];
        for (u32 s = 0; s < n; ++s) yhi[s] = w.yd[s].hi;
        eval_neg_jac(m, w.k32.data(), yhi.data(), a);
        for (u32 i = 0; i < m.nnz; ++i) js[i] = a[i];
        double ghinv = one / (hs * me.gamma0);
        factor(m, (float)ghinv, a);
        double hinv = one / hs;

        for (u32 stg = 0; stg < me.stages; ++stg) {
            u32 packed = stg * (stg - 1) / 2;
            // stage RHS: f(y) from the step start when the stage point is y itself
            // (no nonzero a coefficient, e.g. Rodas3 stage 2), else f(y) + df with
            // df the FP32 increment form at d = Y - y
            bool moved = false;
            if (stg > 0 && me.new_f[stg]) {
                for (u32 s = 0; s < n; ++s) ytmp[s] = y[s];
                for (u32 j = 0; j < stg; ++j) {
                    double av = me.a[packed + j];
                    if (av == 0.0) continue;
                    moved = true;
                    for (u32 s = 0; s < n; ++s) ytmp[s] = std::fma(av, K[j][s], ytmp[s]);
                }
                if (moved) {
                    for (u32 s = 0; s < n; ++s) d32[s] = (float)(ytmp[s] - y[s]);
                    eval_fun_delta32(m, w.k32.data(), yhi.data(), d32.data(), df32.data());
                    for (u32 s = 0; s < n; ++s) fcur[s] = f0[s] + (double)df32[s];
                } else {
                    for (u32 s = 0; s < n; ++s) fcur[s] = f0[s];
                }
            }
            for (u32 s = 0; s < n; ++s) K[stg][s] = fcur[s];
            for (u32 j = 0; j < stg; ++j) {
                double c = me.c[packed + j];
                if (c == 0.0) continue;
                double hc = c * hinv;
                for (u32 s = 0; s < n; ++s) K[stg][s] = std::fma(hc, K[j][s], K[stg][s]);
            }
            double *x = K[stg];
            for (u32 s = 0; s < n; ++s) b[s] = x[s];
            for (u32 s = 0; s < n; ++s) x32[s] = (float)b[s];
            solve(m, a, x32);
            for (u32 s = 0; s < n; ++s) x[s] = (double)x32[s];
            for (u32 sw = 0; sw < sweeps; ++sw) {
                residual64(m, js, ghinv, b, x, rr);
                for (u32 s = 0; s < n; ++s) x32[s] = (float)rr[s];
                solve(m, a, x32);
                for (u32 s = 0; s < n; ++s) x[s] = x[s] + (double)x32[s];
            }
        }

        double err = zero;
        for (u32 s = 0; s < n; ++s) {
            double ynew = y[s], yerr = zero;
            for (u32 stg = 0; stg < me.stages; ++stg) {
                if (me.m[stg] != 0.0) ynew = std::fma(me.m[stg], K[stg][s], ynew);
                if (me.e[stg] != 0.0) yerr = std::fma(me.e[stg], K[stg][s], yerr);
            }
            double scale = std::fma(rtol, vmax(vabs(y[s]), vabs(ynew)), atol);
            double q = yerr / scale;
            err = std::fma(q, q, err);
            ytmp[s] = ynew;
        }
        err = vsqrt(err * inv_n);
        if (!finite(err)) err = 1e10;
        double fac = step_factor(err, me.order);
        bool ok = err <= one || hs <= h_min;
        if (ctl.fixed_step) { ok = true; fac = one; }
        if (ok) {
            for (u32 s = 0; s < n; ++s) {
                double ynew = ytmp[s];
                if (ctl.clamp_negative) ynew = vmax(ynew, zero);
                y[s] = ynew;
            }
            t = last ? t_end : t + hs;
        }
        double h_acc = hs * fac;
        h_acc = reject_last ? vmin(h_acc, hs) : h_acc;
        h_acc = (last && fac >= one) ? vmax(h_acc, h_wanted) : h_acc;
        double h_rej = reject_more ? hs * 0.1 : vmin(hs * fac, hs);
        if (ctl.fixed_step) { h_acc = h_wanted; h_rej = h_wanted; }
        h = ok ? h_acc : h_rej;
        reject_more = !ok && reject_last;
        reject_last = !ok;
        st.steps = st.steps + (ok ? one : zero);
        st.rejects = st.rejects + (ok ? zero : one);
        active = t < t_end && !(st.failed > zero);
    }
}

// Model of the module's mixed path with DOUBLE-FLOAT STATE (mixed variant 1),
// in the GPU kernel's operation order (LaneDf in the module): y and f(y) are
// hi + lo FP32 pairs; -J, LU, stage vectors K and solves FP32; the stage
// right-hand side f(y) [+ df] + sum_j (c_j / h) K_j accumulated in
// double-float and rounded once; y_new = y + sum m K in double-float; the
// error norm in FP32; only t and h stay FP64.
static inline Df2 df_add_f(Df2 a, float b) {
    float s = a.hi + b;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b - bb);
    e = e + a.lo;
    float t = s + e;
    return Df2{t, e - (t - s)};
}
static inline Df2 df_prod_f(float a, float b) {
    float p = a * b;
    return Df2{p, std::fma(a, b, -p)};
}

static void integrate_mixed_df(const Mechanism &m, const Method &me, const Control &ctl, Df2 *y, double &t, double t_end,
                               double &h, Stats<double> &st, MixedWork &w) {
    const u32 n = m.n();
    std::vector<float> yhi(n), d32(n), df32(n), nhi(n), nlo(n), kst((size_t)4 * n);
    float *K[4] = {kst.data(), kst.data() + n, kst.data() + 2 * n, kst.data() + 3 * n};
    float *a = w.a.data();
    const float rtol = (float)ctl.rtol, atol = (float)ctl.atol, inv_n = 1.0f / (float)n;
    bool active = t < t_end && !(st.failed > 0.0);
    bool reject_last = false, reject_more = false;
    h = h > 0.0 ? h : ctl.h_start;
    u32 iterations = 0;
    while (active) {
        if (++iterations > ctl.max_steps) { st.failed = 1.0; break; }
        double remaining = t_end - t;
        double h_cap = remaining;
        if (ctl.h_max > 0.0) h_cap = vmin(h_cap, ctl.h_max);
        double h_wanted = vmax(h, ctl.h_min);
        bool last = h_wanted >= remaining;
        double hs = last ? remaining : vmin(h_wanted, h_cap);
        const float hs32 = (float)hs;

        eval_fun_df(m, w.kd.data(), w.sd.data(), y, w.fd.data());
        for (u32 s = 0; s < n; ++s) yhi[s] = y[s].hi;
        eval_neg_jac(m, w.k32.data(), yhi.data(), a);
        factor(m, 1.0f / (hs32 * (float)me.gamma0), a);
        const float hinv = 1.0f / hs32;

        bool last_moved = false;
        for (u32 stg = 0; stg < me.stages; ++stg) {
            u32 packed = stg * (stg - 1) / 2;
            if (stg > 0 && me.new_f[stg]) {
                bool moved = false;
                for (u32 s = 0; s < n; ++s) d32[s] = 0.0f;
                for (u32 j = 0; j < stg; ++j) {
                    float av = (float)me.a[packed + j];
                    if (av == 0.0f) continue;
                    moved = true;
                    for (u32 s = 0; s < n; ++s) d32[s] = std::fma(av, K[j][s], d32[s]);
                }
                if (moved) eval_fun_delta32(m, w.k32.data(), yhi.data(), d32.data(), df32.data());
                last_moved = moved;
            }
            for (u32 s = 0; s < n; ++s) {
                Df2 b = w.fd[s];
                if (last_moved) b = df_add_f(b, df32[s]);
                for (u32 j = 0; j < stg; ++j) {
                    float c = (float)me.c[packed + j];
                    if (c == 0.0f) continue;
                    b = df_add(b, df_prod_f(c * hinv, K[j][s]));
                }
                K[stg][s] = b.hi + b.lo;
            }
            solve(m, a, K[stg]);
        }

        float err = 0.0f;
        for (u32 s = 0; s < n; ++s) {
            Df2 yn = y[s];
            float yerr = 0.0f;
            for (u32 stg = 0; stg < me.stages; ++stg) {
                float mc = (float)me.m[stg], ec = (float)me.e[stg];
                if (mc != 0.0f) yn = df_add(yn, df_prod_f(mc, K[stg][s]));
                if (ec != 0.0f) yerr = std::fma(ec, K[stg][s], yerr);
            }
            float scale = std::fma(rtol, std::fmax(std::fabs(y[s].hi), std::fabs(yn.hi)), atol);
            float q = yerr / scale;
            err = std::fma(q, q, err);
            nhi[s] = yn.hi;
            nlo[s] = yn.lo;
        }
        err = vsqrt(err * inv_n);
        if (!finite(err)) err = 1e10f;
        float fac32 = step_factor(err, me.order);
        bool ok = err <= 1.0f || hs <= ctl.h_min;
        if (ctl.fixed_step) { ok = true; fac32 = 1.0f; }
        if (ok) {
            for (u32 s = 0; s < n; ++s) {
                float hi = nhi[s], lo = nlo[s];
                if (ctl.clamp_negative && (hi < 0.0f || (hi == 0.0f && lo < 0.0f))) { hi = 0.0f; lo = 0.0f; }
                y[s] = Df2{hi, lo};
            }
            t = last ? t_end : t + hs;
        }
        const double fac = (double)fac32;
        double h_acc = hs * fac;
        h_acc = reject_last ? vmin(h_acc, hs) : h_acc;
        h_acc = (last && fac >= 1.0) ? vmax(h_acc, h_wanted) : h_acc;
        double h_rej = reject_more ? hs * 0.1 : vmin(hs * fac, hs);
        if (ctl.fixed_step) { h_acc = h_wanted; h_rej = h_wanted; }
        h = ok ? h_acc : h_rej;
        reject_more = !ok && reject_last;
        reject_last = !ok;
        st.steps = st.steps + (ok ? 1.0 : 0.0);
        st.rejects = st.rejects + (ok ? 0.0 : 1.0);
        active = t < t_end && !(st.failed > 0.0);
    }
}

static void advance_mixed_df_lane(const Mechanism &m, const Method &me, const Control &ctl, const LaneArrays &a, u32 i,
                                  double duration, MixedWork &w, std::vector<Df2> &y) {
    const u32 n = m.n(), R = m.R(), p = a.padded;
    for (u32 s = 0; s < n; ++s) {
        y[s] = df_from(a.y[(size_t)s * p + i]);
        w.sd[s] = df_from(a.src[(size_t)s * p + i]);
    }
    for (u32 r = 0; r < R; ++r) {
        w.kd[r] = df_from(a.k[(size_t)r * p + i]);
        w.k32[r] = w.kd[r].hi;
    }
    double h = a.h[i], per = a.period[i], first = a.pulse_first[i], count = a.pulse_count[i];
    Stats<double> st = {0.0, 0.0, 0.0, a.failed[i]};
    double t = 0.0, applied = 0.0;
    for (;;) {
        bool pending = applied < count;
        double next_pulse = std::fma(applied, per, first);
        double seg_end = pending ? vmin(next_pulse, duration) : duration;
        integrate_mixed_df(m, me, ctl, y.data(), t, seg_end, h, st, w);
        bool alive = !(st.failed > 0.0);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            for (u32 s = 0; s < n; ++s) y[s] = df_add(y[s], df_from(a.pulse[(size_t)s * p + i]));
            applied = applied + 1.0;
            st.pulses = st.pulses + 1.0;
            h = ctl.h_start;
        }
        if ((t >= duration && applied >= count) || !alive) break;
    }
    for (u32 s = 0; s < n; ++s) a.y[(size_t)s * p + i] = df_to(y[s]);
    a.h[i] = h;
    a.failed[i] = st.failed;
    a.steps[i] += st.steps;
    a.rejects[i] += st.rejects;
    a.pulses[i] += st.pulses;
}

// kin_advance for the mixed model: segments between pulses, as advance() above.
static void advance_mixed_lane(const Mechanism &m, const Method &me, const Control &ctl, u32 sweeps, const LaneArrays &a,
                               u32 i, double duration, MixedWork &w, std::vector<double> &y) {
    const u32 n = m.n(), R = m.R(), p = a.padded;
    for (u32 s = 0; s < n; ++s) {
        y[s] = a.y[(size_t)s * p + i];
        w.sd[s] = df_from(a.src[(size_t)s * p + i]);
    }
    for (u32 r = 0; r < R; ++r) {
        w.kd[r] = df_from(a.k[(size_t)r * p + i]);
        w.k32[r] = w.kd[r].hi;
    }
    double h = a.h[i], per = a.period[i], first = a.pulse_first[i], count = a.pulse_count[i];
    Stats<double> st = {0.0, 0.0, 0.0, a.failed[i]};
    double t = 0.0, applied = 0.0;
    for (;;) {
        bool pending = applied < count;
        double next_pulse = std::fma(applied, per, first);
        double seg_end = pending ? vmin(next_pulse, duration) : duration;
        integrate_mixed(m, me, ctl, sweeps, y.data(), t, seg_end, h, st, w);
        bool alive = !(st.failed > 0.0);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            for (u32 s = 0; s < n; ++s) y[s] = y[s] + a.pulse[(size_t)s * p + i];
            applied = applied + 1.0;
            st.pulses = st.pulses + 1.0;
            h = ctl.h_start;
        }
        if ((t >= duration && applied >= count) || !alive) break;
    }
    for (u32 s = 0; s < n; ++s) a.y[(size_t)s * p + i] = y[s];
    a.h[i] = h;
    a.failed[i] = st.failed;
    a.steps[i] += st.steps;
    a.rejects[i] += st.rejects;
    a.pulses[i] += st.pulses;
}

// Model of the module's mixed path with DOUBLE-FLOAT STATE AND REFINED STAGES
// (mixed variant 2), in the GPU kernel's operation order: every per-species
// quantity -- the state y, f at each stage point, the stage right-hand sides,
// the stage vectors K, y_new and the error norm -- is a double-float (hi + lo
// FP32 pair, ~48-bit significand) on the FP32 pipe; -J, the LU of W and the
// triangular solves are FP32 and serve as the preconditioner of one
// refinement sweep per stage, whose residual r = b - ghinv x + J x is
// evaluated in double-float with J x formed reaction by reaction at y (no
// stored Jacobian); only t, h and the per-step scalars are FP64.
static inline Df2 df_mul_f(Df2 a, float b) {   // double-float times float
    float p = a.hi * b;
    float e = std::fma(a.hi, b, -p);
    e = std::fma(a.lo, b, e);
    float s = p + e;
    return Df2{s, e - (s - p)};
}
static inline Df2 df_neg(Df2 a) { return Df2{-a.hi, -a.lo}; }
static inline Df2 df_abs(Df2 a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? df_neg(a) : a; }
static inline bool df_less(Df2 a, Df2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
static inline Df2 df_two_sum(float a, float b) {   // exact a + b as a normalised pair
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return Df2{s, e};
}
// times a small integer coefficient: exact for +-1, +-2, +-4, else a double-float product
static inline Df2 df_times_int(Df2 a, int c) {
    if (c == 1) return a;
    if (c == -1 || c == 2 || c == -2 || c == 4 || c == -4) return df_scale(a, (float)c);
    return df_mul(a, Df2{(float)c, 0.0f});
}
static inline Df2 df_times_coef(Df2 a, double c) {   // method coefficients a_ij, m_i, e_i
    if (c == 1.0) return a;
    if (c == -1.0 || c == 2.0 || c == -2.0 || c == 4.0 || c == -4.0 || c == 0.5 || c == -0.5) return df_scale(a, (float)c);
    return df_mul(a, df_from(c));
}

// Lazily normalised double-float arithmetic for the refined variant's sums: df_acc adds a
// pair to an accumulator whose hi holds the rounded running sum and whose lo collects the
// low parts and every two-sum rounding error (8 operations instead of df_add's 11); the
// products skip their final renormalisation (|lo| stays within a few ulp of hi); a sum is
// normalised once, with a two-sum, when it is complete.
static inline Df2 df_acc(Df2 a, Df2 t) {
    float s = a.hi + t.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (t.hi - bb);
    return Df2{s, a.lo + (t.lo + e)};
}
static inline Df2 df_mul_u(Df2 a, Df2 b) {
    float p = a.hi * b.hi;
    float e = std::fma(a.hi, b.hi, -p);
    e = std::fma(a.hi, b.lo, e);
    e = std::fma(a.lo, b.hi, e);
    return Df2{p, e};
}
static inline Df2 df_mul_fu(Df2 a, float b) {
    float p = a.hi * b;
    float e = std::fma(a.hi, b, -p);
    e = std::fma(a.lo, b, e);
    return Df2{p, e};
}
static inline Df2 df_norm(Df2 a) { return df_two_sum(a.hi, a.lo); }
static inline Df2 df_times_coef_u(Df2 a, double c) {   // method coefficients, lazily normalised product
    if (c == 1.0) return a;
    if (c == -1.0 || c == 2.0 || c == -2.0 || c == 4.0 || c == -4.0 || c == 0.5 || c == -0.5) return df_scale(a, (float)c);
    return df_mul_u(a, df_from(c));
}
static inline Df2 df_times_int_u(Df2 a, int c) {
    if (c == 1) return a;
    if (c == -1 || c == 2 || c == -2 || c == 4 || c == -4) return df_scale(a, (float)c);
    return df_mul_u(a, Df2{(float)c, 0.0f});
}

// f(y) in lazily normalised double-float: the terms of eval_fun_df in the same order.
static void eval_fun_dfl(const Mechanism &m, const Df2 *k, const Df2 *src, const Df2 *y, Df2 *f) {
    for (u32 s = 0; s < m.n(); ++s) f[s] = src[s];
    for (u32 r = 0; r < m.R(); ++r) {
        const Reaction &rx = m.reactions[r];
        Df2 rate = k[r];
        for (u32 p = 0; p < rx.reactant_count; ++p) rate = df_mul_u(rate, y[rx.reactant[p]]);
        for (u32 e = 0; e < rx.net_count; ++e) f[rx.net_species[e]] = df_acc(f[rx.net_species[e]], df_times_int_u(rate, rx.net_coef[e]));
    }
    for (u32 s = 0; s < m.n(); ++s) f[s] = df_norm(f[s]);
}

// The refinement residual, whole: r = b - ghinv x + J(y) x, accumulated per species from
// b - ghinv x through the terms of J(y) x in reaction order: d rate_r = sum_p k_r (prod_{q != p}
// y[q]) x[q_p], each term multiplied out from k_r (which keeps products of large number
// densities in FP32 range), then r_s += net_{r,s} d rate_r (no intermediate J x vector);
// returns the FP32 rounding of each r_s as the right-hand side of the correction solve.
static void eval_residual_df(const Mechanism &m, const Df2 *k, const Df2 *y, const float *x, const Df2 *b, Df2 gd, float *x2) {
    const u32 n = m.n();
    std::vector<Df2> acc(n);
    for (u32 s = 0; s < n; ++s) acc[s] = df_acc(b[s], df_neg(df_mul_fu(gd, x[s])));
    for (u32 r = 0; r < m.R(); ++r) {
        const Reaction &rx = m.reactions[r];
        Df2 drate{0.0f, 0.0f};
        for (u32 p = 0; p < rx.reactant_count; ++p) {
            Df2 t = k[r];
            for (u32 q = 0; q < rx.reactant_count; ++q)
                if (q != p) t = df_mul_u(t, y[rx.reactant[q]]);
            t = df_mul_fu(t, x[rx.reactant[p]]);
            drate = p == 0 ? t : df_acc(drate, t);
        }
        for (u32 e = 0; e < rx.net_count; ++e) acc[rx.net_species[e]] = df_acc(acc[rx.net_species[e]], df_times_int_u(drate, rx.net_coef[e]));
    }
    for (u32 s = 0; s < n; ++s) x2[s] = acc[s].hi + acc[s].lo;
}

static void integrate_mixed_ir(const Mechanism &m, const Method &me, const Control &ctl, Df2 *y, double &t, double t_end,
                               double &h, Stats<double> &st, MixedWork &w) {
    const u32 n = m.n();
    std::vector<float> yhi(n), x(n), x2(n);
    std::vector<Df2> Y(n), fy(n), b(n), kd((size_t)4 * n), ynew(n);
    Df2 *K[4] = {kd.data(), kd.data() + n, kd.data() + 2 * n, kd.data() + 3 * n};
    float *a = w.a.data();
    const Df2 rtol = df_from(ctl.rtol), atol = df_from(ctl.atol);
    const double inv_n = 1.0 / (double)n;
    bool active = t < t_end && !(st.failed > 0.0);
    bool reject_last = false, reject_more = false;
    h = h > 0.0 ? h : ctl.h_start;
    u32 iterations = 0;
    while (active) {
        if (++iterations > ctl.max_steps) { st.failed = 1.0; break; }
        double remaining = t_end - t;
        double h_cap = remaining;
        if (ctl.h_max > 0.0) h_cap = vmin(h_cap, ctl.h_max);
        double h_wanted = vmax(h, ctl.h_min);
        bool last = h_wanted >= remaining;
        double hs = last ? remaining : vmin(h_wanted, h_cap);
        const double ghinv = 1.0 / (hs * me.gamma0), hinv = 1.0 / hs;
        const Df2 gd = df_from(ghinv), hd = df_from(hinv);

        eval_fun_dfl(m, w.kd.data(), w.sd.data(), y, fy.data());
        for (u32 s = 0; s < n; ++s) yhi[s] = y[s].hi;
        eval_neg_jac(m, w.k32.data(), yhi.data(), a);
        factor(m, (float)ghinv, a);

        for (u32 stg = 0; stg < me.stages; ++stg) {
            u32 packed = stg * (stg - 1) / 2;
            if (stg > 0 && me.new_f[stg]) {   // stage point Y = y + sum_j a_j K_j; f(y) reused when it is y
                bool moved = false;
                for (u32 s = 0; s < n; ++s) Y[s] = y[s];
                for (u32 j = 0; j < stg; ++j) {
                    double av = me.a[packed + j];
                    if (av == 0.0) continue;
                    moved = true;
                    for (u32 s = 0; s < n; ++s) Y[s] = df_acc(Y[s], df_times_coef_u(K[j][s], av));
                }
                if (moved) {
                    for (u32 s = 0; s < n; ++s) Y[s] = df_norm(Y[s]);
                    eval_fun_dfl(m, w.kd.data(), w.sd.data(), Y.data(), fy.data());
                } else {
                    eval_fun_dfl(m, w.kd.data(), w.sd.data(), y, fy.data());
                }
            }
            for (u32 s = 0; s < n; ++s) b[s] = fy[s];
            for (u32 j = 0; j < stg; ++j) {
                double c = me.c[packed + j];
                if (c == 0.0) continue;
                const Df2 ch = df_mul(df_from(c), hd);   // c / h in double-float
                for (u32 s = 0; s < n; ++s) b[s] = df_acc(b[s], df_mul_u(ch, K[j][s]));
            }
            for (u32 s = 0; s < n; ++s) b[s] = df_norm(b[s]);
            for (u32 s = 0; s < n; ++s) x[s] = b[s].hi;
            solve(m, a, x.data());
            // one refinement sweep: r = b - ghinv x + J x in double-float, x += W32^-1 r
            eval_residual_df(m, w.kd.data(), y, x.data(), b.data(), gd, x2.data());
            solve(m, a, x2.data());
            for (u32 s = 0; s < n; ++s) K[stg][s] = df_two_sum(x[s], x2[s]);
        }

        Df2 err2{0.0f, 0.0f};
        for (u32 s = 0; s < n; ++s) {
            Df2 yn = y[s], ye{0.0f, 0.0f};
            bool first_e = true;
            for (u32 stg = 0; stg < me.stages; ++stg) {
                if (me.m[stg] != 0.0) yn = df_acc(yn, df_times_coef_u(K[stg][s], me.m[stg]));
                if (me.e[stg] != 0.0) {
                    ye = first_e ? df_times_coef_u(K[stg][s], me.e[stg]) : df_acc(ye, df_times_coef_u(K[stg][s], me.e[stg]));
                    first_e = false;
                }
            }
            yn = df_norm(yn);
            ye = df_norm(ye);
            Df2 ay = df_abs(y[s]), an = df_abs(yn);
            const Df2 scale = df_add(df_mul(rtol, df_less(ay, an) ? an : ay), atol);
            const float inv = 1.0f / scale.hi;
            const float q1 = ye.hi * inv;
            const float q2 = df_add(ye, df_neg(df_mul_f(scale, q1))).hi * inv;
            const Df2 q = df_two_sum(q1, q2);
            err2 = df_add(err2, df_mul(q, q));
            ynew[s] = yn;
        }
        double err = std::sqrt(df_to(err2) * inv_n);
        if (!finite(err)) err = 1e10;
        double fac = step_factor_mixed(err, me.order);
        bool ok = err <= 1.0 || hs <= ctl.h_min;
        if (ctl.fixed_step) { ok = true; fac = 1.0; }
        if (ok) {
            for (u32 s = 0; s < n; ++s) {
                Df2 v = ynew[s];
                if (ctl.clamp_negative && (v.hi < 0.0f || (v.hi == 0.0f && v.lo < 0.0f))) v = Df2{0.0f, 0.0f};
                y[s] = v;
            }
            t = last ? t_end : t + hs;
        }
        double h_acc = hs * fac;
        h_acc = reject_last ? vmin(h_acc, hs) : h_acc;
        h_acc = (last && fac >= 1.0) ? vmax(h_acc, h_wanted) : h_acc;
        double h_rej = reject_more ? hs * 0.1 : vmin(hs * fac, hs);
        if (ctl.fixed_step) { h_acc = h_wanted; h_rej = h_wanted; }
        h = ok ? h_acc : h_rej;
        reject_more = !ok && reject_last;
        reject_last = !ok;
        st.steps = st.steps + (ok ? 1.0 : 0.0);
        st.rejects = st.rejects + (ok ? 0.0 : 1.0);
        active = t < t_end && !(st.failed > 0.0);
    }
}

static void advance_mixed_ir_lane(const Mechanism &m, const Method &me, const Control &ctl, const LaneArrays &a, u32 i,
                                  double duration, MixedWork &w, std::vector<Df2> &y) {
    const u32 n = m.n(), R = m.R(), p = a.padded;
    for (u32 s = 0; s < n; ++s) {
        y[s] = df_from(a.y[(size_t)s * p + i]);
        w.sd[s] = df_from(a.src[(size_t)s * p + i]);
    }
    for (u32 r = 0; r < R; ++r) {
        w.kd[r] = df_from(a.k[(size_t)r * p + i]);
        w.k32[r] = w.kd[r].hi;
    }
    double h = a.h[i], per = a.period[i], first = a.pulse_first[i], count = a.pulse_count[i];
    Stats<double> st = {0.0, 0.0, 0.0, a.failed[i]};
    double t = 0.0, applied = 0.0;
    for (;;) {
        bool pending = applied < count;
        double next_pulse = std::fma(applied, per, first);
        double seg_end = pending ? vmin(next_pulse, duration) : duration;
        integrate_mixed_ir(m, me, ctl, y.data(), t, seg_end, h, st, w);
        bool alive = !(st.failed > 0.0);
        bool hit = pending && alive && t >= seg_end;
        if (hit) {
            for (u32 s = 0; s < n; ++s) y[s] = df_add(y[s], df_from(a.pulse[(size_t)s * p + i]));
            applied = applied + 1.0;
            st.pulses = st.pulses + 1.0;
            h = ctl.h_start;
        }
        if ((t >= duration && applied >= count) || !alive) break;
    }
    for (u32 s = 0; s < n; ++s) a.y[(size_t)s * p + i] = df_to(y[s]);
    a.h[i] = h;
    a.failed[i] = st.failed;
    a.steps[i] += st.steps;
    a.rejects[i] += st.rejects;
    a.pulses[i] += st.pulses;
}

static void advance_mixed_range(const Mechanism *m, const Method *me, const Control *ctl, u32 sweeps, u32 variant,
                                const LaneArrays *a, u32 begin, u32 end, double duration) {
    MixedWork w;
    w.size(*m);
    std::vector<double> y(m->n());
    std::vector<Df2> yd(m->n());
    for (u32 i = begin; i < end; ++i) {
        if (variant == 2) advance_mixed_ir_lane(*m, *me, *ctl, *a, i, duration, w, yd);
        else if (variant == 1) advance_mixed_df_lane(*m, *me, *ctl, *a, i, duration, w, yd);
        else advance_mixed_lane(*m, *me, *ctl, sweeps, *a, i, duration, w, y);
    }
}

// ---------------------------------------------------------------------------
// Discharge source (air_mech.cpp:184-276): per-second (averaged) or per-pulse
// species change for energy_J_cm3 deposited into gas y at temperature T.

struct AirIdx { u32 O, O3, N, NO, NO2, NO3, N2O5, N2O, HNO2, HNO3, OH, HO2, H2O2, H, N2, O2, H2O; };
static AirIdx air_index() { return AirIdx{0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16}; }

struct Channel { double k; u32 partner; };

static void branch(const Channel *ch, u32 count, const double *y, double amount, double *share) {
    double sum = 0.0;
    u32 big = 0;
    for (u32 c = 0; c < count; ++c) {
        share[c] = ch[c].k * y[ch[c].partner];
        if (share[c] > share[big]) big = c;
        sum += share[c];
    }
    if (sum <= 0.0) {
        for (u32 c = 0; c < count; ++c) share[c] = c == big ? 1.0 : 0.0;
        return;
    }
    double moved = 0.0;
    for (u32 c = 0; c < count; ++c) {
        share[c] /= sum;
        double cap = amount > 0.0 ? 0.5 * y[ch[c].partner] / amount : 1.0;
        if (c != big && share[c] > cap) {
            moved += share[c] - cap;
            share[c] = cap;
        }
    }
    share[big] += moved;
}

// G-values per 100 eV of the default (non-Boltzmann) source model, air_mech.cpp:164-175.
static void source_delta(const double *y, u32 n, double energy_J_cm3, double T_K, double *delta) {
    const AirIdx sp = air_index();
    const double g_O2_diss = 1.5, f_O1D = 0.5, g_N2A = 1.5, g_N2_diss = 0.4, g_OH = 0.3;
    for (u32 s = 0; s < n; ++s) delta[s] = 0.0;
    double total = 0.0;
    for (u32 s = 0; s < n; ++s) total += y[s];
    if (total <= 0.0 || energy_J_cm3 <= 0.0) return;
    double hundreds_eV = energy_J_cm3 * 6.241509074e18 * 0.01;
    double dO2 = g_O2_diss * (y[sp.O2] / total / 0.21) * hundreds_eV;
    double dA = g_N2A * (y[sp.N2] / total / 0.78) * hundreds_eV;
    double dN2 = g_N2_diss * (y[sp.N2] / total / 0.78) * hundreds_eV;
    double dOH = g_OH * (y[sp.H2O] / total / 0.02) * hundreds_eV;
    double d1D = f_O1D * dO2;
    delta[sp.O2] -= dO2;
    delta[sp.O] += 2.0 * dO2 - d1D;
    delta[sp.N2] -= dA + dN2;
    delta[sp.N] += dN2;
    delta[sp.OH] += dOH;
    delta[sp.H] += dOH;
    delta[sp.H2O] -= dOH;
    double t3 = T_K / 300.0;
    double k_o2 = pow(t3, 0.55);
    double f[10];
    const Channel a_ch[] = {
        {2.5e-12 * k_o2, sp.O2}, {1.3e-12 * k_o2, sp.O2}, {7.8e-14 * k_o2, sp.O2}, {7.0e-12, sp.O},   {7.0e-11, sp.NO},
        {1.0e-12, sp.NO2},       {8.0e-11, sp.N2O},       {5.0e-14, sp.H2O},       {3.0e-16, sp.N2},
    };
    branch(a_ch, 9, y, dA, f);
    delta[sp.N2] += dA * (f[0] + f[1] + f[4] + f[5] + f[6] + f[7] + f[8]);
    delta[sp.O2] -= dA * (f[0] + f[2]);
    delta[sp.O] += dA * (2.0 * f[0] + f[2] + f[5]);
    delta[sp.N2O] += dA * (f[2] - f[6]);
    delta[sp.O] -= dA * f[3];
    delta[sp.NO] += dA * (f[3] + f[5] + f[6]);
    double n2d = dN2 + dA * f[3];
    delta[sp.NO2] -= dA * f[5];
    delta[sp.N] += dA * f[6];
    delta[sp.H2O] -= dA * f[7];
    delta[sp.H] += dA * f[7];
    delta[sp.OH] += dA * f[7];
    const Channel n_ch[] = {{5.2e-12, sp.O2}, {1.7e-14, sp.N2}, {6.9e-13, sp.O}, {6.0e-11, sp.NO}, {2.2e-12, sp.N2O}};
    branch(n_ch, 5, y, n2d, f);
    delta[sp.O2] -= n2d * f[0];
    delta[sp.NO] += n2d * (f[0] - f[3] + f[4]);
    delta[sp.O] += n2d * (f[0] + f[3]);
    delta[sp.N] += n2d * (f[1] + f[2]);
    delta[sp.N2] += n2d * (f[3] + f[4]);
    delta[sp.N2O] -= n2d * f[4];
    const Channel o_ch[] = {
        {2.15e-11 * exp(110.0 / T_K), sp.N2}, {3.3e-11 * exp(55.0 / T_K), sp.O2},   {1.63e-10 * exp(60.0 / T_K), sp.H2O},
        {7.26e-11 * exp(20.0 / T_K), sp.N2O}, {4.63e-11 * exp(20.0 / T_K), sp.N2O}, {2.4e-10, sp.O3},
    };
    branch(o_ch, 6, y, d1D, f);
    delta[sp.O] += d1D * (f[0] + f[1]);
    delta[sp.O3] -= d1D * f[5];
    delta[sp.O2] += d1D * f[5] * 1.5;
    delta[sp.O] += d1D * f[5];
    delta[sp.H2O] -= d1D * f[2];
    delta[sp.OH] += d1D * f[2] * 2.0;
    delta[sp.N2O] -= d1D * (f[3] + f[4]);
    delta[sp.NO] += d1D * f[3] * 2.0;
    delta[sp.N2] += d1D * f[4];
    delta[sp.O2] += d1D * f[4];
}

}   // namespace oracle

// ===========================================================================
// C ABI for ctypes (tests and the CPU-baseline leg of bench.py).

using namespace oracle;

extern "C" {

void *or_mech_new(void) { return new Mechanism(); }
void *or_mech_new_air(void) {
    Mechanism *m = new Mechanism();
    define_air(m);
    finalize(m);
    return m;
}
void or_mech_free(void *h) { delete (Mechanism *)h; }
u32 or_add_species(void *h, const char *name, s32 abstract_species) { return add_species((Mechanism *)h, name, abstract_species != 0); }
// kind 0 Arrhenius(A,n,E), 1 third body(A,n,E), 2 Troe(A,n,A_inf,n_inf,fc), 3 eq-reverse(ref, keq_A, keq_B)
u32 or_add_reaction(void *h, const char *equation, s32 kind, const double *p, s32 ref) {
    RateLaw l = {};
    if (kind == kArrhenius) l = law_arr(p[0], p[1], p[2]);
    else if (kind == kThirdBody) l = law_m(p[0], p[1], p[2]);
    else if (kind == kTroe) l = law_troe(p[0], p[1], p[2], p[3], p[4]);
    else l = law_eq_reverse((u32)ref, p[0], p[1]);
    return add_reaction((Mechanism *)h, equation, l);
}
void or_finalize(void *h) { finalize((Mechanism *)h); }
const char *or_error(void *h) { return ((Mechanism *)h)->failed ? ((Mechanism *)h)->error.c_str() : ""; }
// counts[0..7] = n, R, nnz, pivots, updates, lower, upper, failed
void or_counts(void *h, u64 *counts) {
    Mechanism *m = (Mechanism *)h;
    counts[0] = m->n(); counts[1] = m->R(); counts[2] = m->nnz; counts[3] = m->pivots.size();
    counts[4] = m->updates.size(); counts[5] = m->lower.size(); counts[6] = m->upper.size(); counts[7] = m->failed;
}
// Reference-layout KinMech bytes (30,044) and their FNV-1a; returns 0 if it does not fit.
s32 or_export_kinmech(void *h, void *out, u64 *signature) {
    RefKinMech *km = (RefKinMech *)out;
    if (!export_ref_layout((Mechanism *)h, km)) return 0;
    if (signature) *signature = fnv1a(km, sizeof(RefKinMech));
    return 1;
}
// Pattern after fill (n*n bytes), elimination lists and solve lists, for table-level comparison.
void or_pattern(void *h, u8 *out) {
    Mechanism *m = (Mechanism *)h;
    memcpy(out, m->pattern.data(), m->pattern.size());
}
void or_lu_ops(void *h, u32 *pivots4, u32 *updates2) {
    Mechanism *m = (Mechanism *)h;
    for (size_t d = 0; d < m->pivots.size(); ++d) {
        pivots4[4 * d] = m->pivots[d].ik; pivots4[4 * d + 1] = m->pivots[d].kk;
        pivots4[4 * d + 2] = m->pivots[d].sub_begin; pivots4[4 * d + 3] = m->pivots[d].sub_end;
    }
    for (size_t s = 0; s < m->updates.size(); ++s) { updates2[2 * s] = m->updates[s].ij; updates2[2 * s + 1] = m->updates[s].kj; }
}
void or_rate_constants(void *h, double T, double M, double *k) { rate_constants((Mechanism *)h, T, M, k); }

// Rate constants of `cells` cells into a [reaction][padded] block (T, M per cell).
void or_rate_block(void *h, const double *T, const double *M, u32 cells, u32 padded, double *k) {
    const Mechanism *m = (const Mechanism *)h;
    std::vector<double> kk(m->R() ? m->R() : 1);
    for (u32 i = 0; i < cells; ++i) {
        rate_constants(m, T[i], M[i], kk.data());
        for (u32 r = 0; r < m->R(); ++r) k[(size_t)r * padded + i] = kk[r];
    }
}

// The seeded synthetic initial states of the shipped-mechanism workloads, drawn
// exactly as the module's workload generator draws them (so the CPU baselines
// integrate the same inputs without loading the module): a counter-based
// splitmix64 stream per cell, draw j of cell c = mix(seed + (c*256 + j + 1) *
// golden gamma); T ~ U[T_lo, T_hi], pH ~ U[3, 7] (drawn, unused), then each of
// the n species c ~ 10^U[lc_lo, lc_hi] mol/L (the last, H2O, = 55.5 mol/L),
// y = c * 6.02214076e20 cm^-3, M = 101325 / (1.380649e-23 T) * 1e-6 cm^-3.
static inline u64 wl_mix64(u64 z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static inline double wl_uniform(u64 seed, u64 cell, u32 j) {
    return (double)(wl_mix64(seed + (cell * 256ull + j + 1ull) * 0x9E3779B97F4A7C15ull) >> 11) * (1.0 / 9007199254740992.0);
}
// The uneven-stiffness workload's discharge power per cell: P0 x 10^(decades x draw 250).
void or_workload_air_power(u64 seed, u64 first_cell, u32 cells, double P0, double decades, double *power) {
    for (u32 i = 0; i < cells; ++i) power[i] = P0 * std::pow(10.0, decades * wl_uniform(seed, first_cell + i, 250));
}

void or_workload_air(u64 seed, u64 first_cell, u32 cells, u32 padded, u32 n, double T_lo, double T_hi, double lc_lo,
                     double lc_hi, double *y, double *T_out, double *M_out) {
    for (u32 i = 0; i < cells; ++i) {
        const u64 c = first_cell + i;
        const double T = T_lo + (T_hi - T_lo) * wl_uniform(seed, c, 0);
        for (u32 s = 0; s < n; ++s) {
            const double lc = lc_lo + (lc_hi - lc_lo) * wl_uniform(seed, c, 2 + s);
            const double conc = s == n - 1 ? 55.5 : std::pow(10.0, lc);
            y[(size_t)s * padded + i] = conc * 6.02214076e20;
        }
        T_out[i] = T;
        M_out[i] = 101325.0 / (1.380649e-23 * T) * 1e-6;
    }
}

// Single-cell kernels (Jacobian / LU unit tests). T = f64.
void or_fun(void *h, const double *k, const double *src, const double *y, double *f) { eval_fun(*(Mechanism *)h, k, src, y, f); }
void or_jac(void *h, const double *k, const double *y, double *jac) { eval_jac(*(Mechanism *)h, k, y, jac); }
void or_decomp_solve(void *h, const double *jac, double ghinv, double *x, double *lu_out) {
    Mechanism *m = (Mechanism *)h;
    std::vector<double> a(m->nnz);
    for (u32 i = 0; i < m->nnz; ++i) a[i] = -jac[i];
    factor(*m, ghinv, a.data());
    solve(*m, a.data(), x);
    if (lu_out) memcpy(lu_out, a.data(), sizeof(double) * m->nnz);
}

// One scalar f64 integration (Robertson / order tests): kin_integrate with V = f64.
s32 or_integrate_f64(void *h, s32 method_id, const Control *ctl, const double *k, const double *src, double *y,
                     double *t, double t_end, double *hh, double *stats4) {
    Mechanism *m = (Mechanism *)h;
    Method me = method_coefficients(method_id);
    Work<double> w;
    w.size(*m);
    Stats<double> st = {stats4[0], stats4[1], stats4[2], stats4[3]};
    integrate<double, false>(*m, me, *ctl, k, src, y, *t, t_end, *hh, st, nullptr, w);
    stats4[0] = st.steps; stats4[1] = st.rejects; stats4[2] = st.pulses; stats4[3] = st.failed;
    return 0;
}

// Lanes [begin, end) of a zone block, over local time [0, duration], on
// `threads` host threads (0 = all cores) in ~4 contiguous chunks per thread.
// precision 0: f64 lanes; 1: f32 lanes with the Delta formulation.
s32 or_advance(void *h, s32 method_id, const Control *ctl, const LaneArrays *arrays, u32 begin, u32 end,
               double duration, u32 precision, u32 threads) {
    Mechanism *m = (Mechanism *)h;
    Method me = method_coefficients(method_id);
    if (threads == 0) threads = std::thread::hardware_concurrency();
    if (threads == 0) threads = 1;
    if (end <= begin) return 0;
    u32 lanes = end - begin;
    u32 chunks = std::min<u32>(lanes, 4 * threads);
    u32 per = (lanes + chunks - 1) / chunks;
    auto run = [&](u32 b, u32 e) {
        if (precision == 1) advance_range<float, true>(m, &me, ctl, arrays, b, e, duration);
        else advance_range<double, false>(m, &me, ctl, arrays, b, e, duration);
    };
    if (threads == 1 || chunks == 1) {
        run(begin, end);
        return 0;
    }
    std::vector<std::thread> pool;
    u32 nchunk = (lanes + per - 1) / per;
    std::atomic<u32> cursor(0);
    for (u32 tI = 0; tI < threads; ++tI)
        pool.emplace_back([&]() {
            for (;;) {
                u32 c = cursor.fetch_add(1);
                if (c >= nchunk) break;
                u32 b = begin + c * per, e = std::min(end, b + per);
                run(b, e);
            }
        });
    for (auto &t : pool) t.join();
    return 0;
}

// Model of the module's mixed-precision path, lanes [begin, end): variant 0 =
// FP64 state with `sweeps` FP64-residual refinement sweeps (integrate_mixed),
// variant 1 = double-float state (integrate_mixed_df).
s32 or_advance_mixed(void *h, s32 method_id, const Control *ctl, const LaneArrays *arrays, u32 begin, u32 end,
                     double duration, u32 sweeps, u32 variant, u32 threads) {
    Mechanism *m = (Mechanism *)h;
    Method me = method_coefficients(method_id);
    if (threads == 0) threads = std::thread::hardware_concurrency();
    if (threads == 0) threads = 1;
    if (end <= begin) return 0;
    u32 lanes = end - begin, chunks = std::min<u32>(lanes, 4 * threads), per = (lanes + chunks - 1) / chunks;
    u32 nchunk = (lanes + per - 1) / per;
    std::atomic<u32> cursor(0);
    std::vector<std::thread> pool;
    for (u32 tI = 0; tI < std::min(threads, nchunk); ++tI)
        pool.emplace_back([&]() {
            for (;;) {
                u32 c = cursor.fetch_add(1);
                if (c >= nchunk) break;
                u32 b = begin + c * per, e = std::min(end, b + per);
                advance_mixed_range(m, &me, ctl, sweeps, variant, arrays, b, e, duration);
            }
        });
    for (auto &t : pool) t.join();
    return 0;
}

// Per-second averaged discharge source of the shipped mechanism (air_mech.cpp:205-276).
void or_source_delta(const double *y, u32 n, double energy_J_cm3, double T_K, double *delta) {
    source_delta(y, n, energy_J_cm3, T_K, delta);
}

// Explicit upwind advection of a [species][cells] channel block: `substeps`
// sweeps of x_j = fma(c, x_{j-1} - x_j, x_j), outlet to inlet so every cell
// reads its upstream neighbour's old value, cell 0 reading `inlet`
// (src/sim/nft.cpp:1066-1079, flux form and sweep order).
void or_advect(double *x, u32 species, u32 cells, u32 stride, const double *inlet, double courant, u32 substeps) {
    for (u32 it = 0; it < substeps; ++it)
        for (u32 s = 0; s < species; ++s) {
            double *row = x + (size_t)s * stride;
            for (u32 j = cells; j-- > 0;) {
                double v = row[j];
                double up = j == 0 ? inlet[s] : row[j - 1];
                row[j] = std::fma(courant, up - v, v);
            }
        }
}

u64 or_fnv1a(const void *data, u64 size) { return fnv1a(data, size); }

}   // extern "C"
