// Host-side mechanism compiler (see mech.h). Compiled with -ffp-contract=off:
// the rate constants are evaluated with host libm and uploaded, and their
// bits must match the reference's kin_eval_rate_constants.

#include "mech.h"
#include "air_source.h"

#include <math.h>
#include <string.h>

namespace sgb {

uint64_t fnv1a(const void *data, uint64_t size) {
    const uint8_t *p = (const uint8_t *)data;
    uint64_t h = 14695981039346656037ull;
    for (uint64_t i = 0; i < size; ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

void Model::fail(const char *what, const std::string &detail) {
    if (error.empty()) error = std::string(what) + ": " + detail;
}

int Model::find(const std::string &name) const {
    for (size_t s = 0; s < species.size(); ++s)
        if (species[s].name == name) return (int)s;
    return -1;
}

// Formula over N, O, H with counts; a parenthesised suffix is an electronic
// state label ("N2(A)", "O(1D)"): kin_build.cpp:62-76.
static bool atoms_of(const char *name, uint8_t atoms[3]) {
    atoms[0] = atoms[1] = atoms[2] = 0;
    const char *p = name;
    while (*p && *p != '(') {
        const char *letters = "NOH";
        const char *hit = strchr(letters, *p);
        if (!hit || !*p) return false;
        ++p;
        unsigned count = 0;
        while (*p >= '0' && *p <= '9') count = count * 10 + (unsigned)(*p++ - '0');
        atoms[hit - letters] = (uint8_t)(atoms[hit - letters] + (count ? count : 1));
    }
    return true;
}

uint32_t Model::add_species(const char *name, bool abstract_species) {
    Species s;
    s.name = name;
    if (!abstract_species && !atoms_of(name, s.atoms)) fail("species formula must use N, O, H", name);
    species.push_back(s);
    finalized = false;
    return n() - 1;
}

// Equation grammar of kin_build.cpp:100-148: tokens split on ' ' and '+',
// "->" separates reactants from products, "M" (third body) is skipped,
// tokens are at most 15 characters.
uint32_t Model::add_reaction(const char *equation, const RateLaw &law) {
    Reaction rx;
    rx.equation = equation;
    rx.law = law;
    const uint32_t r = R();
    std::vector<int> net(n(), 0);
    int balance[3] = {0, 0, 0};
    bool products = false, ok = true;
    for (const char *p = equation; *p;) {
        if (*p == ' ' || *p == '+') { ++p; continue; }
        if (p[0] == '-' && p[1] == '>') { products = true; p += 2; continue; }
        std::string token;
        while (*p && *p != ' ' && *p != '+' && !(p[0] == '-' && p[1] == '>') && token.size() < 15) token += *p++;
        if (token == "M") continue;
        int s = find(token);
        if (s < 0) { fail("unknown species in reaction", equation); ok = false; break; }
        int sign = products ? 1 : -1;
        if (!products) {
            if (rx.reactants.size() >= KIN_MAX_REACTANTS) { fail("too many reactants", equation); ok = false; break; }
            rx.reactants.push_back((uint32_t)s);
        }
        net[s] += sign;
        for (int e = 0; e < 3; ++e) balance[e] += sign * species[s].atoms[e];
    }
    if (ok) {
        if (!products || rx.reactants.empty()) fail("reaction needs reactants and '->'", equation);
        if (balance[0] || balance[1] || balance[2]) fail("element balance violated", equation);
        if (law.kind == kRateEqReverse && (uint32_t)law.ref >= r) fail("reverse reaction must follow its forward reaction", equation);
        for (uint32_t s = 0; s < n(); ++s) {
            if (!net[s]) continue;
            if (rx.net.size() >= KIN_MAX_NET) { fail("too many net species", equation); break; }
            rx.net.push_back({s, net[s]});
        }
    }
    reactions.push_back(rx);
    finalized = false;
    return r;
}

bool Model::finalize() {
    if (!error.empty()) return false;
    Symbolic &S = sym;
    const uint32_t N = n();
    S = Symbolic();
    S.n = N;
    auto at = [N](std::vector<uint8_t> &v, uint32_t i, uint32_t j) -> uint8_t & { return v[(size_t)i * N + j]; };
    S.pattern.assign((size_t)N * N, 0);
    for (uint32_t i = 0; i < N; ++i) at(S.pattern, i, i) = 1;
    for (const Reaction &rx : reactions)
        for (uint32_t q : rx.reactants)
            for (auto &e : rx.net) at(S.pattern, e.first, q) = 1;
    S.jac_pattern = S.pattern;
    // symbolic no-pivot elimination, row by row (IKJ)
    for (uint32_t i = 1; i < N; ++i)
        for (uint32_t k = 0; k < i; ++k) {
            if (!at(S.pattern, i, k)) continue;
            for (uint32_t j = k + 1; j < N; ++j)
                if (at(S.pattern, k, j)) at(S.pattern, i, j) = 1;
        }
    S.slot.assign((size_t)N * N, ~0u);
    for (uint32_t i = 0; i < N; ++i)
        for (uint32_t j = 0; j < N; ++j)
            if (at(S.pattern, i, j)) S.slot[(size_t)i * N + j] = S.nnz++;
    auto slot = [&](uint32_t i, uint32_t j) { return S.slot[(size_t)i * N + j]; };
    S.diag.resize(N);
    for (uint32_t i = 0; i < N; ++i) S.diag[i] = slot(i, i);
    // elimination ops: for row i, every k < i in the pattern in ascending k,
    // and its updates over the pattern of row k right of the diagonal
    S.div_begin.assign(N + 1, 0);
    for (uint32_t i = 0; i < N; ++i) {
        S.div_begin[i] = (uint32_t)S.divs.size();
        for (uint32_t k = 0; k < i; ++k) {
            if (!at(S.pattern, i, k)) continue;
            Symbolic::Div d = {slot(i, k), slot(k, k), (uint32_t)S.subs.size(), 0};
            for (uint32_t j = k + 1; j < N; ++j)
                if (at(S.pattern, k, j)) S.subs.push_back({slot(i, j), slot(k, j)});
            d.sub_end = (uint32_t)S.subs.size();
            S.divs.push_back(d);
        }
    }
    S.div_begin[N] = (uint32_t)S.divs.size();
    // triangular solves: lower ascending column, upper descending column
    S.lower_begin.assign(N + 1, 0);
    S.upper_begin.assign(N + 1, 0);
    for (uint32_t i = 0; i < N; ++i) {
        S.lower_begin[i] = (uint32_t)S.lower.size();
        S.upper_begin[i] = (uint32_t)S.upper.size();
        for (uint32_t j = 0; j < i; ++j)
            if (at(S.pattern, i, j)) S.lower.push_back({slot(i, j), j});
        for (uint32_t j = N - 1; j > i; --j)
            if (at(S.pattern, i, j)) S.upper.push_back({slot(i, j), j});
    }
    S.lower_begin[N] = (uint32_t)S.lower.size();
    S.upper_begin[N] = (uint32_t)S.upper.size();
    for (Reaction &rx : reactions) {
        rx.jac_slot.assign(rx.reactants.size(), std::vector<uint32_t>(rx.net.size()));
        for (size_t p = 0; p < rx.reactants.size(); ++p)
            for (size_t e = 0; e < rx.net.size(); ++e) rx.jac_slot[p][e] = slot(rx.net[e].first, rx.reactants[p]);
    }
    finalized = true;
    return true;
}

// kin_build.cpp:226-244, same operand order in every product.
void Model::rate_constants(double T, double M, double *k) const {
    const double t300 = T / 300.0;
    for (uint32_t r = 0; r < R(); ++r) {
        const RateLaw &l = reactions[r].law;
        switch (l.kind) {
            case kRateArrhenius: k[r] = l.p[0] * pow(t300, l.p[1]) * exp(-l.p[2] / T); break;
            case kRateThirdBody: k[r] = l.p[0] * pow(t300, l.p[1]) * exp(-l.p[2] / T) * M; break;
            case kRateTroe: {
                double k0m = l.p[0] * pow(t300, l.p[1]) * M;
                double kinf = l.p[2] * pow(t300, l.p[3]);
                double ratio = k0m / kinf;
                double lg = log10(ratio);
                k[r] = (k0m / (1.0 + ratio)) * pow(l.p[4], 1.0 / (1.0 + lg * lg));
            } break;
            case kRateEqReverse: k[r] = k[l.ref] / (l.p[0] * exp(l.p[1] / T)); break;
            default: k[r] = 0.0; break;
        }
    }
}

bool Model::to_kinmech(KinMech *out) const {
    memset(out, 0, sizeof(*out));
    const Symbolic &S = sym;
    if (!finalized || n() > KIN_MAX_SPECIES || R() > KIN_MAX_REACTIONS || S.nnz > KIN_MAX_NNZ ||
        S.divs.size() > KIN_MAX_LU_DIV || S.subs.size() > KIN_MAX_LU_SUB)
        return false;
    out->species_count = n();
    out->reaction_count = R();
    for (uint32_t r = 0; r < R(); ++r) {
        const Reaction &rx = reactions[r];
        KinReaction &o = out->reactions[r];
        for (uint32_t p = 0; p < KIN_MAX_REACTANTS; ++p) o.reactant[p] = p < rx.reactants.size() ? (uint8_t)rx.reactants[p] : KIN_NONE;
        o.reactant_count = (uint8_t)rx.reactants.size();
        o.net_count = (uint8_t)rx.net.size();
        for (size_t e = 0; e < rx.net.size(); ++e) {
            o.net_species[e] = (uint8_t)rx.net[e].first;
            o.net_coef[e] = (int8_t)rx.net[e].second;
        }
        for (size_t p = 0; p < rx.reactants.size(); ++p)
            for (size_t e = 0; e < rx.net.size(); ++e) o.jac_index[p][e] = (uint16_t)rx.jac_slot[p][e];
    }
    out->nnz = S.nnz;
    for (uint32_t i = 0; i < n(); ++i) out->diag[i] = (uint16_t)S.diag[i];
    out->lu_div_count = (uint32_t)S.divs.size();
    out->lu_sub_count = (uint32_t)S.subs.size();
    for (uint32_t i = 0; i <= n(); ++i) {
        out->div_begin[i] = (uint16_t)S.div_begin[i];
        out->lower_begin[i] = (uint16_t)S.lower_begin[i];
        out->upper_begin[i] = (uint16_t)S.upper_begin[i];
    }
    for (size_t d = 0; d < S.divs.size(); ++d)
        out->lu_div[d] = {(uint16_t)S.divs[d].ik, (uint16_t)S.divs[d].kk, (uint16_t)S.divs[d].sub_begin, (uint16_t)S.divs[d].sub_end};
    for (size_t s = 0; s < S.subs.size(); ++s) out->lu_sub[s] = {(uint16_t)S.subs[s].ij, (uint16_t)S.subs[s].kj};
    for (size_t e = 0; e < S.lower.size(); ++e) out->lower[e] = {(uint16_t)S.lower[e].index, (uint8_t)S.lower[e].col, 0};
    for (size_t e = 0; e < S.upper.size(); ++e) out->upper[e] = {(uint16_t)S.upper[e].index, (uint8_t)S.upper[e].col, 0};
    return true;
}

// ---------------------------------------------------------------------------
// The shipped humid-air mechanism. The species order, equations and rate data
// are the reference's table (src/sim/kinetics/air_mech.cpp:30-103); the
// mechanism signature and the solver's op order both depend on them.

namespace {
struct AirRow {
    const char *equation;
    int32_t kind;
    double p[5];
    int32_t ref;
};
const char *const kAirSpecies[17] = {"O",    "O3", "N",   "NO",   "NO2", "NO3", "N2O5", "N2O", "HNO2",
                                     "HNO3", "OH", "HO2", "H2O2", "H",   "N2",  "O2",   "H2O"};
const AirRow kAirReactions[44] = {
    {"O + O2 + M -> O3 + M", 1, {6.0e-34, -2.4, 0.0}, 0},
    {"O + O3 -> O2 + O2", 0, {8.0e-12, 0.0, 2060.0}, 0},
    {"O + O + M -> O2 + M", 1, {5.2e-35, 0.0, -900.0}, 0},
    {"O + NO + M -> NO2 + M", 2, {9.0e-32, -1.5, 3.0e-11, 0.0, 0.6}, 0},
    {"O + NO2 -> NO + O2", 0, {5.1e-12, 0.0, -210.0}, 0},
    {"O + NO2 + M -> NO3 + M", 2, {2.5e-31, -1.8, 2.2e-11, -0.7, 0.6}, 0},
    {"O3 + NO -> NO2 + O2", 0, {3.0e-12, 0.0, 1500.0}, 0},
    {"O3 + NO2 -> NO3 + O2", 0, {1.2e-13, 0.0, 2450.0}, 0},
    {"NO3 + NO -> NO2 + NO2", 0, {1.5e-11, 0.0, -170.0}, 0},
    {"NO2 + NO3 + M -> N2O5 + M", 2, {2.0e-30, -4.4, 1.4e-12, -0.7, 0.6}, 0},
    {"N2O5 + M -> NO2 + NO3 + M", 3, {2.7e-27, 11000.0}, 9},
    {"NO + NO + O2 -> NO2 + NO2", 0, {3.3e-39, 0.0, -530.0}, 0},
    {"N2O5 + H2O -> HNO3 + HNO3", 0, {2.5e-22, 0.0, 0.0}, 0},
    {"N + NO -> N2 + O", 0, {2.1e-11, 0.0, -100.0}, 0},
    {"N + O2 -> NO + O", 0, {1.5e-11, 0.0, 3600.0}, 0},
    {"N + NO2 -> N2O + O", 0, {0.434 * 5.8e-12, 0.0, -220.0}, 0},
    {"N + NO2 -> NO + NO", 0, {0.333 * 5.8e-12, 0.0, -220.0}, 0},
    {"N + NO2 -> N2 + O + O", 0, {0.132 * 5.8e-12, 0.0, -220.0}, 0},
    {"N + NO2 -> N2 + O2", 0, {0.101 * 5.8e-12, 0.0, -220.0}, 0},
    {"N + O + M -> NO + M", 1, {5.5e-33, 0.0, -155.0}, 0},
    {"N + N + M -> N2 + M", 1, {8.3e-34, 0.0, -500.0}, 0},
    {"N + OH -> NO + H", 0, {4.7e-11, 0.0, 0.0}, 0},
    {"OH + OH + M -> H2O2 + M", 2, {6.9e-31, -1.0, 2.6e-11, 0.0, 0.6}, 0},
    {"OH + OH -> H2O + O", 0, {1.8e-12, 0.0, 0.0}, 0},
    {"OH + O -> H + O2", 0, {1.8e-11, 0.0, -180.0}, 0},
    {"OH + O3 -> HO2 + O2", 0, {1.7e-12, 0.0, 940.0}, 0},
    {"OH + HO2 -> H2O + O2", 0, {4.8e-11, 0.0, -250.0}, 0},
    {"OH + H2O2 -> HO2 + H2O", 0, {1.8e-12, 0.0, 0.0}, 0},
    {"HO2 + HO2 -> H2O2 + O2", 0, {3.0e-13, 0.0, -460.0}, 0},
    {"HO2 + O -> OH + O2", 0, {3.0e-11, 0.0, -200.0}, 0},
    {"HO2 + O3 -> OH + O2 + O2", 0, {1.0e-14, 0.0, 490.0}, 0},
    {"H + O2 + M -> HO2 + M", 2, {4.4e-32, -1.3, 7.5e-11, 0.2, 0.6}, 0},
    {"H + O3 -> OH + O2", 0, {1.4e-10, 0.0, 470.0}, 0},
    {"H + HO2 -> OH + OH", 0, {7.2e-11, 0.0, 0.0}, 0},
    {"O + H2O2 -> OH + HO2", 0, {1.4e-12, 0.0, 2000.0}, 0},
    {"OH + NO + M -> HNO2 + M", 2, {7.0e-31, -2.6, 3.6e-11, -0.1, 0.6}, 0},
    {"OH + NO2 + M -> HNO3 + M", 2, {1.8e-30, -3.0, 2.8e-11, 0.0, 0.6}, 0},
    {"OH + HNO2 -> NO2 + H2O", 0, {1.8e-11, 0.0, 390.0}, 0},
    {"OH + HNO3 -> NO3 + H2O", 0, {1.5e-13, 0.0, 0.0}, 0},
    {"HO2 + NO -> OH + NO2", 0, {3.3e-12, 0.0, -270.0}, 0},
    {"H + NO2 -> OH + NO", 0, {4.0e-10, 0.0, 340.0}, 0},
    {"OH + NO3 -> HO2 + NO2", 0, {2.2e-11, 0.0, 0.0}, 0},
    {"HO2 + NO3 -> OH + NO2 + O2", 0, {3.5e-12, 0.0, 0.0}, 0},
    {"O3 + M -> O2 + O + M", 1, {7.2e-10, 0.0, 11400.0}, 0},
};
}   // namespace

void define_air(Model *m) {
    *m = Model();
    for (const char *s : kAirSpecies) m->add_species(s, false);
    for (const AirRow &row : kAirReactions) {
        RateLaw l;
        l.kind = row.kind;
        for (int i = 0; i < 5; ++i) l.p[i] = row.p[i];
        l.ref = row.ref;
        m->add_reaction(row.equation, l);
    }
}

// Rosenbrock coefficients in KPP form (Sandu et al., Atmos. Env. 1997); the
// values are the reference's (src/sim/kinetics/kin_solver.h:352-395).
KinMethod method_coefficients(uint32_t id) {
    KinMethod r;
    memset(&r, 0, sizeof(r));
    switch (id) {
        case 0: {
            double g = 1.0 + 1.0 / 1.4142135623730950488;
            r.name = "ros2";
            r.stages = 2; r.order = 2;
            r.a[0] = 1.0 / g;
            r.c[0] = -2.0 / g;
            r.m[0] = 3.0 / (2.0 * g); r.m[1] = 1.0 / (2.0 * g);
            r.e[0] = 1.0 / (2.0 * g); r.e[1] = 1.0 / (2.0 * g);
            r.gamma0 = g;
            r.new_f[0] = r.new_f[1] = 1;
        } break;
        case 1: {
            r.name = "ros3";
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
        } break;
        case 2: {
            r.name = "rodas3";
            r.stages = 4; r.order = 3;
            const double a[6] = {0.0, 2.0, 0.0, 2.0, 0.0, 1.0};
            const double c[6] = {4.0, 1.0, -1.0, 1.0, -1.0, -8.0 / 3.0};
            const double mm[4] = {2.0, 0.0, 1.0, 1.0};
            const double e[4] = {0.0, 0.0, 0.0, 1.0};
            memcpy(r.a, a, sizeof(a));
            memcpy(r.c, c, sizeof(c));
            memcpy(r.m, mm, sizeof(mm));
            memcpy(r.e, e, sizeof(e));
            r.gamma0 = 0.5;
            r.new_f[0] = r.new_f[1] = r.new_f[2] = r.new_f[3] = 1;
        } break;
        default: break;
    }
    return r;
}

// ---------------------------------------------------------------------------
// Averaged / per-pulse discharge source (air_mech.cpp:164-276, default G-values): the
// shared restatement of air_source.h with the temperature factors from host libm.

void air_source_temperature(double T_K, double *tf) {
    tf[0] = pow(T_K / 300.0, 0.55);
    tf[1] = exp(110.0 / T_K);
    tf[2] = exp(55.0 / T_K);
    tf[3] = exp(60.0 / T_K);
    tf[4] = exp(20.0 / T_K);
}

void air_source_delta(const double *y, uint32_t n, double energy_J_cm3, double T_K, double *d) {
    double tf[kAirTempFactors];
    air_source_temperature(T_K, tf);
    air_source_delta_tf(y, n, energy_J_cm3, air_source_defaults(), tf, d);
}

}   // namespace sgb
