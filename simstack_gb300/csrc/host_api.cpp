// Host-side exports: the mechanism compiler (kin_model_*) and the seeded
// synthetic workloads the benchmarks and tests run (sgb_workload_*).
// Compiled with -ffp-contract=off (rate constants must match host libm bit
// for bit wherever they are recomputed).

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "../../include/simstack_gpu.h"
#include "mech.h"

using namespace sgb;

struct KinModelHandle {
    Model model;
};

namespace sgb {
const Model *model_of(const KinModelHandle *h) { return h ? &h->model : nullptr; }
}   // namespace sgb

SGB_API KinModelHandle *kin_model_new(void) { return new (std::nothrow) KinModelHandle(); }

SGB_API KinModelHandle *kin_model_air(void) {
    KinModelHandle *h = new (std::nothrow) KinModelHandle();
    if (!h) return nullptr;
    define_air(&h->model);
    h->model.finalize();
    return h;
}

SGB_API void kin_model_free(KinModelHandle *h) { delete h; }

SGB_API uint32_t kin_model_add_species(KinModelHandle *h, const char *name, int32_t abstract_species) {
    return h->model.add_species(name, abstract_species != 0);
}

SGB_API uint32_t kin_model_add_reaction(KinModelHandle *h, const char *equation, int32_t kind, const double *params, int32_t ref) {
    RateLaw l;
    l.kind = kind;
    int count = kind == kRateTroe ? 5 : kind == kRateEqReverse ? 2 : 3;
    for (int i = 0; i < count; ++i) l.p[i] = params ? params[i] : 0.0;
    if (kind == kRateTroe && params == nullptr) l.p[4] = 0.6;
    l.ref = ref;
    return h->model.add_reaction(equation, l);
}

SGB_API int32_t kin_model_finalize(KinModelHandle *h) { return h->model.finalize() ? 0 : 1; }

// Equation text of reaction r (NUL-terminated, truncated to size); 0 if r is out of range.
SGB_API int32_t kin_model_equation(const KinModelHandle *h, uint32_t r, char *out, uint32_t size) {
    if (r >= h->model.R() || size == 0) return 0;
    snprintf(out, size, "%s", h->model.reactions[r].equation.c_str());
    return 1;
}

SGB_API const char *kin_model_error(const KinModelHandle *h) { return h->model.error.c_str(); }

SGB_API void kin_model_counts(const KinModelHandle *h, uint64_t *c) {
    const Model &m = h->model;
    c[0] = m.n();
    c[1] = m.R();
    c[2] = m.sym.nnz;
    c[3] = m.sym.divs.size();
    c[4] = m.sym.subs.size();
    c[5] = m.sym.lower.size();
    c[6] = m.sym.upper.size();
}

SGB_API int32_t kin_model_kinmech(const KinModelHandle *h, KinMech *out) { return h->model.to_kinmech(out) ? 0 : 1; }

SGB_API uint64_t kin_mech_signature(const KinMech *mech) { return fnv1a(mech, sizeof(KinMech)); }

// The cooperative kernels' wide-index image of a finalized model or of a KinMech: its size
// (0 if it cannot be built); copied to `out` when `capacity` suffices.
SGB_API uint64_t kin_model_coop_image(const KinModelHandle *h, void *out, uint64_t capacity) {
    std::vector<uint8_t> img;
    if (!h || !coop_image(h->model, &img)) return 0;
    if (out && capacity >= img.size()) memcpy(out, img.data(), img.size());
    return img.size();
}

SGB_API uint64_t kin_mech_coop_image(const KinMech *mech, void *out, uint64_t capacity) {
    std::vector<uint8_t> img;
    if (!mech || !coop_image(*mech, &img)) return 0;
    if (out && capacity >= img.size()) memcpy(out, img.data(), img.size());
    return img.size();
}

SGB_API void kin_model_rate_constants(const KinModelHandle *h, double T, double M, double *k) { h->model.rate_constants(T, M, k); }

SGB_API void kin_model_rate_block(const KinModelHandle *h, const double *T, const double *M, uint32_t cells, uint32_t padded,
                                  double *k) {
    const uint32_t R = h->model.R();
    std::vector<double> kk(R ? R : 1);
    for (uint32_t i = 0; i < cells; ++i) {
        h->model.rate_constants(T[i], M[i], kk.data());
        for (uint32_t r = 0; r < R; ++r) k[(size_t)r * padded + i] = kk[r];
    }
}

SGB_API KinMethod kin_method_coefficients(uint32_t method_id) { return method_coefficients(method_id); }

SGB_API void kin_air_source_delta(const double *y, uint32_t species, double energy_J_cm3, double T_K, double *delta) {
    air_source_delta(y, species, energy_J_cm3, T_K, delta);
}

// ---------------------------------------------------------------------------
// Seeded synthetic workloads. Counter-based splitmix64: draw j of cell c is
// mix(seed + (c * 256 + j + 1) * golden-gamma), so any subset of cells (the
// first 4,096 of a 1,048,576-cell batch) draws the same values wherever it
// is generated, and cells can be generated in any order or in parallel.

namespace {
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
inline double uniform(uint64_t seed, uint64_t cell, uint32_t j) {
    uint64_t x = mix64(seed + (cell * 256ull + j + 1ull) * 0x9E3779B97F4A7C15ull);
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}
const double kAvogadroPerCm3 = 6.02214076e20;   // mol/L -> molecules/cm^3
const double kBoltzmann = 1.380649e-23;
const double kPressure = 101325.0;
}   // namespace

// Shipped-mechanism cells [first_cell, first_cell + cells) into columns
// [0, cells) of a [species][padded] y block and [reaction][padded] k block.
// Draw order per cell: T ~ U[T_lo, T_hi] K, pH ~ U[3, 7] (drawn and unused:
// the mechanism has no H+), then every species in mechanism order
// c ~ 10^U[lc_lo, lc_hi] mol/L; H2O is then set to 55.5 mol/L.
// y = c * 6.02214076e20 cm^-3; M = p / (kB T) * 1e-6 cm^-3 at p = 1 atm.
SGB_API void sgb_workload_air(uint64_t seed, uint64_t first_cell, uint32_t cells, uint32_t padded, double T_lo, double T_hi,
                              double lc_lo, double lc_hi, double *y, double *k, double *T_out, double *pH_out) {
    static Model air;
    static bool built = false;
    if (!built) {
        define_air(&air);
        air.finalize();
        built = true;
    }
    const uint32_t n = air.n(), R = air.R();
    const uint32_t h2o = n - 1;
    std::vector<double> kk(R);
    for (uint32_t i = 0; i < cells; ++i) {
        const uint64_t c = first_cell + i;
        double T = T_lo + (T_hi - T_lo) * uniform(seed, c, 0);
        double pH = 3.0 + 4.0 * uniform(seed, c, 1);
        for (uint32_t s = 0; s < n; ++s) {
            double lc = lc_lo + (lc_hi - lc_lo) * uniform(seed, c, 2 + s);
            double conc = s == h2o ? 55.5 : pow(10.0, lc);
            y[(size_t)s * padded + i] = conc * kAvogadroPerCm3;
        }
        double M = kPressure / (kBoltzmann * T) * 1e-6;
        air.rate_constants(T, M, kk.data());
        for (uint32_t r = 0; r < R; ++r) k[(size_t)r * padded + i] = kk[r];
        if (T_out) T_out[i] = T;
        if (pH_out) pH_out[i] = pH;
    }
}

// Averaged discharge source per cell: power = P0 * 10^U[0, decades] W/cm^3
// (draw 250 of the cell's stream), src = the per-second species change of the
// shipped source model at the cell's initial composition and temperature.
SGB_API void sgb_workload_air_source(uint64_t seed, uint64_t first_cell, uint32_t cells, uint32_t padded, double P0,
                                     double decades, const double *y, const double *T, double *src, double *power_out) {
    const uint32_t n = 17;
    double yy[17], d[17];
    for (uint32_t i = 0; i < cells; ++i) {
        const uint64_t c = first_cell + i;
        double power = P0 * pow(10.0, decades * uniform(seed, c, 250));
        for (uint32_t s = 0; s < n; ++s) yy[s] = y[(size_t)s * padded + i];
        air_source_delta(yy, n, power, T[i], d);
        for (uint32_t s = 0; s < n; ++s) src[(size_t)s * padded + i] = d[s];
        if (power_out) power_out[i] = power;
    }
}

// Synthetic abstract mechanism: `species` species S0..S{n-1}, `reactions`
// reactions, a fraction `bimolecular` with two reactants (the rest one),
// reactant indices uniform, `products` distinct product species drawn
// uniformly among the species that are not reactants of that reaction, rate
// constants k ~ 10^U[lk_lo, lk_hi] (one per reaction, the same in every cell).
// Stream: cell index 2^40 + r, so it never overlaps cell draws.
SGB_API KinModelHandle *sgb_workload_synthetic_mech(uint64_t seed, uint32_t species, uint32_t reactions, double bimolecular,
                                                    uint32_t products, double lk_lo, double lk_hi, double *k_out) {
    KinModelHandle *h = new (std::nothrow) KinModelHandle();
    if (!h) return nullptr;
    char name[32];
    for (uint32_t s = 0; s < species; ++s) {
        snprintf(name, sizeof(name), "S%u", s);
        h->model.add_species(name, true);
    }
    for (uint32_t r = 0; r < reactions; ++r) {
        const uint64_t c = (1ull << 40) + r;
        uint32_t j = 0;
        bool bi = uniform(seed, c, j++) < bimolecular;
        uint32_t a = (uint32_t)(uniform(seed, c, j++) * species) % species;
        uint32_t b = bi ? (uint32_t)(uniform(seed, c, j++) * species) % species : a;
        std::vector<uint32_t> prod;
        while (prod.size() < products && j < 240) {
            uint32_t p = (uint32_t)(uniform(seed, c, j++) * species) % species;
            bool clash = p == a || (bi && p == b);
            for (uint32_t q : prod) clash = clash || q == p;
            if (!clash) prod.push_back(p);
        }
        std::string eq = "S" + std::to_string(a);
        if (bi) eq += " + S" + std::to_string(b);
        eq += " ->";
        for (size_t q = 0; q < prod.size(); ++q) eq += (q ? " + S" : " S") + std::to_string(prod[q]);
        double lk = lk_lo + (lk_hi - lk_lo) * uniform(seed, c, 245);
        double kval = pow(10.0, lk);
        RateLaw l;
        l.kind = kRateArrhenius;
        l.p[0] = kval;
        h->model.add_reaction(eq.c_str(), l);
        if (k_out) k_out[r] = kval;
    }
    h->model.finalize();
    return h;
}

// Synthetic-mechanism cells: c ~ 10^U[lc_lo, lc_hi] for every species (draws 0..n-1).
SGB_API void sgb_workload_synthetic_cells(uint64_t seed, uint64_t first_cell, uint32_t cells, uint32_t padded, uint32_t species,
                                          double lc_lo, double lc_hi, double *y) {
    for (uint32_t i = 0; i < cells; ++i)
        for (uint32_t s = 0; s < species; ++s)
            y[(size_t)s * padded + i] = pow(10.0, lc_lo + (lc_hi - lc_lo) * uniform(seed, first_cell + i, s));
}
