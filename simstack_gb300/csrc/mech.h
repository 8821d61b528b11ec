// Host-side mechanism model of the GB300 kinetics module.
//
// Builds a mass-action mechanism from readable equations and compiles its
// symbolic sparse LU: the non-zero pattern of J plus the diagonal, the fill-in
// of a no-pivot IKJ elimination, a row-major compact numbering, and the flat
// elimination / triangular-solve op lists the solver walks. The rules are the
// reference's (src/sim/kinetics/kin_build.cpp:78-223): the same pattern, the
// same pivot order and the same op order, because the solver's results are
// only bit-identical to the reference's when every floating-point operation
// happens in the same sequence. Indices here are 32-bit, so the same compiler
// serves mechanisms beyond the reference's u16 tables (200 species, 1,200
// reactions); KinMech (the reference layout) is emitted when it fits.

#ifndef SGB_MECH_H
#define SGB_MECH_H

#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/simstack_gpu.h"

namespace sgb {

enum RateKind : int32_t { kRateArrhenius = 0, kRateThirdBody = 1, kRateTroe = 2, kRateEqReverse = 3 };

struct RateLaw {
    int32_t kind = kRateArrhenius;
    double p[5] = {0, 0, 0, 0, 0};   // Arrhenius/third body: A n E; Troe: A0 n0 Ainf ninf fc; eq-reverse: KeqA KeqB
    int32_t ref = 0;                   // eq-reverse: forward reaction
};

struct Species {
    std::string name;
    uint8_t atoms[3] = {0, 0, 0};   // N, O, H
};

struct Reaction {
    std::string equation;
    RateLaw law;
    std::vector<uint32_t> reactants;                  // equation order (repeats kept)
    std::vector<std::pair<uint32_t, int32_t>> net;    // (species, net change), species order, non-zero only
    std::vector<std::vector<uint32_t>> jac_slot;      // [reactant position][net entry] -> compact index
};

// The compiled symbolic phase.
struct Symbolic {
    uint32_t n = 0, nnz = 0;
    std::vector<uint8_t> pattern;                 // n*n after fill-in
    std::vector<uint32_t> slot;                   // n*n -> compact index or ~0u
    std::vector<uint32_t> diag;                   // n
    std::vector<uint32_t> div_begin;              // n+1, into divs
    struct Div { uint32_t ik, kk, sub_begin, sub_end; };
    struct Sub { uint32_t ij, kj; };
    struct Entry { uint32_t index, col; };
    std::vector<Div> divs;
    std::vector<Sub> subs;
    std::vector<uint32_t> lower_begin, upper_begin;   // n+1
    std::vector<Entry> lower, upper;                  // upper rows in DESCENDING column order
    std::vector<uint8_t> jac_pattern;                 // n*n pattern of J + diag before fill
};

class Model {
public:
    std::vector<Species> species;
    std::vector<Reaction> reactions;
    Symbolic sym;
    bool finalized = false;
    std::string error;

    uint32_t add_species(const char *name, bool abstract_species);
    uint32_t add_reaction(const char *equation, const RateLaw &law);
    bool finalize();
    void rate_constants(double T, double M, double *k) const;
    // Reference-layout tables; false if a capacity is exceeded.
    bool to_kinmech(KinMech *out) const;
    uint32_t n() const { return (uint32_t)species.size(); }
    uint32_t R() const { return (uint32_t)reactions.size(); }

private:
    void fail(const char *what, const std::string &detail);
    int find(const std::string &name) const;
};

// Wide-index image for the cooperative kernels (coop.h); false if the model is not finalized.
bool coop_image(const Model &m, std::vector<uint8_t> *out);
bool coop_image(const KinMech &k, std::vector<uint8_t> *out);

void define_air(Model *m);   // the shipped 17-species, 44-reaction humid-air mechanism
uint64_t fnv1a(const void *data, uint64_t size);
KinMethod method_coefficients(uint32_t id);
void air_source_delta(const double *y, uint32_t n, double energy_J_cm3, double T_K, double *delta);
// The five temperature factors of the source's channel rates (host libm), for air_source_delta_tf.
void air_source_temperature(double T_K, double *tf);

}   // namespace sgb

#endif
