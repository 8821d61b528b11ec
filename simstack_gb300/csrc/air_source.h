// Discharge source of the shipped humid-air mechanism (src/sim/kinetics/air_mech.cpp:110-276),
// shared by the host (rate tables, tests) and the device zone driver: electron-impact
// channels scaled by the parents' mole fractions, then the quasi-steady fates of N2(A),
// N(2D) and O(1D), each distributed over its partners in proportion to k [partner] with a
// half-partner cap. The five temperature factors the channel rates need (one pow, four
// exp of T) are computed once per zone on the host with libm (air_source_temperature) and
// passed in, so host and device perform the same IEEE operations on them; built with
// -ffp-contract=off on the host and -fmad=false on the device, the two give the same bits.

#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define SGB_HD __host__ __device__ __forceinline__
#else
#define SGB_HD inline
#endif

namespace sgb {

// AirSourceModel (air_mech.cpp:133-148) with its G-values resolved: per 100 eV, at the
// reference gas's mole fractions; filament_J_cm3 > 0 selects the filament picture for
// the pulse rate (power / filament_J_cm3) instead of one pulse per half-cycle.
struct AirSourceParams {
    double g_O2_diss, f_O1D, g_N2A, g_N2_diss, g_OH_per_100eV, filament_J_cm3;
};

SGB_HD AirSourceParams air_source_defaults() { return AirSourceParams{1.5, 0.5, 1.5, 0.4, 0.3, 0.0}; }

namespace air {
enum : uint32_t { O = 0, O3, N, NO, NO2, NO3, N2O5, N2O, HNO2, HNO3, OH, HO2, H2O2, H, N2, O2, H2O, kSpecies };
}
constexpr int kAirTempFactors = 5;   // (T/300)^0.55, exp(110/T), exp(55/T), exp(60/T), exp(20/T)

struct AirFate {
    double k;
    uint32_t partner;
};

SGB_HD void air_split_fates(const AirFate *fate, uint32_t count, const double *y, double amount, double *share) {
    double sum = 0.0;
    uint32_t big = 0;
    for (uint32_t c = 0; c < count; ++c) {
        share[c] = fate[c].k * y[fate[c].partner];
        if (share[c] > share[big]) big = c;
        sum += share[c];
    }
    if (sum <= 0.0) {
        for (uint32_t c = 0; c < count; ++c) share[c] = c == big ? 1.0 : 0.0;
        return;
    }
    double moved = 0.0;
    for (uint32_t c = 0; c < count; ++c) {
        share[c] /= sum;
        double cap = amount > 0.0 ? 0.5 * y[fate[c].partner] / amount : 1.0;
        if (c != big && share[c] > cap) {
            moved += share[c] - cap;
            share[c] = cap;
        }
    }
    share[big] += moved;
}

// Species change per cm^3 for energy_J_cm3 deposited into gas y (n = 17 species);
// tf = the zone's five temperature factors.
SGB_HD void air_source_delta_tf(const double *y, uint32_t n, double energy_J_cm3, const AirSourceParams &p, const double *tf,
                                double *d) {
    using namespace air;
    for (uint32_t s = 0; s < n; ++s) d[s] = 0.0;
    double total = 0.0;
    for (uint32_t s = 0; s < n; ++s) total += y[s];
    if (total <= 0.0 || energy_J_cm3 <= 0.0) return;
    double hundreds_eV = energy_J_cm3 * 6.241509074e18 * 0.01;
    double dO2 = p.g_O2_diss * (y[O2] / total / 0.21) * hundreds_eV;
    double dA = p.g_N2A * (y[N2] / total / 0.78) * hundreds_eV;
    double dN2 = p.g_N2_diss * (y[N2] / total / 0.78) * hundreds_eV;
    double dOH = p.g_OH_per_100eV * (y[H2O] / total / 0.02) * hundreds_eV;
    double d1D = p.f_O1D * dO2;
    d[O2] -= dO2;
    d[O] += 2.0 * dO2 - d1D;
    d[N2] -= dA + dN2;
    d[N] += dN2;
    d[OH] += dOH;
    d[H] += dOH;
    d[H2O] -= dOH;
    const double k_o2 = tf[0];
    double f[10];
    const AirFate n2a[9] = {{2.5e-12 * k_o2, O2}, {1.3e-12 * k_o2, O2}, {7.8e-14 * k_o2, O2}, {7.0e-12, O}, {7.0e-11, NO},
                            {1.0e-12, NO2},       {8.0e-11, N2O},       {5.0e-14, H2O},       {3.0e-16, N2}};
    air_split_fates(n2a, 9, y, dA, f);
    d[N2] += dA * (f[0] + f[1] + f[4] + f[5] + f[6] + f[7] + f[8]);
    d[O2] -= dA * (f[0] + f[2]);
    d[O] += dA * (2.0 * f[0] + f[2] + f[5]);
    d[N2O] += dA * (f[2] - f[6]);
    d[O] -= dA * f[3];
    d[NO] += dA * (f[3] + f[5] + f[6]);
    double n2d = dN2 + dA * f[3];
    d[NO2] -= dA * f[5];
    d[N] += dA * f[6];
    d[H2O] -= dA * f[7];
    d[H] += dA * f[7];
    d[OH] += dA * f[7];
    const AirFate n2dfate[5] = {{5.2e-12, O2}, {1.7e-14, N2}, {6.9e-13, O}, {6.0e-11, NO}, {2.2e-12, N2O}};
    air_split_fates(n2dfate, 5, y, n2d, f);
    d[O2] -= n2d * f[0];
    d[NO] += n2d * (f[0] - f[3] + f[4]);
    d[O] += n2d * (f[0] + f[3]);
    d[N] += n2d * (f[1] + f[2]);
    d[N2] += n2d * (f[3] + f[4]);
    d[N2O] -= n2d * f[4];
    const AirFate o1d[6] = {{2.15e-11 * tf[1], N2}, {3.3e-11 * tf[2], O2}, {1.63e-10 * tf[3], H2O},
                            {7.26e-11 * tf[4], N2O}, {4.63e-11 * tf[4], N2O}, {2.4e-10, O3}};
    air_split_fates(o1d, 6, y, d1D, f);
    d[O] += d1D * (f[0] + f[1]);
    d[O3] -= d1D * f[5];
    d[O2] += d1D * f[5] * 1.5;
    d[O] += d1D * f[5];
    d[H2O] -= d1D * f[2];
    d[OH] += d1D * f[2] * 2.0;
    d[N2O] -= d1D * (f[3] + f[4]);
    d[NO] += d1D * f[3] * 2.0;
    d[N2] += d1D * f[4];
    d[O2] += d1D * f[4];
}

}   // namespace sgb
