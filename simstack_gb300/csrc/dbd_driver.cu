// The zone driver of a DBD master step on the device (src/sim/dbd.cpp:118-158, 466-483):
// the discharge source and pulse schedule, the pulse commit and the plug flow between
// zones, as kernels on the module stream over a zone block that stays in device memory.
// The reference runs these on the host and uploads the whole block before every advance
// (dbd.cpp:279, 294); here a multi-step run uploads nothing between steps.
//
// Every zone is a thread; each performs the reference's IEEE operations in the
// reference's order (built with -fmad=false), so the results are bit-identical to the
// host driver. What needs libm stays on the host: the rate constants (uploaded when T
// or p change, as dbd_zones_prepare_rates is called) and the source's five temperature
// factors per zone (kin_air_source_temperature).

#include <cuda_runtime.h>
#include <string.h>

#include "../../include/simstack_gpu.h"
#include "air_source.h"

namespace sgb {
cudaError_t module_enqueue_advance(const GpuKinLaunch *L);
cudaError_t module_finish(float *device_ms);
cudaError_t module_mark_start();
cudaStream_t module_stream();
cudaError_t module_scratch(size_t bytes, void **out);
void air_source_temperature(double T_K, double *tf);
}   // namespace sgb

using namespace sgb;

namespace {

constexpr uint32_t kDbdBlock = 128;
// Guard of the pulse-count loop: more pulses than this in one master step is not a
// schedule this driver accepts (the zone is marked failed instead of looping on).
constexpr double kMaxPulsesPerStep = 16777216.0;

__global__ void dbd_source_kernel(const __grid_constant__ GpuDbdZones z, const AirSourceParams prm, uint32_t pulsed, double t0,
                                  double t1) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t P = z.padded;
    if (i >= P) return;
    double y[air::kSpecies], delta[air::kSpecies], tf[kAirTempFactors];
    for (uint32_t s = 0; s < air::kSpecies; ++s) y[s] = z.y[(size_t)s * P + i];
    for (int j = 0; j < kAirTempFactors; ++j) tf[j] = z.source_temp[(size_t)j * P + i];
    const double power = z.power_W_cm3[i], freq = z.freq_Hz[i];
    const bool on = power > 0.0 && freq > 0.0;
    const double pulses_per_s = prm.filament_J_cm3 > 0.0 && on ? power / prm.filament_J_cm3 : 2.0 * freq;
    if (pulsed && on) {
        air_source_delta_tf(y, air::kSpecies, power / pulses_per_s, prm, tf, delta);
        for (uint32_t s = 0; s < air::kSpecies; ++s) {
            z.pulse[(size_t)s * P + i] = delta[s];
            z.src[(size_t)s * P + i] = 0.0;
        }
        const double period = 1.0 / pulses_per_s;
        z.period[i] = period;
        const double next = z.pulse_index[i] + 1.0;
        double count = 0.0;
        while ((next + count) * period <= t1 && count < kMaxPulsesPerStep) count += 1.0;
        if (count >= kMaxPulsesPerStep) z.failed[i] = 1.0;
        z.pulse_first[i] = next * period - t0;
        z.pulse_count[i] = count;
    } else {
        air_source_delta_tf(y, air::kSpecies, on ? power : 0.0, prm, tf, delta);
        for (uint32_t s = 0; s < air::kSpecies; ++s) {
            z.src[(size_t)s * P + i] = delta[s];
            z.pulse[(size_t)s * P + i] = 0.0;
        }
        z.period[i] = 0.0;
        z.pulse_first[i] = 0.0;
        z.pulse_count[i] = 0.0;
    }
}

__global__ void dbd_commit_kernel(const __grid_constant__ GpuDbdZones z) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < z.padded) z.pulse_index[i] += z.pulse_count[i];
}

// y[s][i] += a (up - y[s][i]) for zones i < count, up = zone i-1's state before this
// exchange (from `old`, a copy of the y rows) or, for zone 0, the feed gas at zone 0's
// operating point (air_feed, air_mech.cpp:280-288).
__global__ void dbd_flow_kernel(const __grid_constant__ GpuDbdZones z, const double *__restrict__ old, double a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= z.count) return;
    const uint32_t P = z.padded;
    double up;
    if (i == 0) {
        const double total = z.p_Pa[0] / (1.380649e-23 * z.T_K[0]) * 1e-6;
        const double dry = 1.0 - z.x_H2O[0];
        up = s == air::N2 ? total * dry * 0.79 : s == air::O2 ? total * dry * 0.21 : s == air::H2O ? total * z.x_H2O[0] : 0.0;
    } else {
        up = old[(size_t)s * P + i - 1];
    }
    double *yp = z.y + (size_t)s * P + i;
    *yp += a * (up - *yp);
}

bool zones_valid(const GpuDbdZones *z) {
    if (!z || z->padded == 0 || z->count > z->padded || z->n_species != air::kSpecies) return false;
    const double *rows[] = {z->y, z->h, z->steps, z->rejects, z->pulses, z->failed, z->k, z->src, z->pulse, z->period,
                            z->pulse_first, z->pulse_count, z->pulse_index, z->T_K, z->p_Pa, z->x_H2O, z->power_W_cm3,
                            z->freq_Hz, z->source_temp};
    for (const double *r : rows)
        if (!r) return false;
    return true;
}

AirSourceParams params_of(const GpuAirSource *src) {
    if (!src) return air_source_defaults();
    return AirSourceParams{src->g_O2_diss, src->f_O1D, src->g_N2A, src->g_N2_diss, src->g_OH_per_100eV, src->filament_J_cm3};
}

cudaError_t enqueue_source(const GpuDbdZones *z, const GpuAirSource *src, uint32_t pulsed, double t0, double t1) {
    dbd_source_kernel<<<(z->padded + kDbdBlock - 1) / kDbdBlock, kDbdBlock, 0, module_stream()>>>(*z, params_of(src), pulsed, t0, t1);
    return cudaGetLastError();
}

cudaError_t enqueue_commit(const GpuDbdZones *z) {
    dbd_commit_kernel<<<(z->padded + kDbdBlock - 1) / kDbdBlock, kDbdBlock, 0, module_stream()>>>(*z);
    return cudaGetLastError();
}

cudaError_t enqueue_flow(const GpuDbdZones *z, double residence_s, double dt) {
    if (residence_s <= 0.0 || z->count == 0) return cudaSuccess;   // dbd.cpp:470
    const double a = dt * (double)z->count / residence_s;
    if (!(a <= 1.0)) return cudaErrorInvalidValue;                  // the explicit step's stability bound (dbd.cpp:472)
    void *old = nullptr;
    const size_t bytes = (size_t)z->n_species * z->padded * sizeof(double);
    cudaError_t e = module_scratch(bytes, &old);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(old, z->y, bytes, cudaMemcpyDeviceToDevice, module_stream());
    if (e != cudaSuccess) return e;
    dim3 grid((z->count + kDbdBlock - 1) / kDbdBlock, z->n_species);
    dbd_flow_kernel<<<grid, kDbdBlock, 0, module_stream()>>>(*z, (const double *)old, a);
    return cudaGetLastError();
}

GpuKinLaunch launch_of(const GpuDbdZones *z, uint32_t precision, double duration) {
    GpuKinLaunch L;
    memset(&L, 0, sizeof(L));
    L.y = z->y; L.h = z->h; L.steps = z->steps; L.rejects = z->rejects; L.pulses = z->pulses; L.failed = z->failed;
    L.k = z->k; L.src = z->src; L.pulse = z->pulse; L.period = z->period;
    L.pulse_first = z->pulse_first; L.pulse_count = z->pulse_count;
    L.padded = z->padded;
    L.lane_count = 0;   // every padded lane, as dbd_advance_gpu (dbd.cpp:286-291)
    L.precision = precision;
    L.duration = duration;
    return L;
}

}   // namespace

SGB_API void kin_air_source_temperature(const double *T_K, uint32_t count, uint32_t padded, double *tf) {
    double v[kAirTempFactors];
    for (uint32_t i = 0; i < count; ++i) {
        air_source_temperature(T_K[i], v);
        for (int j = 0; j < kAirTempFactors; ++j) tf[(size_t)j * padded + i] = v[j];
    }
}

SGB_API int32_t gpu_dbd_prepare_source(const GpuDbdZones *z, const GpuAirSource *src, uint32_t pulsed, double t0, double t1) {
    if (!zones_valid(z)) return (int32_t)cudaErrorInvalidValue;
    cudaError_t e = enqueue_source(z, src, pulsed, t0, t1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(module_stream());
    return (int32_t)e;
}

SGB_API int32_t gpu_dbd_commit_pulses(const GpuDbdZones *z) {
    if (!zones_valid(z)) return (int32_t)cudaErrorInvalidValue;
    cudaError_t e = enqueue_commit(z);
    if (e == cudaSuccess) e = cudaStreamSynchronize(module_stream());
    return (int32_t)e;
}

SGB_API int32_t gpu_dbd_flow_exchange(const GpuDbdZones *z, double residence_s, double dt) {
    if (!zones_valid(z)) return (int32_t)cudaErrorInvalidValue;
    cudaError_t e = enqueue_flow(z, residence_s, dt);
    if (e == cudaSuccess) e = cudaStreamSynchronize(module_stream());
    return (int32_t)e;
}

SGB_API int32_t gpu_dbd_step(const GpuDbdZones *z, const GpuAirSource *src, uint32_t pulsed, double t0, double dt,
                             uint32_t precision, uint32_t chained, double residence_s, float *step_ms) {
    if (!zones_valid(z) || !(dt >= 0.0) || precision > 2) return (int32_t)cudaErrorInvalidValue;
    if (chained && residence_s > 0.0 && z->count > 0 && !(dt * (double)z->count / residence_s <= 1.0))
        return (int32_t)cudaErrorInvalidValue;
    const double t1 = t0 + dt;   // the scene clock (dbd_scene.cpp:232)
    cudaError_t e = module_mark_start();
    if (e == cudaSuccess) e = enqueue_source(z, src, pulsed, t0, t1);
    if (e == cudaSuccess) {
        const GpuKinLaunch L = launch_of(z, precision, dt);
        e = module_enqueue_advance(&L);
    }
    if (e == cudaSuccess) e = enqueue_commit(z);
    if (e == cudaSuccess && chained) e = enqueue_flow(z, residence_s, dt);
    cudaError_t f = module_finish(step_ms);   // waits for the stream; reads the bounded-wait flag
    return (int32_t)(e != cudaSuccess ? e : f);
}
