// The NFT film transport of one coupling window on the device (src/sim/nft.cpp:1028-1106,
// nft_transport): per channel (lane) and substep, flux-form upwind advection of the nine
// film fields in f32 deltas from the inlet, the linearised wall / radiant / latent heat
// update, O2 exchange toward saturation, and the plant sites' uptake booked as what was
// actually removed; then the window's outlet sums and film evaporation.
//
// Data: device copies of the reference's group arrays in the reference's byte layout
// (nft.cpp:134-203: groups of 8 channels, every per-cell quantity a [8] f32 lane array),
// packed group after group. One CTA per group; thread (lane l, chunk q) owns a contiguous
// run of cells of channel l. Within a substep the reference sweeps outlet -> inlet so
// that every cell reads its upstream neighbour's value from before the substep; the cells
// of a substep are therefore independent, and each thread sweeps its own run the same way
// (outlet end first). The one value a run needs from outside is the old state of the
// previous run's last cell: it is published in shared memory (double-buffered by
// substep parity) before the sweep, so a substep costs one CTA barrier. A warp covers 4
// runs x 8 lanes: each field access is four full 32-byte sectors.
//
// Every element receives the reference's f32 operations in the reference's order, issued
// as explicit PTX (no contraction, no reassociation). The reference runs the transport
// with x86 FTZ/DAZ set (NftFlushDenormals, nft.cpp:1130-1136) on x86-64 hosts and IEEE
// elsewhere; flush_denormals selects the matching PTX forms (.ftz or not), so the result
// is bit-identical to the reference on either kind of host. Bounded: no waits; every
// loop has a fixed trip count.

#include <cuda_runtime.h>

#include "../../include/simstack_gpu.h"

namespace sgb {
cudaError_t module_mark_start();
cudaError_t module_finish(float *device_ms);
cudaStream_t module_stream();
}   // namespace sgb

using namespace sgb;

namespace {

constexpr uint32_t kLanes = 8;
constexpr uint32_t kFields = 9;
// group-array strides and field offsets, in floats (nft.cpp:134-178)
constexpr uint32_t kRow = kFields * kLanes;   // NftRow: f[9][8]
constexpr uint32_t kHot = 4 * kLanes;         // NftCellHot: c, kT, bT, ko
constexpr uint32_t kHotC = 0, kHotKT = 8, kHotBT = 16, kHotKO = 24;
constexpr uint32_t kCold = 80;                // NftCellCold: vol_L f64[8] (16 floats), inv_v, kw, kr, ge, ev, depth, phi, vel
constexpr uint32_t kColdKW = 24, kColdKR = 32, kColdGE = 40, kColdEV = 48;
constexpr uint32_t kSite = 288;               // NftSiteRow, 1,152 B
constexpr uint32_t kSiteDrop = 16, kSiteRemoved = 216;
constexpr uint32_t kFieldT = 0, kFieldDO = 1;
constexpr uint32_t kMaxRuns = 128;            // runs per channel: 8 x 128 = 1,024 threads

// f32 arithmetic with an explicit denormal mode: kFtz = the reference's x86 mode.
template <bool kFtz>
struct F32 {
    static __device__ __forceinline__ float add(float a, float b) {
        float r;
        if constexpr (kFtz) asm("add.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        else asm("add.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        return r;
    }
    static __device__ __forceinline__ float sub(float a, float b) {
        float r;
        if constexpr (kFtz) asm("sub.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        else asm("sub.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        return r;
    }
    static __device__ __forceinline__ float mul(float a, float b) {
        float r;
        if constexpr (kFtz) asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        else asm("mul.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        return r;
    }
    // a * b + c, one rounding (lane_fmadd)
    static __device__ __forceinline__ float fma(float a, float b, float c) {
        float r;
        if constexpr (kFtz) asm("fma.rn.ftz.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
        else asm("fma.rn.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
        return r;
    }
    // c - a * b, one rounding (lane_fnmadd: the product's sign flipped, then fused)
    static __device__ __forceinline__ float fnma(float a, float b, float c) { return fma(-a, b, c); }
    // lane_max for f32: a > b ? a : b (the comparison sees the denormal mode)
    static __device__ __forceinline__ float max(float a, float b) {
        uint32_t gt;
        if constexpr (kFtz) asm("{ .reg .pred p; setp.gt.ftz.f32 p, %1, %2; selp.u32 %0, 1, 0, p; }" : "=r"(gt) : "f"(a), "f"(b));
        else asm("{ .reg .pred p; setp.gt.f32 p, %1, %2; selp.u32 %0, 1, 0, p; }" : "=r"(gt) : "f"(a), "f"(b));
        return gt ? a : b;
    }
};

// O2 saturation in fresh water at 1 atm, mg/L (nft.cpp:491-497): the f64 coefficients
// rounded to f32, Horner with fused steps.
template <bool kFtz>
__device__ __forceinline__ float do_sat(float T) {
    using F = F32<kFtz>;
    return F::fma(F::fma(F::fma((float)-0.000077774, T, (float)0.007991), T, (float)-0.41022), T, (float)14.652);
}

// The plant site on cell j, as the reference's sweep finds it: it counts sites down from
// the last site row (site_offset + (sites - 1) * stride) and only matches a row equal to
// the next one, so when that last row lies beyond the channel no site is ever applied.
__device__ __forceinline__ int site_on(uint32_t j, const GpuNftTransport &t) {
    if (t.sites_count == 0) return -1;
    const uint32_t last = t.site_offset + (t.sites_count - 1) * t.site_stride;
    if (last >= t.cells) return -1;
    if (t.site_stride == 0) return j == t.site_offset ? (int)t.sites_count - 1 : -1;
    if (j < t.site_offset || (j - t.site_offset) % t.site_stride) return -1;
    const uint32_t s = (j - t.site_offset) / t.site_stride;
    return s < t.sites_count ? (int)s : -1;
}

template <bool kFtz>
__global__ void __launch_bounds__(1024) nft_transport_kernel(const __grid_constant__ GpuNftTransport t, uint32_t run_len) {
    using F = F32<kFtz>;
    extern __shared__ float boundary[];   // [2][runs][9][8]: the old state of each run's last cell
    const uint32_t g = blockIdx.x;
    const uint32_t l = threadIdx.x & (kLanes - 1), q = threadIdx.x / kLanes;
    const uint32_t runs = blockDim.x / kLanes;
    const uint32_t cells = t.cells;
    const uint32_t j0 = q * run_len;
    const uint32_t j1 = min(cells, j0 + run_len);
    float *rows = t.rows + (size_t)g * cells * kRow + l;
    float *hot = t.hot + (size_t)g * cells * kHot + l;
    const float *cold = t.cold + (size_t)g * cells * kCold + l;
    float *sites = t.sites + (size_t)g * t.sites_count * kSite + l;

    // this window's heat coefficients, linear in the cell temperature delta (nft.cpp:1036-1047)
    const float tamb_rel = F::sub(t.T_amb, t.ref[kFieldT]);
    for (uint32_t j = j0; j < j1; ++j) {
        const float kw = cold[(size_t)j * kCold + kColdKW];
        const float ge = cold[(size_t)j * kCold + kColdGE];
        const float kr = cold[(size_t)j * kCold + kColdKR];
        hot[(size_t)j * kHot + kHotKT] = F::fma(ge, t.es_slope, kw);
        hot[(size_t)j * kHot + kHotBT] = F::fnma(ge, t.e0, F::fma(kw, tamb_rel, F::mul(kr, t.radiant)));
    }
    float floor_[kFields];
    for (uint32_t k = 0; k < kFields; ++k) floor_[k] = -t.ref[k];
    const float refT = t.ref[kFieldT], refDO = t.ref[kFieldDO];
    float out[kFields];
    for (uint32_t k = 0; k < kFields; ++k) out[k] = 0.0f;
    const bool owns_last = j0 < j1 && j1 == cells;

    for (uint32_t s = 0; s < t.substeps; ++s) {
        float *pub = boundary + ((s & 1) * runs + q) * kRow + l;
        float v[kFields];
        if (j0 < j1) {
            const float *last = rows + (size_t)(j1 - 1) * kRow;
            for (uint32_t k = 0; k < kFields; ++k) {
                v[k] = last[k * kLanes];
                pub[k * kLanes] = v[k];
            }
            if (owns_last)
                for (uint32_t k = 0; k < kFields; ++k) out[k] = F::add(out[k], v[k]);
        }
        __syncthreads();
        const float *upstream_run = boundary + ((s & 1) * runs + (q ? q - 1 : 0)) * kRow + l;
        for (uint32_t j = j1; j-- > j0;) {
            float *row = rows + (size_t)j * kRow;
            const float *h = hot + (size_t)j * kHot;
            const float c = h[kHotC];
            float x[kFields], up[kFields];
            if (j > 0) {
                if (j > j0) {
                    const float *u = row - kRow;
                    for (uint32_t k = 0; k < kFields; ++k) up[k] = u[k * kLanes];
                } else {
                    for (uint32_t k = 0; k < kFields; ++k) up[k] = upstream_run[k * kLanes];
                }
                for (uint32_t k = 0; k < kFields; ++k) x[k] = F::fma(c, F::sub(up[k], v[k]), v[k]);
            } else {
                for (uint32_t k = 0; k < kFields; ++k) x[k] = F::fnma(c, v[k], v[k]);   // inflow delta is 0
            }
            // heat: walls, radiant load, evaporative cooling of the open surface
            x[kFieldT] = F::add(F::fnma(h[kHotKT], x[kFieldT], x[kFieldT]), h[kHotBT]);
            // O2 exchange with the gully air (saturation at the absolute temperature)
            x[kFieldDO] = F::fma(h[kHotKO], F::sub(do_sat<kFtz>(F::add(refT, x[kFieldT])), F::add(refDO, x[kFieldDO])),
                                 x[kFieldDO]);
            // plant site: uptake and root respiration, booked as what was actually removed
            const int site = site_on(j, t);
            if (site >= 0) {
                float *sr = sites + (size_t)site * kSite;
                for (uint32_t k = 1; k < kFields; ++k) {
                    const float before = x[k];
                    x[k] = F::max(F::sub(x[k], sr[kSiteDrop + k * kLanes]), floor_[k]);
                    sr[kSiteRemoved + k * kLanes] = F::add(sr[kSiteRemoved + k * kLanes], F::sub(before, x[k]));
                }
            }
            for (uint32_t k = 0; k < kFields; ++k) row[k * kLanes] = x[k];
            if (j > j0)
                for (uint32_t k = 0; k < kFields; ++k) v[k] = up[k];
        }
    }
    if (owns_last)
        for (uint32_t k = 0; k < kFields; ++k) t.out_sum[(size_t)g * kRow + k * kLanes + l] = out[k];
    __syncthreads();
    // water evaporated from the film this window, summed inlet -> outlet (nft.cpp:1101-1105)
    if (q == 0) {
        float evap = 0.0f;
        for (uint32_t j = 0; j < cells; ++j)
            evap = F::fma(cold[(size_t)j * kCold + kColdEV], F::fma(t.es_slope, rows[(size_t)j * kRow + kFieldT * kLanes], t.e0), evap);
        t.evap_kg[(size_t)g * kLanes + l] = F::mul(evap, (float)t.substeps);
    }
}

// Runs per channel and cells per run: as many runs as a 1,024-thread CTA holds, then
// runs of equal length (the last may be shorter).
void launch_shape(uint32_t cells, uint32_t *runs, uint32_t *run_len) {
    const uint32_t len = (cells + kMaxRuns - 1) / kMaxRuns;
    *run_len = len;
    *runs = (cells + len - 1) / len;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

}   // namespace

SGB_API int32_t gpu_nft_transport(const GpuNftTransport *t, float *kernel_ms) {
    if (!t || !t->rows || !t->hot || !t->cold || !t->out_sum || !t->evap_kg) return (int32_t)cudaErrorInvalidValue;
    if (t->groups == 0 || t->cells == 0 || (t->sites_count && !t->sites)) return (int32_t)cudaErrorInvalidValue;
    if (t->groups > 0x7fffffffu) return (int32_t)cudaErrorInvalidValue;
    // the reference's last site row is a u32: refuse layouts where it would wrap
    if (t->sites_count && (uint64_t)t->site_offset + (uint64_t)(t->sites_count - 1) * t->site_stride > 0xffffffffull)
        return (int32_t)cudaErrorInvalidValue;
    if (!aligned16(t->rows) || !aligned16(t->hot) || !aligned16(t->cold) || (t->sites && !aligned16(t->sites)))
        return (int32_t)cudaErrorInvalidValue;
    uint32_t runs = 0, run_len = 0;
    launch_shape(t->cells, &runs, &run_len);
    const uint32_t threads = runs * kLanes;
    const size_t smem = (size_t)2 * runs * kRow * sizeof(float);
    auto kernel = t->flush_denormals ? nft_transport_kernel<true> : nft_transport_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int32_t)e;
    e = module_mark_start();
    if (e != cudaSuccess) return (int32_t)e;
    kernel<<<t->groups, threads, smem, module_stream()>>>(*t, run_len);
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int32_t)e;
    return (int32_t)module_finish(kernel_ms);
}
