// Instruction-throughput probes: the measured peaks that the roofline of the
// integrator is reported against (FP64 FMA for the plain path, FP32 FMA for the
// mixed path's chemistry, and the FP64<->FP32 conversions the mixed path adds).
// Each thread runs 8 independent dependency chains so the pipe, not latency,
// bounds the loop.

#include <cuda_runtime.h>
#include <stdint.h>

namespace sgb {

template <int KIND>
__global__ void __launch_bounds__(256) probe_kernel(double *out, uint32_t iters) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (KIND == 0 || KIND == 3 || KIND == 4 || KIND == 5) {
        double a[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = 1.0 + 1e-3 * (double)(tid % 97 + j);
        const double b = 0.9999999, c = 1e-7;
        for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (KIND == 0) a[j] = fma(a[j], b, c);
                if (KIND == 3) a[j] = a[j] + c;
                if (KIND == 4) a[j] = 1.0 / a[j];
                if (KIND == 5) a[j] = sqrt(a[j]);
            }
        }
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < 8; ++j) s += a[j];
        out[tid] = s;
    } else if (KIND == 1) {
        float a[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = 1.0f + 1e-3f * (float)(tid % 97 + j);
        const float b = 0.9999999f, c = 1e-7f;
        for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
            for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], b, c);
        }
        float s = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) s += a[j];
        out[tid] = (double)s;
    } else {   // KIND 2: f32 -> f64 -> f32 conversion round trips (2 conversions per op)
        float a[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = 1.0f + 1e-3f * (float)(tid % 97 + j);
        for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                double d = (double)a[j];
                a[j] = __int_as_float(__double2hiint(d) ^ (int)j) ;
            }
        }
        float s = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) s += a[j];
        out[tid] = (double)s;
    }
}

// kind: 0 DFMA, 1 FFMA, 2 F2F pair (f32->f64, f64->f32; plus one DMUL and one FMUL),
// 3 DADD, 4 FP64 reciprocal (1.0 / x, IEEE), 5 FP64 sqrt. Returns operations per
// second (an FMA counts as one operation) over the whole device.
cudaError_t run_probe(uint32_t kind, int sms, cudaStream_t stream, double *ops_per_s) {
    const uint32_t block = 256, grid = (uint32_t)sms * 8;
    const uint32_t iters = (kind == 1) ? 1u << 16 : (kind == 4 || kind == 5) ? 1u << 9 : 1u << 12;
    double *out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(double) * grid * block);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(a, stream);
        switch (kind) {
            case 0: probe_kernel<0><<<grid, block, 0, stream>>>(out, iters); break;
            case 1: probe_kernel<1><<<grid, block, 0, stream>>>(out, iters); break;
            case 2: probe_kernel<2><<<grid, block, 0, stream>>>(out, iters); break;
            case 3: probe_kernel<3><<<grid, block, 0, stream>>>(out, iters); break;
            case 4: probe_kernel<4><<<grid, block, 0, stream>>>(out, iters); break;
            default: probe_kernel<5><<<grid, block, 0, stream>>>(out, iters); break;
        }
        cudaEventRecord(b, stream);
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;   // first run warms up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return e;
    *ops_per_s = (double)grid * block * 8.0 * iters / (best * 1e-3);
    return cudaGetLastError();
}

}   // namespace sgb
