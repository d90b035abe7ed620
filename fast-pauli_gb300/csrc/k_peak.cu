// k_peak.cu -- fpg_measure_peak: the float32 / float64 fused multiply-add
// rate of the current device, measured.
//
// The float64 expectation stage runs in double-float arithmetic on the
// float32 pipes, so its binding roof is the rate at which the SMs issue
// float32 FMA-pipe instructions; the float64 forms are bound by the float64
// pipe.  Neither rate is in the HBM / tensor-core peaks a benchmark is
// usually given, so this entry point measures them with a kernel of
// independent FMA chains (8 per thread, 256 threads, 8 CTAs per SM): every
// issue slot of the FMA pipe does useful work, as in a throughput
// microbenchmark.  The result counts lane operations (one FMA = 1) per second.
#include "fpg.h"

#include "common.cuh"
#include "host_internal.hpp"

namespace fpg
{
namespace
{

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_fma_rate(int iters, T a, T b, T *__restrict__ sink)
{
    T v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        v[c] = (T)(threadIdx.x + c) * (T)1e-3;
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int k = 0; k < 16; ++k)
#pragma unroll
            for (int c = 0; c < kChains; ++c)
                v[c] = v[c] * a + b; // one fused multiply-add per chain (contracted by nvcc)
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += v[c];
    if (s == (T)-1.2345) // never true for these inputs; keeps the chains live
        sink[threadIdx.x] = s;
}

} // namespace
} // namespace fpg

using namespace fpg;

extern "C" int fpg_measure_peak(int32_t dtype, double *fma_per_s, void *stream)
{
    if (!fma_per_s)
        return set_error(FPG_ERR_INVALID, "fma_per_s is null");
    if (dtype != FPG_C128 && dtype != FPG_C64)
        return set_error(FPG_ERR_INVALID, "dtype must be FPG_C128 (float64) or FPG_C64 (float32)");
    cudaStream_t st = (cudaStream_t)stream;
    const bool f32 = dtype == FPG_C64;
    const unsigned blocks = (unsigned)sm_count() * 8;
    const int iters = f32 ? 4096 : 128; // ~10 ms of float32 work; float64 runs at 1/64 of it
    void *sink = nullptr;
    if (int rc = fpg_device_alloc(&sink, 256 * sizeof(double), stream))
        return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    float best_ms = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) // first run warms up; keep the fastest
    {
        if ((e = cudaEventRecord(e0, st)))
            break;
        if (f32)
            k_fma_rate<float><<<blocks, 256, 0, st>>>(iters, 0.999f, 1e-4f, (float *)sink);
        else
            k_fma_rate<double><<<blocks, 256, 0, st>>>(iters, 0.999, 1e-4, (double *)sink);
        if ((e = launched()) || (e = cudaEventRecord(e1, st)) || (e = cudaEventSynchronize(e1)))
            break;
        float ms = 0.f;
        if ((e = cudaEventElapsedTime(&ms, e0, e1)))
            break;
        if (rep > 0 && (best_ms == 0.f || ms < best_ms))
            best_ms = ms;
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    fpg_device_free(sink, stream);
    if (e != cudaSuccess)
        return cuda_error(e, "fpg_measure_peak");
    const double ops = (double)blocks * 256.0 * (double)iters * 16.0 * kChains;
    *fma_per_s = best_ms > 0.f ? ops / (best_ms * 1e-3) : 0.0;
    return FPG_OK;
}
