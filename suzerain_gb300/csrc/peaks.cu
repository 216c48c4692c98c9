// Pipe-throughput microbenchmarks: the denominators that the factor and
// residual kernels are compared with (FP64 FMA, FP32 FMA, packed FP32 FMA,
// shared-memory load bandwidth), measured on the device the library runs on.
// Each kernel keeps eight independent chains per thread so that the pipe,
// not the dependency latency, bounds it; the results are stored only if they
// equal a value no chain reaches, which keeps the work from being removed.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_common.cuh"

#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void k_fma_chain(int iters, T a, T b, T *sink)
{
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (T) (threadIdx.x + c);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == (T) -1.2345e-7) sink[threadIdx.x] = s;
}

__global__ void k_ffma2_chain(int iters, float a, float b, float *sink)
{
    float2 x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = make_float2((float) threadIdx.x + c, (float) c);
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = ffma2(x[c], a2, b2);
    float s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c].x + x[c].y;
    if (s == -1.2345e-7f) sink[threadIdx.x] = s;
}

// 64-bit shared-memory loads, conflict-free (consecutive lanes, consecutive
// words), eight independent loads in flight per thread.
__global__ void k_smem_ld(int iters, float2 *sink)
{
    __shared__ float2 buf[2048];
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) buf[i] = make_float2((float) i, 0.f);
    __syncthreads();
    float2 acc = make_float2(0.f, 0.f);
    int base = threadIdx.x & 255;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) {
            const float2 v = buf[(base + 256 * c) & 2047];
            acc.x += v.x;
            acc.y += v.y;
        }
        base = (base + 32) & 255;
    }
    if (acc.x == -1.2345e-7f) sink[threadIdx.x] = acc;
}

template <typename Launch>
float time_ms(Launch launch, cudaStream_t st)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch();                    // warm-up
    cudaEventRecord(e0, st);
    launch();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

}  // namespace

// out[0] FP64 FMA TFLOP/s, out[1] FP32 FMA TFLOP/s, out[2] packed FP32 FMA
// TFLOP/s, out[3] shared-memory load bandwidth TB/s, out[4] the same in bytes
// per SM per SM clock (with out[5] = the SM clock in MHz the device reports
// as its maximum), out[6] SM count.
extern "C" int sgb_measure_peaks(double *out, void *stream)
{
    if (!out) return -1;
    cudaStream_t st = (cudaStream_t) stream;
    int dev = 0, sms = 0, clk_khz = 0;
    SGB_CUDA_TRY(cudaGetDevice(&dev));
    SGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SGB_CUDA_TRY(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev));
    void *sink = nullptr;
    SGB_CUDA_TRY(cudaMalloc(&sink, 1 << 16));
    const int threads = 256, blocks = sms * 8;
    const double nthr = (double) threads * blocks;

    const int it64 = 4096, it32 = 65536;
    const float t64 = time_ms([&] { k_fma_chain<double><<<blocks, threads, 0, st>>>(it64, 0.999, 1e-3, (double *) sink); }, st);
    const float t32 = time_ms([&] { k_fma_chain<float><<<blocks, threads, 0, st>>>(it32, 0.999f, 1e-3f, (float *) sink); }, st);
    const float t2 = time_ms([&] { k_ffma2_chain<<<blocks, threads, 0, st>>>(it32, 0.999f, 1e-3f, (float *) sink); }, st);
    const int itsm = 16384;
    const float tsm = time_ms([&] { k_smem_ld<<<blocks, threads, 0, st>>>(itsm, (float2 *) sink); }, st);
    cudaError_t e = cudaGetLastError();
    cudaFree(sink);
    if (e != cudaSuccess) return sgb_set_error(e, "sgb_measure_peaks", __FILE__, __LINE__);

    out[0] = 2.0 * kChains * it64 * nthr / (t64 * 1e-3) / 1e12;
    out[1] = 2.0 * kChains * it32 * nthr / (t32 * 1e-3) / 1e12;
    out[2] = 4.0 * kChains * it32 * nthr / (t2 * 1e-3) / 1e12;
    const double smem_bytes = 8.0 * kChains * itsm * nthr;
    out[3] = smem_bytes / (tsm * 1e-3) / 1e12;
    out[5] = clk_khz / 1e3;
    out[4] = smem_bytes / (tsm * 1e-3) / sms / (clk_khz * 1e3);
    out[6] = sms;
    return 0;
}
