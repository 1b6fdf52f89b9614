/*
 * k_probe.cu - FP32 and FP64 FMA throughput probes (the roofline denominators
 * for the pair kernels).
 *
 * Each thread runs 8 independent FMA chains (scalar FFMA, packed FFMA2 for
 * FP32; DFMA for FP64) for a fixed number of iterations; the grid fills every
 * SM several times over.  FLOP/s = 2 * FMAs / CUDA-event time.  Thread 0 of
 * block 0 also reads clock64() at both ends, which gives the SM clock the
 * probe ran at.
 */
#include <cstdio>

#include "nbg_internal.cuh"

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c);
template <>
__device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <>
__device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T *out, int iters, T a, T b, ll *cycles)
{
    ll c0 = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) c0 = clock64();
    T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = fma_t(x0, a, b);
            x1 = fma_t(x1, a, b);
            x2 = fma_t(x2, a, b);
            x3 = fma_t(x3, a, b);
            x4 = fma_t(x4, a, b);
            x5 = fma_t(x5, a, b);
            x6 = fma_t(x6, a, b);
            x7 = fma_t(x7, a, b);
        }
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    if (blockIdx.x == 0 && threadIdx.x == 0) *cycles = clock64() - c0;
}

__global__ void __launch_bounds__(256) k_ffma2_probe(float *out, int iters, float a, float b, ll *cycles)
{
    ll c0 = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) c0 = clock64();
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
    float2 x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = make_float2(threadIdx.x * 1e-3f + k, threadIdx.x * 2e-3f + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
#pragma unroll
            for (int k = 0; k < 8; k++) x[k] = __ffma2_rn(x[k], a2, b2);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k].x + x[k].y;
    if (s == -12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    if (blockIdx.x == 0 && threadIdx.x == 0) *cycles = clock64() - c0;
}

/* one warp, one long dependent chain: SM clock = cycles / event time */
__global__ void k_clock_probe(float *out, int iters, ll *cycles)
{
    const ll c0 = clock64();
    float x = threadIdx.x * 1e-3f;
    for (int i = 0; i < iters; i++) x = fmaf(x, 0.999f, 0.001f);
    const ll c1 = clock64();
    if (x == -1.0f) out[threadIdx.x] = x;
    if (threadIdx.x == 0) *cycles = c1 - c0;
}

int nbg_run_probes(int device, double *fp32, double *fp64, double *mhz)
{
    if (cudaSetDevice(device) != cudaSuccess) return NBG_E_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256;
    float *of = nullptr;
    double *od = nullptr;
    ll *cyc = nullptr;
    if (cudaMalloc(&of, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return NBG_E_CUDA;
    if (cudaMalloc(&od, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return NBG_E_CUDA;
    if (cudaMalloc(&cyc, sizeof(ll)) != cudaSuccess) return NBG_E_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    /* warm up */
    k_fma_probe<float><<<blocks, threads>>>(of, 64, 0.999f, 0.001f, cyc);
    cudaDeviceSynchronize();
    double best32 = 0, best64 = 0, clk = 0;
    for (int rep = 0; rep < 3; rep++) {
        const int it32 = 4096;
        cudaEventRecord(e0);
        k_fma_probe<float><<<blocks, threads>>>(of, it32, 0.999f, 0.001f, cyc);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ll c = 0;
        cudaMemcpy(&c, cyc, sizeof c, cudaMemcpyDeviceToHost);
        double fl = 2.0 * 8 * 16 * (double)it32 * blocks * threads / (ms * 1e-3);
        if (fl > best32) best32 = fl;
        (void)c;

        cudaEventRecord(e0);
        k_ffma2_probe<<<blocks, threads>>>(of, it32 / 2, 0.999f, 0.001f, cyc);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        fl = 2.0 * 2 * 8 * 8 * (double)(it32 / 2) * blocks * threads / (ms * 1e-3);
        if (fl > best32) best32 = fl;

        const int it64 = 64;
        cudaEventRecord(e0);
        k_fma_probe<double><<<blocks, threads>>>(od, it64, 0.999, 0.001, cyc);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        fl = 2.0 * 8 * 16 * (double)it64 * blocks * threads / (ms * 1e-3);
        if (fl > best64) best64 = fl;

        cudaEventRecord(e0);
        k_clock_probe<<<1, 32>>>(of, 1 << 22, cyc);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        ll cc = 0;
        cudaMemcpy(&cc, cyc, sizeof cc, cudaMemcpyDeviceToHost);
        const double m = (double)cc / (ms * 1e3);
        if (m > clk) clk = m;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(of);
    cudaFree(od);
    cudaFree(cyc);
    if (err != cudaSuccess) return NBG_E_CUDA;
    if (fp32) *fp32 = best32;
    if (fp64) *fp64 = best64;
    if (mhz) *mhz = clk;
    return NBG_OK;
}
