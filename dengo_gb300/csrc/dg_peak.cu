/*
 * CUDA-core FMA throughput of this GPU, the roofline denominator of the
 * solver kernels (their work is scalar FP64/FP32 arithmetic, not tensor-core
 * contractions).  Each thread runs 8 independent FMA chains; the grid fills
 * every SM.  dg_measure_fma_peak() returns TFLOP/s (2 flops per FMA) timed
 * with CUDA events after a warm-up launch.
 */
#include <cuda_runtime.h>

template <class T>
__global__ void __launch_bounds__(256) fma_chains(T *out, int iters, T a, T b)
{
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-1.2345) out[0] = s;   /* keeps the chains live */
}

template <class T>
static int measure(int iters, double *tflops)
{
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int block = 256, grid = nsm * 8;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<grid, block>>>(out, iters / 8 + 1, (T)0.999999, (T)1e-7);
    cudaEventRecord(e0);
    fma_chains<T><<<grid, block>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0) return -1;
    const double flops = 2.0 * 32.0 * (double)iters * block * (double)grid;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return 0;
}

extern "C" int dg_measure_fma_peak(int fp64, int iters, double *tflops)
{
    return fp64 ? measure<double>(iters, tflops) : measure<float>(iters, tflops);
}

/* FP64 issue model: `chains` independent dependent-FMA chains per thread,
 * `warps` warps per SM (one block per SM).  Returns cycles per FMA per warp
 * (clock64 inside the kernel, averaged over warps). */
template <int CH>
__global__ void fma_lat(double *out, long long *cyc, int iters, int active_lanes)
{
    if ((int)(threadIdx.x & 31) >= active_lanes) return;
    double x[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) x[c] = threadIdx.x + c;
    const double a = 0.999999, b = 1e-7;
    const long long t0 = clock64();
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < CH; c++) x[c] = fma(x[c], a, b);
    }
    const long long t1 = clock64();
    double s = 0;
#pragma unroll
    for (int c = 0; c < CH; c++) s += x[c];
    if (s == -1.2345) out[0] = s;
    if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long *)cyc, (unsigned long long)(t1 - t0));
}

extern "C" int dg_measure_fma_latency_lanes(int chains, int warps, int iters, int lanes,
                                            double *cycles_per_fma);

extern "C" int dg_measure_fma_latency(int chains, int warps, int iters, double *cycles_per_fma)
{
    return dg_measure_fma_latency_lanes(chains, warps, iters, 32, cycles_per_fma);
}

/* As above with only `lanes` active lanes per warp. */
extern "C" int dg_measure_fma_latency_lanes(int chains, int warps, int iters, int lanes,
                                            double *cycles_per_fma)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    double *out;
    long long *cyc;
    cudaMalloc(&out, 8);
    cudaMalloc(&cyc, 8);
    cudaMemset(cyc, 0, 8);
    const int threads = 32 * warps;
    switch (chains) {
    case 1: fma_lat<1><<<nsm, threads>>>(out, cyc, iters, lanes); break;
    case 2: fma_lat<2><<<nsm, threads>>>(out, cyc, iters, lanes); break;
    case 4: fma_lat<4><<<nsm, threads>>>(out, cyc, iters, lanes); break;
    default: fma_lat<8><<<nsm, threads>>>(out, cyc, iters, lanes); chains = 8; break;
    }
    long long h = 0;
    cudaMemcpy(&h, cyc, 8, cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    cudaFree(out);
    cudaFree(cyc);
    if (e != cudaSuccess) return -1;
    *cycles_per_fma = (double)h / ((double)nsm * warps) / ((double)iters * chains);
    return 0;
}
