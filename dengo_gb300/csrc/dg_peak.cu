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
