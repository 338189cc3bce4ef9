// msx_fp64_peak.cu -- the FP64 pipe's DFMA rate on this GPU, the denominator
// of the plain FP64 element kernel's pipe roofline (bench.py runs it).  Eight
// independent FMA chains per thread keep the pipe fed; every SM runs 2, 4 and
// 8 CTAs of 256 threads in turn and the best rate is printed as
// "fp64_dfma_gops <value>" (one DFMA counted as one operation, as the
// kernel's FP64 instruction count is).  No memory traffic but the final store.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void dfma_chains(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = threadIdx.x + j;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int r = 0; r < 8; r++)
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
    double s = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main()
{
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess || sms < 1) return 1;
    const int threads = 256, iters = 2000;
    double best = 0;
    for (int per_sm : {2, 4, 8}) {
        const int blocks = sms * per_sm;
        double *out = nullptr;
        if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return 1;
        dfma_chains<<<blocks, threads>>>(out, 10, 0.999999, 1e-7);   // warm-up
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0);
        dfma_chains<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const double ops = (double)blocks * threads * iters * 64;
        if (ms > 0 && ops / (ms * 1e-3) / 1e9 > best) best = ops / (ms * 1e-3) / 1e9;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(out);
    }
    if (cudaGetLastError() != cudaSuccess || best <= 0) return 1;
    printf("fp64_dfma_gops %.1f\n", best);
    return 0;
}
