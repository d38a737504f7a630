// fp64_peak.cu — measures the sustained FP64 instruction rate of the current
// GPU (the roofline denominator of the FP64-bound kernels of this library).
//
// Every thread runs 8 independent chains of FP64 FMA (or ADD, MUL) so that
// the pipe, not latency, bounds the loop; 8 CTAs of 256 threads per SM.
// Output (stdout, one JSON line): G thread-instructions per second for each
// operation and the TFLOP/s of FMA counted as 2 flops.
#include <cstdio>

#include <cuda_runtime.h>

namespace {

constexpr int kIter = 4096;

template <int OP>
__global__ void chains(double *out, double a, double b) {
    double x[8];
#pragma unroll
    for(int c = 0; c < 8; c++) x[c] = threadIdx.x * 1e-3 + c;
#pragma unroll 16
    for(int i = 0; i < kIter; i++) {
#pragma unroll
        for(int c = 0; c < 8; c++) {
            if(OP == 0) x[c] = fma(x[c], a, b);
            if(OP == 1) x[c] = x[c] + b;
            if(OP == 2) x[c] = x[c] * a;
        }
    }
    double r = 0;
#pragma unroll
    for(int c = 0; c < 8; c++) r += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

template <int OP>
double rate(double *d, int blocks, int threads) {
    chains<OP><<<blocks, threads>>>(d, 0.999999, 1e-9);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    const int reps = 5;
    for(int r = 0; r < reps; r++) chains<OP><<<blocks, threads>>>(d, 0.999999, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return (double) reps * blocks * threads * kIter * 8.0 / (ms * 1e-3) / 1e9;
}

}  // namespace

int main() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int blocks = sms * 8, threads = 256;
    double *d = nullptr;
    if(cudaMalloc(&d, sizeof(double) * (size_t) blocks * threads) != cudaSuccess) {
        std::printf("{\"error\": \"cudaMalloc failed\"}\n");
        return 1;
    }
    double fma_r = rate<0>(d, blocks, threads);
    double add_r = rate<1>(d, blocks, threads);
    double mul_r = rate<2>(d, blocks, threads);
    cudaError_t e = cudaGetLastError();
    cudaFree(d);
    if(e != cudaSuccess) {
        std::printf("{\"error\": \"%s\"}\n", cudaGetErrorString(e));
        return 1;
    }
    std::printf("{\"dfma_ginst_s\": %.2f, \"dadd_ginst_s\": %.2f, \"dmul_ginst_s\": %.2f, \"fma_tflops\": %.4f, "
                "\"sms\": %d}\n",
                fma_r, add_r, mul_r, 2.0 * fma_r / 1e3, sms);
    return 0;
}
