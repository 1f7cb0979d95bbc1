// singularity_gb300/csrc/sgx_probe.cu
//
// Measurement helper, no counterpart in the reference: the FP32 FMA issue
// ceiling of the device, measured with a register-resident kernel (eight
// independent FMA chains per thread, so the pipe, not latency, is the limit).
// bench.py divides the tracer's algorithmic FLOP rate by this number.

#include <cuda_runtime.h>

#include "sgx.h"

namespace {

__global__ void __launch_bounds__(256) fma_ceiling_kernel(float* out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" sgx_status sgx_measure_fp32_peak(int device, int iters, double* tflops) {
    if (tflops == nullptr || iters <= 0) return SGX_ERR_INVALID_ARGUMENT;
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return SGX_ERR_CUDA;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float* out = nullptr;
    const int threads = 256, blocks = sms * 8;
    if (cudaMalloc(&out, size_t(blocks) * threads * sizeof(float)) != cudaSuccess) return SGX_ERR_OUT_OF_MEMORY;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_ceiling_kernel<<<blocks, threads>>>(out, iters / 8 + 1, 1.0f);  // warm-up
    cudaEventRecord(e0);
    fma_ceiling_kernel<<<blocks, threads>>>(out, iters, 1.0f);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return SGX_ERR_CUDA;
    const double flops = double(blocks) * threads * double(iters) * 16.0 * 8.0 * 2.0;
    *tflops = flops / (double(ms) * 1e-3) / 1e12;
    return SGX_OK;
}
