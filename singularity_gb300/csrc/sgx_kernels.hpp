// singularity_gb300/csrc/sgx_kernels.hpp
//
// Internal launch interface between the C-ABI layer (sgx_api.cu) and the
// kernels (sgx_trace.cu).  Not installed; no CUDA types leak past the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "sgx.h"

namespace sgxk {

// Device counters of one pass, reduced per warp then added with atomics.
struct PassCounters {
    unsigned long long next_ray;     // work queue head
    unsigned long long steps;        // integrator steps (accepted + rejected)
    unsigned long long rejected;     // adaptive rejections
    unsigned long long zone_steps;   // mixed-form FP64-controlled steps
    unsigned long long budget_hits;  // rays that exhausted max_steps
    unsigned long long rays;         // rays traced
    unsigned long long pad[2];
};

// One pass of the trace: samples [s0, s0 + S) of every pixel of one view.
struct PassDesc {
    std::uint64_t total_rays;  // npix * S
    std::uint32_t npix;
    std::uint32_t S;
    std::uint32_t s0;
    std::uint32_t refill;       // steps between refills
    void* results;              // [S][npix] hit records, record_bytes(precision) each
    PassCounters* counters;
    // adaptive options
    float tol, h_init_frac, h_max_frac, zone;
};

struct LaunchShape {
    int block_threads;
    int blocks_per_sm;
};

// Prepares the per-view constants (device) from a device copy of the uniforms.
cudaError_t launch_setup_view(const sgx_uniforms* d_u, void* d_view, int precision, cudaStream_t st);

// Persistent tracer.  precision: sgx_precision; integrator: sgx_integrator.
cudaError_t launch_trace(const void* d_view, int metric, int precision, int integrator, bool fast_math,
                         const PassDesc& pass, LaunchShape shape, cudaStream_t st);

// Per-sample probe (parity tests): n samples, device arrays.
cudaError_t launch_probe(const void* d_view, int metric, int precision, int integrator, bool fast_math,
                         std::uint64_t n, const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s,
                         float* hdr3, std::uint32_t* steps, std::uint32_t* term, float tol, float h_init_frac,
                         float h_max_frac, float zone, cudaStream_t st);

// Shades the pass's hit records and adds them in sample order into acc
// (float4 per pixel); when `finalize`, also writes the frame in `format` to
// out (scale = 1/spp).
cudaError_t launch_accumulate(const void* d_view, int precision, const void* results, float4* acc,
                              std::uint32_t npix, std::uint32_t S, bool first, bool finalize, float scale,
                              std::uint32_t format, void* out, cudaStream_t st);

// Bytes of one hit record (16 for FP32 and mixed, 32 for FP64).
std::size_t record_bytes(int precision);

// Samples one pass may hold (the per-block offset table).
constexpr std::uint32_t kMaxPassSamplesHost = 1024;

// Re-encodes the accumulated frame (acc, float4 mean-sum) in another format.
cudaError_t launch_encode(const float4* acc, std::uint32_t npix, float scale, std::uint32_t format, void* out,
                          cudaStream_t st);

std::size_t view_bytes();

}  // namespace sgxk
