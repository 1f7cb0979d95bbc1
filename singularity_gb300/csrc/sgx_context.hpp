// singularity_gb300/csrc/sgx_context.hpp
//
// Internal definition of the C ABI's opaque sgx_context (shared by the
// single-view entry points in sgx_api.cu and the batch entry points in
// sgx_batch.cu).  Not installed.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "sgx.h"
#include "sgx_kernels.hpp"

struct sgx_diff_state;  // differentiable form (sgx_diff.cu)

struct sgx_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::uint32_t width = 0, height = 0;
    void* d_image = nullptr;       // npix * 16 bytes
    float4* d_acc = nullptr;       // npix
    void* d_results = nullptr;     // results_cap bytes (hit records)
    std::size_t results_cap = 0;
    void* d_view = nullptr;            // kMaxLaunchViews view slots
    sgx_uniforms* d_u = nullptr;       // kMaxLaunchViews uniform blocks
    std::uint64_t* d_words = nullptr;  // view-set layout words
    sgxk::PassCounters* d_counters = nullptr;
    sgxk::PassCounters* h_counters = nullptr;  // pinned
    void* h_view = nullptr;            // pinned host copy of view slot 0 (single-view tracer parameter)
    sgx_uniforms h_view_u{};           // ... made from these uniforms
    int h_view_precision = -1;         // ... at this precision (-1: none yet)
    cudaEvent_t ev_begin = nullptr, ev_trace0 = nullptr, ev_trace1 = nullptr, ev_end = nullptr;
    bool frame_valid = false;     // accumulator holds a complete frame
    std::uint32_t frame_spp = 0;
    std::uint32_t frame_format = SGX_FORMAT_RGBA8_SRGB;
    std::uint32_t next_sample = 0;  // progressive passes: next expected sample
    std::size_t workspace_budget = std::size_t(4) << 30;
    sgx_render_stats stats{};
    std::string err;
    sgx_uniforms last_u{};        // uniforms of the last render (bloom reads exposure, threshold, strength)
    void* d_bloom = nullptr;      // two half-resolution half4 targets
    std::size_t bloom_cap = 0;    // bytes of one target
    bool bloom_ext_valid = false; // the first target holds the extract the last HDR render fused in ...
    float bloom_ext_threshold = 0.0f;  // ... at this threshold
    void* d_post = nullptr;       // composed frame after sgx_bloom (16 B / pixel)
    bool post_valid = false;
    std::uint32_t post_format = SGX_FORMAT_RGBA8_SRGB;
    sgx_diff_state* diff = nullptr;  // forward records of sgx_diff_forward
};

// Releases the differentiable form's buffers (defined in sgx_diff.cu).
void sgx_internal_free_diff(sgx_context* ctx);


namespace sgx_internal {
// The two half-resolution bloom targets of a W x H frame (sgx_post.cu).
sgx_status ensure_bloom_targets(sgx_context* ctx, std::uint32_t W, std::uint32_t H);
inline sgx_status fail(sgx_context* ctx, sgx_status s, const std::string& msg) {
    if (ctx != nullptr) ctx->err = msg;
    return s;
}
inline sgx_status cuda_fail(sgx_context* ctx, cudaError_t e, const char* where) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? SGX_ERR_OUT_OF_MEMORY : SGX_ERR_CUDA,
                std::string(where) + ": " + cudaGetErrorString(e));
}
// Validates and completes render options (defaults for absent fields).
sgx_status resolve_and_check(sgx_context* ctx, const sgx_render_opts* in, sgx_render_opts& out);
}  // namespace sgx_internal
