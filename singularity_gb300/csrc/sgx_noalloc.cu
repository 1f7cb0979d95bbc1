// singularity_gb300/csrc/sgx_noalloc.cu
//
// sgx_render_noalloc: a render entry point that allocates nothing.
//
// Who needs it.  Some callers of this library cannot call cudaMalloc, or let
// a library call it for them: host applications (game engines, renderers
// embedded as plug-ins) that reserve all of a GPU's memory for their own pool
// or arena at start-up and forbid third-party allocations after it; and
// frame-paced callers that cannot take the device-wide synchronisation that
// cudaFree implies in the middle of a frame.  The context-based entry points
// (sgx_create / sgx_render / sgx_render_device) allocate their images and
// per-sample buffers, so those callers cannot use them.
//
// How.  The per-sample results, the per-pixel accumulator, the pass counters,
// the uniform block and the per-view constants live in one file-scope device
// array of fixed size, SGX_NOALLOC_SCRATCH_BYTES (64 MiB), that every GPU
// loading this library holds until the process exits.  The caller still
// provides the output buffer.  The same kernels as sgx_render_device run over
// it, so results are identical.
//
// Rules for callers:
//   * A frame needs 4096 + align256(16 * width * height) + R * width * height *
//     spp bytes of scratch (R = 16 for FP32, 32 for FP64; align256 rounds up
//     to a multiple of 256); larger requests are rejected with
//     SGX_ERR_INVALID_ARGUMENT and a message saying so.  spp is the clamped
//     samples per pixel.
//   * The first call on each device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture begins.
//   * Every call shares the one array, which keeps the previous call's
//     contents; each call clears what must start at zero (the counters) and
//     overwrites the rest.  Calls whose GPU work overlaps — two streams, or two
//     host threads — race on the array: keep them on one stream.

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "sgx.h"
#include "sgx_kernels.hpp"

namespace {

constexpr std::size_t kHeaderBytes = 4096;  // counters | uniforms | view constants | view-set words
constexpr std::size_t kCountersOff = 0;
constexpr std::size_t kUniformsOff = 256;
constexpr std::size_t kViewOff = 512;
constexpr std::size_t kWordsOff = 2048;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[SGX_NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

void set_err(char* err, std::size_t len, const char* msg) {
    if (err == nullptr || len == 0) return;
    std::snprintf(err, len, "%s", msg);
}

// Device address of the scratch array for `dev`, looked up once per device
// with that device current (the caller guarantees it is).
sgx_status scratch_address(int dev, unsigned char** out, char* err, std::size_t len) {
    if (dev < 0 || dev >= kMaxDevices) {
        set_err(err, len, "sgx_render_noalloc: device ordinal out of range");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            char buf[256];
            std::snprintf(buf, sizeof(buf), "sgx_render_noalloc: cudaGetSymbolAddress failed: %s",
                          cudaGetErrorString(e));
            set_err(err, len, buf);
            return SGX_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_addr[dev]);
    return SGX_OK;
}

}  // namespace

extern "C" sgx_status sgx_render_noalloc(const sgx_uniforms* u, const sgx_render_opts* opts, void* d_out,
                                         uint32_t format, void* stream, char* err, size_t err_len) {
    static_assert(kViewOff >= kUniformsOff + sizeof(sgx_uniforms), "header layout");
    if (u == nullptr || d_out == nullptr) {
        set_err(err, err_len, "sgx_render_noalloc: uniforms and d_out must not be NULL");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    if (u->width == 0 || u->height == 0 ||
        (u->metric_type != SGX_METRIC_KERR && u->metric_type != SGX_METRIC_SCHWARZSCHILD)) {
        set_err(err, err_len, "sgx_render_noalloc: width/height must be > 0 and metric_type known");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    if (kViewOff + sgxk::view_bytes() > kWordsOff) {
        set_err(err, err_len, "sgx_render_noalloc: internal header layout too small");
        return SGX_ERR_UNSUPPORTED;
    }
    sgx_render_opts o;
    sgx_render_opts_default(&o);
    if (opts != nullptr) {
        const std::size_t n = opts->struct_size == 0 || opts->struct_size > sizeof(o) ? sizeof(o) : opts->struct_size;
        std::memcpy(&o, opts, n);
    }
    if (o.precision != SGX_PRECISION_FP32 && o.precision != SGX_PRECISION_FP64) {
        set_err(err, err_len, "sgx_render_noalloc: precision must be FP32 or FP64 with the fixed-step integrator");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    if (o.integrator != SGX_INTEGRATOR_FIXED || o.rhs_form > 2 ||
        (format != SGX_FORMAT_RGBA8_SRGB && format != SGX_FORMAT_RGBA32F)) {
        set_err(err, err_len, "sgx_render_noalloc: fixed-step integrator and RGBA8/RGBA32F output only");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    if (o.block_threads != 0 && (o.block_threads % 32u != 0 || o.block_threads > 256u)) {
        set_err(err, err_len, "sgx_render_noalloc: block_threads must be 0 or a multiple of 32 up to 256");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    if ((o.tile_w == 0) != (o.tile_h == 0) || o.tile_w > 4096 || o.tile_h > 4096) {
        set_err(err, err_len, "sgx_render_noalloc: tile_w and tile_h must both be 0 or both in [1, 4096]");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    if (o.slice_count > 1u) {
        set_err(err, err_len, "sgx_render_noalloc: renders whole frames only (no frame slices)");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    const std::uint32_t spp = u->supersample < 1u ? 1u : (u->supersample > 1024u ? 1024u : u->supersample);
    if (o.sample_begin != 0 || (o.sample_count != 0 && o.sample_count != spp)) {
        set_err(err, err_len, "sgx_render_noalloc: renders whole frames only (sample_begin 0, all samples)");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    const std::uint64_t npix = std::uint64_t(u->width) * u->height;
    const std::uint64_t rec = sgxk::record_bytes(int(o.precision));
    // the hit records start on a 256-byte boundary (an FP64 record is a
    // 32-byte aligned type, and 16 * npix need not be a multiple of 32)
    const std::uint64_t acc_bytes = (16ull * npix + 255ull) / 256ull * 256ull;
    const std::uint64_t need = kHeaderBytes + acc_bytes + rec * npix * std::uint64_t(spp);
    if (need > SGX_NOALLOC_SCRATCH_BYTES) {
        char buf[320];
        std::snprintf(buf, sizeof(buf),
                      "sgx_render_noalloc: frame needs %llu bytes of scratch (4096 + align256(16*w*h) + "
                      "%llu*w*h*spp) but the fixed scratch holds %llu; use fewer pixels or samples, or the "
                      "allocating entry points",
                      (unsigned long long)need, (unsigned long long)rec,
                      (unsigned long long)SGX_NOALLOC_SCRATCH_BYTES);
        set_err(err, err_len, buf);
        return SGX_ERR_INVALID_ARGUMENT;
    }

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_err(err, err_len, "sgx_render_noalloc: no current CUDA device");
        return SGX_ERR_CUDA;
    }
    unsigned char* base = nullptr;
    sgx_status s = scratch_address(dev, &base, err, err_len);
    if (s != SGX_OK) return s;

    auto* counters = reinterpret_cast<sgxk::PassCounters*>(base + kCountersOff);
    auto* d_u = reinterpret_cast<sgx_uniforms*>(base + kUniformsOff);
    void* d_view = base + kViewOff;
    auto* d_words = reinterpret_cast<std::uint64_t*>(base + kWordsOff);
    auto* acc = reinterpret_cast<float4*>(base + kHeaderBytes);
    void* results = base + kHeaderBytes + acc_bytes;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    sgxk::ViewPlan plan;
    if (!sgxk::plan_views(u, 1, 0, spp, o.tile_w, o.tile_h, plan)) {
        set_err(err, err_len, "sgx_render_noalloc: invalid frame");
        return SGX_ERR_INVALID_ARGUMENT;
    }
    sgxk::PassDesc pass{};
    pass.vs = sgxk::make_view_set(plan, d_view, d_words);
    pass.refill = o.refill_interval == 0 ? sgxk::kDefaultRefill : o.refill_interval;
    pass.results = results;
    pass.counters = counters;
    pass.tol = o.tolerance;
    pass.h_init_frac = o.h_init_frac;
    pass.h_max_frac = o.h_max_frac;
    pass.zone = o.fp64_zone;
    pass.project = o.projection;
    sgxk::LaunchShape shape{int(o.block_threads), int(o.blocks_per_sm)};

    e = cudaMemcpyAsync(d_u, u, sizeof(sgx_uniforms), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_words, plan.words, plan.word_count * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, sizeof(sgxk::PassCounters), st);
    if (e == cudaSuccess) e = sgxk::launch_setup_views(d_u, 1, d_view, int(o.precision), st);
    if (e == cudaSuccess)
        e = sgxk::launch_trace(int(u->metric_type), int(o.precision), int(o.integrator), int(o.rhs_form), pass,
                               shape, st);
    if (e == cudaSuccess)
        e = sgxk::launch_accumulate(int(o.precision), pass.vs, results, acc, true, true, format, d_out, st);
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "sgx_render_noalloc: %s", cudaGetErrorString(e));
        set_err(err, err_len, buf);
        return SGX_ERR_CUDA;
    }
    set_err(err, err_len, "");
    return SGX_OK;
}
