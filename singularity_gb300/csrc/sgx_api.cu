// singularity_gb300/csrc/sgx_api.cu
//
// The C ABI (include/sgx.h) over the kernels in sgx_trace.cu: the
// re-creation of the reference's CudaBackend host side
// (render/cuda/cuda_backend.cu:105-166) as a context object.
//
// Memory: the context owns, for its current size, the output image (16 bytes
// per pixel, enough for every format), a float4 accumulator per pixel, the
// per-sample result buffer of one pass ([S][npix] float4; S chosen so the
// buffer stays under the workspace budget) and the pass counters.  A render
// with more samples than one pass holds runs several passes in sample order.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "sgx.h"
#include "sgx_context.hpp"
#include "sgx_kernels.hpp"

namespace {

using sgx_internal::cuda_fail;
using sgx_internal::fail;

#define SGX_CUDA(ctx, call)                                  \
    do {                                                     \
        cudaError_t e__ = (call);                            \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, #call); \
    } while (0)

void free_image(sgx_context* c) {
    if (c->d_image) cudaFree(c->d_image);
    if (c->d_bloom) cudaFree(c->d_bloom);
    if (c->d_post) cudaFree(c->d_post);
    c->d_bloom = nullptr;
    c->d_post = nullptr;
    c->bloom_cap = 0;
    c->bloom_ext_valid = false;
    c->post_valid = false;
    if (c->d_acc) cudaFree(c->d_acc);
    if (c->d_results) cudaFree(c->d_results);
    c->d_image = nullptr;
    c->d_acc = nullptr;
    c->d_results = nullptr;
    c->results_cap = 0;
    c->width = c->height = 0;
    c->frame_valid = false;
    c->next_sample = 0;
}

sgx_status ensure_size(sgx_context* c, std::uint32_t w, std::uint32_t h) {
    if (w == c->width && h == c->height && c->d_image != nullptr) return SGX_OK;
    free_image(c);
    const std::size_t npix = std::size_t(w) * h;
    SGX_CUDA(c, cudaMalloc(&c->d_image, npix * 16));
    SGX_CUDA(c, cudaMalloc(reinterpret_cast<void**>(&c->d_acc), npix * sizeof(float4)));
    c->width = w;
    c->height = h;
    return SGX_OK;
}

sgx_status ensure_results(sgx_context* c, std::size_t bytes) {
    if (bytes <= c->results_cap) return SGX_OK;
    if (c->d_results) cudaFree(c->d_results);
    c->d_results = nullptr;
    c->results_cap = 0;
    SGX_CUDA(c, cudaMalloc(&c->d_results, bytes));
    c->results_cap = bytes;
    return SGX_OK;
}

sgx_status check_uniforms(sgx_context* c, const sgx_uniforms* u) {
    if (u == nullptr) return fail(c, SGX_ERR_INVALID_ARGUMENT, "uniforms is NULL");
    if (u->width == 0 || u->height == 0) return fail(c, SGX_ERR_INVALID_ARGUMENT, "width and height must be > 0");
    if (std::uint64_t(u->width) * u->height > (std::uint64_t(1) << 31))
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "image larger than 2^31 pixels");
    if (u->metric_type != SGX_METRIC_KERR && u->metric_type != SGX_METRIC_SCHWARZSCHILD)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown metric_type");
    return SGX_OK;
}

sgx_render_opts resolve_opts(const sgx_render_opts* o) {
    sgx_render_opts d;
    sgx_render_opts_default(&d);
    if (o == nullptr) return d;
    sgx_render_opts r = d;
    const std::size_t n = std::min<std::size_t>(o->struct_size == 0 ? sizeof(sgx_render_opts) : o->struct_size,
                                                sizeof(sgx_render_opts));
    std::memcpy(&r, o, n);
    r.struct_size = sizeof(sgx_render_opts);
    return r;
}

sgx_status check_opts(sgx_context* c, const sgx_render_opts& o) {
    if (o.precision > SGX_PRECISION_FP64) return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown precision");
    if (o.integrator > SGX_INTEGRATOR_ADAPTIVE) return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown integrator");
    if (o.format > SGX_FORMAT_RGBA16F_HDR) return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown format");
    if (o.rhs_form > 2) return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown rhs_form");
    // the tracer's warp votes assume whole warps, and its launch bounds 256 threads
    if (o.block_threads != 0 && (o.block_threads % 32u != 0 || o.block_threads > 256u))
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "block_threads must be 0 or a multiple of 32 up to 256");
    if ((o.tile_w == 0) != (o.tile_h == 0) || o.tile_w > 4096 || o.tile_h > 4096)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "tile_w and tile_h must both be 0 or both in [1, 4096]");
    if (o.integrator == SGX_INTEGRATOR_ADAPTIVE) {
        if (!(o.tolerance > 0.0f) || !(o.h_init_frac > 0.0f) || !(o.h_max_frac > 0.0f) || !(o.fp64_zone >= 0.0f))
            return fail(c, SGX_ERR_INVALID_ARGUMENT, "adaptive options must be positive (zone >= 0)");
    }
    if (o.precision == SGX_PRECISION_MIXED && o.integrator == SGX_INTEGRATOR_FIXED)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "the mixed precision form applies to the adaptive integrator");
    if (o.projection > 1u) return fail(c, SGX_ERR_INVALID_ARGUMENT, "projection must be 0 or 1");
    return SGX_OK;
}

// Renders (and batches) always project; turning the projection off is a
// diagnostic of the two probes.
sgx_status check_render_projection(sgx_context* c, const sgx_render_opts& o) {
    if (o.integrator == SGX_INTEGRATOR_ADAPTIVE && o.projection == 0u)
        return fail(c, SGX_ERR_UNSUPPORTED,
                    "projection = 0 applies to sgx_trace_samples and sgx_trace_invariants; renders always project");
    if (o.slice_count > 1u && (o.slice_index >= o.slice_count || o.slice_count > 65536u || o.slice_band > 65536u))
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "slice_index must be below slice_count (<= 65536), slice_band <= 65536");
    return SGX_OK;
}

sgxk::SliceSpec slice_of(const sgx_render_opts& o) {
    sgxk::SliceSpec sl;
    if (o.slice_count > 1u) {
        sl.count = o.slice_count;
        sl.index = o.slice_index;
        sl.band = o.slice_band == 0u ? SGX_SLICE_BAND_DEFAULT : o.slice_band;
    }
    return sl;
}

// The integrator options of a probe launch.
sgxk::PassDesc probe_opts(const sgx_render_opts& o) {
    sgxk::PassDesc p{};
    p.tol = o.tolerance;
    p.h_init_frac = o.h_init_frac;
    p.h_max_frac = o.h_max_frac;
    p.zone = o.fp64_zone;
    p.project = o.projection;
    return p;
}

std::uint32_t clamp_spp(std::uint32_t ss) { return ss < 1u ? 1u : (ss > 1024u ? 1024u : ss); }

// One render (all passes of [begin, begin+count)) into `out` with `format`.
sgx_status render_impl(sgx_context* c, const sgx_uniforms* u, const sgx_render_opts& o, void* out,
                       std::uint32_t format, cudaStream_t st) {
    const std::uint32_t spp = clamp_spp(u->supersample);
    const std::uint32_t begin = o.sample_begin;
    if (begin >= spp) return fail(c, SGX_ERR_INVALID_ARGUMENT, "sample_begin beyond samples per pixel");
    if (begin != 0 && begin != c->next_sample)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "progressive passes must continue from the previous pass");
    const std::uint32_t count =
        o.sample_count == 0 ? spp - begin : std::min<std::uint32_t>(o.sample_count, spp - begin);
    const sgxk::SliceSpec slice = slice_of(o);
    const std::uint32_t rows = slice.count > 1u ? sgxk::slice_rows(u->height, slice.band, slice.count, slice.index)
                                                : u->height;
    if (rows == 0u) return fail(c, SGX_ERR_INVALID_ARGUMENT, "the frame slice has no rows");
    const std::uint32_t npix = u->width * rows;

    // Pass size under the workspace budget.
    std::size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    std::size_t budget = std::min(c->workspace_budget, free_b / 2 + c->results_cap);
    std::uint64_t per_sample = std::uint64_t(npix) * sgxk::record_bytes(int(o.precision));
    std::uint32_t S = std::uint32_t(std::max<std::uint64_t>(1, std::min<std::uint64_t>(count, budget / per_sample)));
    S = std::min(S, sgxk::kMaxPassSamplesHost);
    sgx_status s = ensure_results(c, std::size_t(S) * per_sample);
    if (s != SGX_OK) return s;

    SGX_CUDA(c, cudaMemcpyAsync(c->d_u, u, sizeof(sgx_uniforms), cudaMemcpyHostToDevice, st));
    SGX_CUDA(c, sgxk::launch_setup_views(c->d_u, 1, c->d_view, int(o.precision), st));
    // The tracer takes the view's constants as a kernel parameter: a host copy
    // of the device-computed slot, refreshed when the uniforms change.
    if (c->h_view_precision != int(o.precision) || std::memcmp(&c->h_view_u, u, sizeof(sgx_uniforms)) != 0) {
        c->h_view_precision = -1;
        SGX_CUDA(c, cudaMemcpyAsync(c->h_view, c->d_view, sgxk::view_bytes(), cudaMemcpyDeviceToHost, st));
        SGX_CUDA(c, cudaStreamSynchronize(st));
        c->h_view_u = *u;
        c->h_view_precision = int(o.precision);
    }
    const std::uint32_t tw = o.tile_w;
    const std::uint32_t th = o.tile_h;
    // An HDR frame into the context's image fuses the bloom extract into its
    // last accumulation pass (sgx_bloom then blurs and composes only).
    c->bloom_ext_valid = false;
    // Only a render into the context's own image changes what sgx_capture and
    // sgx_bloom see; a render into a caller's buffer leaves that state alone.
    const bool own = out == c->d_image;
    if (own) {
        c->frame_valid = false;
        c->post_valid = false;
    }
    const bool fuse_ext = format == SGX_FORMAT_RGBA16F_HDR && own && slice.count <= 1u &&
                          u->width >= 2u && u->height >= 2u;
    if (fuse_ext) {
        const sgx_status bs = sgx_internal::ensure_bloom_targets(c, u->width, u->height);
        if (bs != SGX_OK) return bs;
    }

    sgx_render_stats acc{};
    for (std::uint32_t done = 0; done < count;) {
        const std::uint32_t n = std::min(S, count - done);
        const std::uint32_t s0 = begin + done;
        sgxk::ViewPlan plan;
        if (!sgxk::plan_views(u, 1, s0, n, tw, th, plan, slice))
            return fail(c, SGX_ERR_INVALID_ARGUMENT, "invalid pass or tile shape");
        SGX_CUDA(c, cudaMemcpyAsync(c->d_words, plan.words, plan.word_count * 8, cudaMemcpyHostToDevice, st));
        sgxk::PassDesc pass{};
        pass.vs = sgxk::make_view_set(plan, c->d_view, c->d_words);
        pass.refill = o.refill_interval == 0 ? sgxk::kDefaultRefill : o.refill_interval;
        pass.results = c->d_results;
        pass.counters = c->d_counters;
        pass.tol = o.tolerance;
        pass.h_init_frac = o.h_init_frac;
        pass.h_max_frac = o.h_max_frac;
        pass.zone = o.fp64_zone;
        pass.project = o.projection;
        SGX_CUDA(c, cudaEventRecord(c->ev_begin, st));
        SGX_CUDA(c, cudaMemsetAsync(c->d_counters, 0, sizeof(sgxk::PassCounters), st));
        SGX_CUDA(c, cudaEventRecord(c->ev_trace0, st));
        sgxk::LaunchShape shape{int(o.block_threads), int(o.blocks_per_sm)};
        SGX_CUDA(c, sgxk::launch_trace(int(u->metric_type), int(o.precision), int(o.integrator), int(o.rhs_form),
                                       pass, shape, st, c->h_view));
        SGX_CUDA(c, cudaEventRecord(c->ev_trace1, st));
        const bool first = (s0 == 0);
        const bool finalize = (s0 + n == spp);
        if (finalize && fuse_ext)
            SGX_CUDA(c, sgxk::launch_accumulate_hdr_extract(int(o.precision), pass.vs, c->d_results, c->d_acc, first,
                                                            out, c->d_bloom, u->width, u->height,
                                                            u->bloom_threshold, st));
        else
            SGX_CUDA(c, sgxk::launch_accumulate(int(o.precision), pass.vs, c->d_results, c->d_acc, first, finalize,
                                                format, out, st));
        SGX_CUDA(c, cudaMemcpyAsync(c->h_counters, c->d_counters, sizeof(sgxk::PassCounters),
                                    cudaMemcpyDeviceToHost, st));
        SGX_CUDA(c, cudaEventRecord(c->ev_end, st));
        SGX_CUDA(c, cudaEventSynchronize(c->ev_end));
        acc.rays += c->h_counters->rays;
        acc.steps += c->h_counters->steps;
        acc.rejected += c->h_counters->rejected;
        acc.zone_steps += c->h_counters->zone_steps;
        acc.budget_hits += c->h_counters->budget_hits;
        cudaEventElapsedTime(&acc.trace_ms, c->ev_trace0, c->ev_trace1);
        cudaEventElapsedTime(&acc.total_ms, c->ev_begin, c->ev_end);
        done += n;
        c->next_sample = s0 + n;
        if (own) c->frame_valid = finalize;
        if (finalize && fuse_ext) {
            c->bloom_ext_valid = true;
            c->bloom_ext_threshold = u->bloom_threshold;
        }
    }
    c->stats = acc;
    if (own) {
        c->frame_spp = spp;
        c->frame_format = format;
        c->last_u = *u;
        c->post_valid = false;
    }
    return SGX_OK;
}

}  // namespace

sgx_status sgx_internal::resolve_and_check(sgx_context* ctx, const sgx_render_opts* in, sgx_render_opts& out) {
    out = resolve_opts(in);
    const sgx_status s = check_opts(ctx, out);
    return s != SGX_OK ? s : check_render_projection(ctx, out);
}

extern "C" {

int sgx_abi_version(void) { return SGX_ABI_VERSION; }

const char* sgx_status_string(sgx_status s) {
    switch (s) {
        case SGX_OK: return "ok";
        case SGX_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SGX_ERR_CUDA: return "CUDA error";
        case SGX_ERR_OUT_OF_MEMORY: return "out of device memory";
        case SGX_ERR_NOT_RENDERED: return "no frame rendered";
        case SGX_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

void sgx_render_opts_default(sgx_render_opts* o) {
    if (o == nullptr) return;
    std::memset(o, 0, sizeof(*o));
    o->struct_size = sizeof(sgx_render_opts);
    o->precision = SGX_PRECISION_FP32;
    o->integrator = SGX_INTEGRATOR_FIXED;
    o->format = SGX_FORMAT_RGBA8_SRGB;
    o->tolerance = 1e-6f;
    o->h_init_frac = 0.1f;
    o->h_max_frac = 0.1f;
    o->fp64_zone = 0.05f;
    o->projection = 1u;
}

sgx_status sgx_create(int device, sgx_context** out) {
    if (out == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return SGX_ERR_CUDA;
    if (device < 0) cudaGetDevice(&device);
    if (device >= n) return SGX_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return SGX_ERR_CUDA;
    sgx_context* c = new sgx_context();
    c->device = device;
    bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&c->d_view, sgxk::view_bytes() * sgxk::kMaxLaunchViews) == cudaSuccess;
    ok = ok && cudaMalloc(reinterpret_cast<void**>(&c->d_u), sizeof(sgx_uniforms) * sgxk::kMaxLaunchViews) ==
                   cudaSuccess;
    ok = ok && cudaMalloc(reinterpret_cast<void**>(&c->d_words), sizeof(sgxk::ViewPlan::words)) == cudaSuccess;
    ok = ok && cudaMalloc(reinterpret_cast<void**>(&c->d_counters), sizeof(sgxk::PassCounters)) == cudaSuccess;
    ok = ok && cudaMallocHost(reinterpret_cast<void**>(&c->h_counters), sizeof(sgxk::PassCounters)) == cudaSuccess;
    ok = ok && cudaMallocHost(&c->h_view, sgxk::view_bytes()) == cudaSuccess;
    ok = ok && cudaEventCreate(&c->ev_begin) == cudaSuccess && cudaEventCreate(&c->ev_trace0) == cudaSuccess
         && cudaEventCreate(&c->ev_trace1) == cudaSuccess && cudaEventCreate(&c->ev_end) == cudaSuccess;
    if (!ok) {
        sgx_destroy(c);
        return SGX_ERR_CUDA;
    }
    *out = c;
    return SGX_OK;
}

void sgx_destroy(sgx_context* c) {
    if (c == nullptr) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_image(c);
    sgx_internal_free_diff(c);
    if (c->d_view) cudaFree(c->d_view);
    if (c->d_u) cudaFree(c->d_u);
    if (c->d_words) cudaFree(c->d_words);
    if (c->d_counters) cudaFree(c->d_counters);
    if (c->h_counters) cudaFreeHost(c->h_counters);
    if (c->h_view) cudaFreeHost(c->h_view);
    for (cudaEvent_t ev : {c->ev_begin, c->ev_trace0, c->ev_trace1, c->ev_end})
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

sgx_status sgx_resize(sgx_context* c, uint32_t width, uint32_t height) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (width == 0 || height == 0) return fail(c, SGX_ERR_INVALID_ARGUMENT, "width and height must be > 0");
    cudaSetDevice(c->device);
    return ensure_size(c, width, height);
}

sgx_status sgx_render(sgx_context* c, const sgx_uniforms* u, const sgx_render_opts* opts) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    sgx_status s = check_uniforms(c, u);
    if (s != SGX_OK) return s;
    const sgx_render_opts o = resolve_opts(opts);
    if ((s = check_opts(c, o)) != SGX_OK) return s;
    if ((s = check_render_projection(c, o)) != SGX_OK) return s;
    if (o.slice_count > 1u)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "a frame slice renders through sgx_render_device");
    cudaSetDevice(c->device);
    if ((s = ensure_size(c, u->width, u->height)) != SGX_OK) return s;
    return render_impl(c, u, o, c->d_image, o.format, c->stream);
}

sgx_status sgx_render_device(sgx_context* c, const sgx_uniforms* u, const sgx_render_opts* opts, void* d_out,
                             uint32_t format, void* stream) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (d_out == nullptr) return fail(c, SGX_ERR_INVALID_ARGUMENT, "d_out is NULL");
    sgx_status s = check_uniforms(c, u);
    if (s != SGX_OK) return s;
    sgx_render_opts o = resolve_opts(opts);
    o.format = format;
    if ((s = check_opts(c, o)) != SGX_OK) return s;
    if ((s = check_render_projection(c, o)) != SGX_OK) return s;
    cudaSetDevice(c->device);
    if ((s = ensure_size(c, u->width, u->height)) != SGX_OK) return s;
    cudaStream_t st = stream != nullptr ? static_cast<cudaStream_t>(stream) : c->stream;
    return render_impl(c, u, o, d_out, format, st);
}

sgx_status sgx_capture(sgx_context* c, void* host_out, size_t bytes, uint32_t format) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (host_out == nullptr) return fail(c, SGX_ERR_INVALID_ARGUMENT, "host_out is NULL");
    if (!c->frame_valid) return fail(c, SGX_ERR_NOT_RENDERED, "no complete frame to capture");
    if (format > SGX_FORMAT_RGBA16F_HDR) return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown format");
    const std::size_t need = std::size_t(c->width) * c->height * sgxk::format_bytes(format);
    if (bytes < need) return fail(c, SGX_ERR_INVALID_ARGUMENT, "host buffer too small");
    cudaSetDevice(c->device);
    const void* src = c->d_image;
    if (c->frame_format == SGX_FORMAT_RGBA16F_HDR) {
        // An HDR frame: the raw half image, or the bloom-composed display image.
        if (format != SGX_FORMAT_RGBA16F_HDR) {
            if (!c->post_valid || c->post_format != format)
                return fail(c, SGX_ERR_NOT_RENDERED,
                            "an HDR frame is captured as RGBA16F, or in the format of its sgx_bloom output");
            src = c->d_post;
        }
    } else {
        if (format == SGX_FORMAT_RGBA16F_HDR)
            return fail(c, SGX_ERR_UNSUPPORTED, "render with SGX_FORMAT_RGBA16F_HDR to capture HDR");
        if (format != c->frame_format) {
            SGX_CUDA(c, sgxk::launch_encode(c->d_acc, c->width * c->height, 1.0f / float(c->frame_spp), format,
                                            c->d_image, c->stream));
            c->frame_format = format;
        }
    }
    SGX_CUDA(c, cudaMemcpyAsync(host_out, src, need, cudaMemcpyDeviceToHost, c->stream));
    SGX_CUDA(c, cudaStreamSynchronize(c->stream));
    return SGX_OK;
}

sgx_status sgx_get_stats(const sgx_context* c, sgx_render_stats* out) {
    if (c == nullptr || out == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    *out = c->stats;
    return SGX_OK;
}

const char* sgx_last_error(const sgx_context* c) {
    if (c == nullptr) return "context is NULL";
    return c->err.c_str();
}

sgx_status sgx_trace_samples(sgx_context* c, const sgx_uniforms* u, const sgx_render_opts* opts, uint64_t n,
                             const uint32_t* gx, const uint32_t* gy, const uint32_t* s, float* hdr3,
                             uint32_t* steps, uint32_t* term) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    sgx_status st = check_uniforms(c, u);
    if (st != SGX_OK) return st;
    const sgx_render_opts o = resolve_opts(opts);
    if ((st = check_opts(c, o)) != SGX_OK) return st;
    if (n == 0) return SGX_OK;
    if (gx == nullptr || gy == nullptr || s == nullptr) return fail(c, SGX_ERR_INVALID_ARGUMENT, "NULL sample arrays");
    for (uint64_t i = 0; i < n; ++i)
        if (gx[i] >= u->width || gy[i] >= u->height) return fail(c, SGX_ERR_INVALID_ARGUMENT, "pixel out of range");
    cudaSetDevice(c->device);
    // Device copies: inputs, then outputs (3 floats + 2 words per sample).
    const std::size_t in_b = n * 3 * sizeof(uint32_t);
    const std::size_t out_b = n * 5 * sizeof(uint32_t);
    void* d = nullptr;
    SGX_CUDA(c, cudaMalloc(&d, in_b + out_b));
    uint32_t* d_gx = static_cast<uint32_t*>(d);
    uint32_t* d_gy = d_gx + n;
    uint32_t* d_s = d_gy + n;
    float* d_hdr = reinterpret_cast<float*>(d_s + n);
    uint32_t* d_steps = reinterpret_cast<uint32_t*>(d_hdr + 3 * n);
    uint32_t* d_term = d_steps + n;
    cudaError_t e = cudaMemcpyAsync(d_gx, gx, n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_gy, gy, n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, s, n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_u, u, sizeof(sgx_uniforms), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = sgxk::launch_setup_views(c->d_u, 1, c->d_view, int(o.precision), c->stream);
    if (e == cudaSuccess)
        e = sgxk::launch_probe(c->d_view, int(u->metric_type), int(o.precision), int(o.integrator), int(o.rhs_form), n, d_gx,
                               d_gy, d_s, d_hdr, d_steps, d_term, probe_opts(o), c->stream);
    if (e == cudaSuccess && hdr3) e = cudaMemcpyAsync(hdr3, d_hdr, n * 12, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && steps) e = cudaMemcpyAsync(steps, d_steps, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && term) e = cudaMemcpyAsync(term, d_term, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_trace_samples");
    return SGX_OK;
}

uint32_t sgx_slice_rows(uint32_t height, uint32_t band, uint32_t count, uint32_t index) {
    if (band == 0u) band = SGX_SLICE_BAND_DEFAULT;
    if (count <= 1u) return index == 0u ? height : 0u;
    if (index >= count) return 0u;
    return sgxk::slice_rows(height, band, count, index);
}

uint32_t sgx_slice_row(uint32_t height, uint32_t band, uint32_t count, uint32_t index, uint32_t local) {
    if (band == 0u) band = SGX_SLICE_BAND_DEFAULT;
    if (local >= sgx_slice_rows(height, band, count, index)) return UINT32_MAX;
    if (count <= 1u) return local;
    return sgxk::slice_row(band, count, index, local);
}

sgx_status sgx_trace_invariants(sgx_context* c, const sgx_uniforms* u, const sgx_render_opts* opts, uint64_t n,
                                const uint32_t* gx, const uint32_t* gy, const uint32_t* s, double* inv5,
                                uint32_t* term) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    sgx_status st = check_uniforms(c, u);
    if (st != SGX_OK) return st;
    const sgx_render_opts o = resolve_opts(opts);
    if ((st = check_opts(c, o)) != SGX_OK) return st;
    if (o.integrator != SGX_INTEGRATOR_ADAPTIVE || u->metric_type != SGX_METRIC_KERR)
        return fail(c, SGX_ERR_UNSUPPORTED, "constants of motion are reported for the error-controlled Kerr form");
    if (n == 0) return SGX_OK;
    if (gx == nullptr || gy == nullptr || s == nullptr || inv5 == nullptr)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "NULL sample or output arrays");
    for (uint64_t i = 0; i < n; ++i)
        if (gx[i] >= u->width || gy[i] >= u->height) return fail(c, SGX_ERR_INVALID_ARGUMENT, "pixel out of range");
    cudaSetDevice(c->device);
    // Device copies: inputs (3 words per sample), then 5 doubles and a word per sample.
    const std::size_t in_b = (n * 3 * sizeof(uint32_t) + 7) / 8 * 8;
    const std::size_t out_b = n * 5 * sizeof(double) + n * sizeof(uint32_t);
    void* d = nullptr;
    SGX_CUDA(c, cudaMalloc(&d, in_b + out_b));
    uint32_t* d_gx = static_cast<uint32_t*>(d);
    uint32_t* d_gy = d_gx + n;
    uint32_t* d_s = d_gy + n;
    double* d_inv = reinterpret_cast<double*>(static_cast<unsigned char*>(d) + in_b);
    uint32_t* d_term = reinterpret_cast<uint32_t*>(d_inv + 5 * n);
    cudaError_t e = cudaMemcpyAsync(d_gx, gx, n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_gy, gy, n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, s, n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_u, u, sizeof(sgx_uniforms), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = sgxk::launch_setup_views(c->d_u, 1, c->d_view, int(o.precision), c->stream);
    if (e == cudaSuccess)
        e = sgxk::launch_invariants(c->d_view, int(o.precision), int(o.rhs_form), n, d_gx, d_gy, d_s, d_inv, d_term,
                                    probe_opts(o), c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(inv5, d_inv, n * 40, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && term) e = cudaMemcpyAsync(term, d_term, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_trace_invariants");
    return SGX_OK;
}

}  // extern "C"
