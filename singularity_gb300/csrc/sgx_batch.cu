// singularity_gb300/csrc/sgx_batch.cu
//
// Batched views (no counterpart in the reference, which renders one view per
// launch: render/cuda/cuda_backend.cu:140-152) and the launch-shape
// autotuner.
//
// A batch is up to kMaxLaunchViews views of one metric, each with its own
// resolution, spin, camera and samples per pixel, traced by ONE persistent
// launch: the ray-id space concatenates the views, each warp refills from the
// single queue, so short views do not idle the GPU while long ones finish.
// The whole frame set — counter reset, per-view constants, trace, ordered
// accumulation and encode — is captured once into a CUDA graph at creation
// and replayed by sgx_batch_launch; sgx_batch_update rewrites the views'
// uniforms in place so the same graph renders new cameras or scenes of the
// same sizes.
//
// The autotuner times candidate launch shapes (threads per block, refill
// interval, ray-order tile) on a reduced copy of the batch (each view's
// samples capped) and returns the fastest as render options.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "sgx.h"
#include "sgx_context.hpp"
#include "sgx_kernels.hpp"

using sgx_internal::cuda_fail;
using sgx_internal::fail;

struct sgx_batch {
    sgx_context* ctx = nullptr;
    std::uint32_t n = 0;
    std::uint32_t metric = 0;
    std::uint32_t format = SGX_FORMAT_RGBA8_SRGB;
    sgx_render_opts opts{};
    sgxk::ViewPlan plan;
    std::vector<sgx_uniforms> views;  // host copy (sizes are fixed for the batch's life)
    sgx_uniforms* d_u = nullptr;
    void* d_views = nullptr;
    std::uint64_t* d_words = nullptr;
    void* d_results = nullptr;
    float4* d_acc = nullptr;
    void* d_out = nullptr;
    sgxk::PassCounters* d_counters = nullptr;
    sgxk::PassCounters* h_counters = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t last_stream = nullptr;
};

namespace {

// Enqueues the batch's work (counter reset .. encode) on st.
cudaError_t enqueue(sgx_batch* b, const sgx_render_opts& o, const sgxk::ViewPlan& plan, void* results,
                    cudaStream_t st) {
    sgxk::PassDesc pass{};
    pass.vs = sgxk::make_view_set(plan, b->d_views, b->d_words);
    pass.refill = o.refill_interval == 0 ? sgxk::kDefaultRefill : o.refill_interval;
    pass.results = results;
    pass.counters = b->d_counters;
    pass.tol = o.tolerance;
    pass.h_init_frac = o.h_init_frac;
    pass.h_max_frac = o.h_max_frac;
    pass.zone = o.fp64_zone;
    pass.project = o.projection;
    cudaError_t e = cudaMemsetAsync(b->d_counters, 0, sizeof(sgxk::PassCounters), st);
    if (e == cudaSuccess) e = sgxk::launch_setup_views(b->d_u, b->n, b->d_views, int(o.precision), st);
    if (e == cudaSuccess)
        e = sgxk::launch_trace(int(b->metric), int(o.precision), int(o.integrator), int(o.rhs_form), pass,
                               sgxk::LaunchShape{int(o.block_threads), int(o.blocks_per_sm)}, st);
    if (e == cudaSuccess)
        e = sgxk::launch_accumulate(int(o.precision), pass.vs, results, b->d_acc, true, true, b->format, b->d_out, st);
    return e;
}

sgx_status check_views(sgx_context* c, const sgx_uniforms* views, std::uint32_t n, std::uint32_t& metric) {
    if (views == nullptr || n == 0) return fail(c, SGX_ERR_INVALID_ARGUMENT, "no views");
    if (n > sgxk::kMaxLaunchViews)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "a batch holds at most 128 views (SGX_BATCH_MAX_VIEWS)");
    metric = views[0].metric_type;
    for (std::uint32_t i = 0; i < n; ++i) {
        const sgx_uniforms& u = views[i];
        if (u.width == 0 || u.height == 0) return fail(c, SGX_ERR_INVALID_ARGUMENT, "view with zero size");
        if (u.metric_type != metric)
            return fail(c, SGX_ERR_INVALID_ARGUMENT, "all views of a batch must use the same metric");
        if (u.metric_type != SGX_METRIC_KERR && u.metric_type != SGX_METRIC_SCHWARZSCHILD)
            return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown metric_type");
    }
    return SGX_OK;
}

// Plan with the options' tile (tile_w = 0: whole rows of each view).
bool plan_batch(const sgx_uniforms* views, std::uint32_t n, const sgx_render_opts& o, std::uint32_t S_cap,
                sgxk::ViewPlan& plan) {
    const std::uint32_t tw = o.tile_w, th = o.tile_h;
    if (S_cap == 0) return sgxk::plan_views(views, n, 0, 0, tw, th, plan);
    std::vector<sgx_uniforms> capped(views, views + n);
    for (auto& u : capped) u.supersample = std::max(1u, std::min(u.supersample, S_cap));
    return sgxk::plan_views(capped.data(), n, 0, 0, tw, th, plan);
}

void free_batch(sgx_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void* p : {static_cast<void*>(b->d_u), b->d_views, static_cast<void*>(b->d_words), b->d_results,
                    static_cast<void*>(b->d_acc), b->d_out, static_cast<void*>(b->d_counters)})
        if (p) cudaFree(p);
    if (b->h_counters) cudaFreeHost(b->h_counters);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
}

}  // namespace

extern "C" {

sgx_status sgx_batch_create(sgx_context* c, const sgx_uniforms* views, uint32_t n, const sgx_render_opts* opts,
                            uint32_t format, sgx_batch** out) {
    if (c == nullptr || out == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::uint32_t metric = 0;
    sgx_status s = check_views(c, views, n, metric);
    if (s != SGX_OK) return s;
    sgx_render_opts o;
    if ((s = sgx_internal::resolve_and_check(c, opts, o)) != SGX_OK) return s;
    if (format != SGX_FORMAT_RGBA8_SRGB && format != SGX_FORMAT_RGBA32F)
        return fail(c, SGX_ERR_UNSUPPORTED, "batch output format must be RGBA8 sRGB or RGBA32F");
    if (o.sample_begin != 0 || o.sample_count != 0)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "a batch renders every sample of every view");
    if (o.slice_count > 1u) return fail(c, SGX_ERR_INVALID_ARGUMENT, "a batch renders whole views (no frame slices)");
    cudaSetDevice(c->device);
    sgx_batch* b = new sgx_batch();
    b->ctx = c;
    b->n = n;
    b->metric = metric;
    b->format = format;
    b->opts = o;
    b->views.assign(views, views + n);
    if (!plan_batch(views, n, o, 0, b->plan)) {
        delete b;
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "invalid tile shape for the batch");
    }
    const std::size_t rec = sgxk::record_bytes(int(o.precision));
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&b->d_u), n * sizeof(sgx_uniforms));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_views, n * sgxk::view_bytes());
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_words), sizeof(b->plan.words));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_results, b->plan.total_recs * rec);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_acc), b->plan.total_pix * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_out, b->plan.total_pix * sgxk::format_bytes(format));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_counters), sizeof(sgxk::PassCounters));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&b->h_counters), sizeof(sgxk::PassCounters));
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_u, views, n * sizeof(sgx_uniforms), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_words, b->plan.words, b->plan.word_count * 8, cudaMemcpyHostToDevice, c->stream);
    // One direct run (sets kernel attributes outside capture), then capture.
    if (e == cudaSuccess) e = enqueue(b, o, b->plan, b->d_results, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t e2 = enqueue(b, o, b->plan, b->d_results, c->stream);
        e = cudaStreamEndCapture(c->stream, &b->graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) {
        free_batch(b);
        delete b;
        return cuda_fail(c, e, "sgx_batch_create");
    }
    *out = b;
    return SGX_OK;
}

sgx_status sgx_batch_update(sgx_batch* b, const sgx_uniforms* views) {
    if (b == nullptr || views == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    for (std::uint32_t i = 0; i < b->n; ++i) {
        const sgx_uniforms& a = b->views[i];
        const sgx_uniforms& u = views[i];
        if (a.width != u.width || a.height != u.height || a.supersample != u.supersample ||
            a.metric_type != u.metric_type)
            return fail(b->ctx, SGX_ERR_INVALID_ARGUMENT,
                        "sgx_batch_update keeps each view's size, samples and metric; create a new batch");
    }
    cudaSetDevice(b->ctx->device);
    std::memcpy(b->views.data(), views, b->n * sizeof(sgx_uniforms));
    // Ordered on the stream of the last launch (or the context's), so a
    // launch in flight finishes with the old views.
    cudaStream_t st = b->last_stream != nullptr ? b->last_stream : b->ctx->stream;
    cudaError_t e = cudaMemcpyAsync(b->d_u, views, b->n * sizeof(sgx_uniforms), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SGX_OK : cuda_fail(b->ctx, e, "sgx_batch_update");
}

sgx_status sgx_batch_launch(sgx_batch* b, void* stream) {
    if (b == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->ctx->device);
    cudaStream_t st = stream != nullptr ? static_cast<cudaStream_t>(stream) : b->ctx->stream;
    cudaError_t e = cudaEventRecord(b->ev0, st);
    if (e == cudaSuccess) e = cudaGraphLaunch(b->exec, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_counters, b->d_counters, sizeof(sgxk::PassCounters), cudaMemcpyDeviceToHost, st);
    b->last_stream = st;
    return e == cudaSuccess ? SGX_OK : cuda_fail(b->ctx, e, "sgx_batch_launch");
}

sgx_status sgx_batch_wait(sgx_batch* b, sgx_render_stats* stats) {
    if (b == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->ctx->device);
    cudaStream_t st = b->last_stream != nullptr ? b->last_stream : b->ctx->stream;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(b->ctx, e, "sgx_batch_wait");
    if (stats != nullptr) {
        sgx_render_stats s{};
        s.rays = b->h_counters->rays;
        s.steps = b->h_counters->steps;
        s.rejected = b->h_counters->rejected;
        s.zone_steps = b->h_counters->zone_steps;
        s.budget_hits = b->h_counters->budget_hits;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, b->ev0, b->ev1) == cudaSuccess) {
            s.trace_ms = ms;
            s.total_ms = ms;
        }
        *stats = s;
    }
    return SGX_OK;
}

sgx_status sgx_batch_output(const sgx_batch* b, const void** d_frames, uint64_t* pixel_offsets) {
    if (b == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (d_frames != nullptr) *d_frames = b->d_out;
    if (pixel_offsets != nullptr) {
        const std::uint64_t* pix_off = b->plan.words + (b->n + 1) + b->n;
        for (std::uint32_t i = 0; i <= b->n; ++i) pixel_offsets[i] = pix_off[i];
    }
    return SGX_OK;
}

sgx_status sgx_batch_capture(sgx_batch* b, uint32_t view, void* host, size_t bytes) {
    if (b == nullptr || host == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (view >= b->n) return fail(b->ctx, SGX_ERR_INVALID_ARGUMENT, "view index out of range");
    const std::uint64_t* pix_off = b->plan.words + (b->n + 1) + b->n;
    const std::size_t px = sgxk::format_bytes(b->format);
    const std::size_t need = (pix_off[view + 1] - pix_off[view]) * px;
    if (bytes < need) return fail(b->ctx, SGX_ERR_INVALID_ARGUMENT, "host buffer too small");
    cudaSetDevice(b->ctx->device);
    cudaStream_t st = b->last_stream != nullptr ? b->last_stream : b->ctx->stream;
    cudaError_t e = cudaMemcpyAsync(host, static_cast<const unsigned char*>(b->d_out) + pix_off[view] * px, need,
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SGX_OK : cuda_fail(b->ctx, e, "sgx_batch_capture");
}

void sgx_batch_destroy(sgx_batch* b) {
    if (b == nullptr) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->last_stream != nullptr ? b->last_stream : b->ctx->stream);
    free_batch(b);
    delete b;
}

sgx_status sgx_autotune(sgx_context* c, const sgx_uniforms* views, uint32_t n, const sgx_render_opts* base,
                        uint32_t sample_cap, sgx_render_opts* best, float* best_ms) {
    if (c == nullptr || best == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    std::uint32_t metric = 0;
    sgx_status s = check_views(c, views, n, metric);
    if (s != SGX_OK) return s;
    sgx_render_opts o;
    if ((s = sgx_internal::resolve_and_check(c, base, o)) != SGX_OK) return s;
    cudaSetDevice(c->device);
    const std::uint32_t cap = sample_cap == 0 ? 4u : sample_cap;

    // A scratch batch object over the context's stream; its buffers are sized
    // for the reduced problem.
    sgx_batch tb;
    tb.ctx = c;
    tb.n = n;
    tb.metric = metric;
    tb.format = SGX_FORMAT_RGBA8_SRGB;
    sgxk::ViewPlan probe;
    sgx_render_opts rows = o;
    rows.tile_w = rows.tile_h = 0;
    if (!plan_batch(views, n, rows, cap, probe)) return fail(c, SGX_ERR_INVALID_ARGUMENT, "autotune: bad views");
    std::vector<sgx_uniforms> capped(views, views + n);
    for (auto& u : capped) u.supersample = std::max(1u, std::min(u.supersample, cap));
    const std::size_t rec = sgxk::record_bytes(int(o.precision));
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&tb.d_u), n * sizeof(sgx_uniforms));
    if (e == cudaSuccess) e = cudaMalloc(&tb.d_views, n * sgxk::view_bytes());
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&tb.d_words), sizeof(probe.words));
    if (e == cudaSuccess) e = cudaMalloc(&tb.d_results, probe.total_recs * rec);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&tb.d_acc), probe.total_pix * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&tb.d_out, probe.total_pix * 4);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&tb.d_counters), sizeof(sgxk::PassCounters));
    if (e == cudaSuccess) e = cudaEventCreate(&tb.ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&tb.ev1);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tb.d_u, capped.data(), n * sizeof(sgx_uniforms), cudaMemcpyHostToDevice, c->stream);

    static const std::uint32_t kThreads[] = {64, 128, 256};
    static const std::uint32_t kRefill[] = {16, 32, 64, 128};
    static const std::uint32_t kTiles[][2] = {{0, 0}, {8, 4}, {16, 8}, {32, 2}};
    float best_t = 1e30f;
    sgx_render_opts best_o = o;
    for (std::uint32_t bt : kThreads)
        for (std::uint32_t rf : kRefill)
            for (auto& tl : kTiles) {
                if (e != cudaSuccess) break;
                sgx_render_opts cand = o;
                cand.block_threads = bt;
                cand.refill_interval = rf;
                cand.tile_w = tl[0];
                cand.tile_h = tl[1];
                sgxk::ViewPlan plan;
                if (!plan_batch(capped.data(), n, cand, 0, plan)) continue;
                e = cudaMemcpyAsync(tb.d_words, plan.words, plan.word_count * 8, cudaMemcpyHostToDevice, c->stream);
                float t_min = 1e30f;
                for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
                    e = cudaEventRecord(tb.ev0, c->stream);
                    if (e == cudaSuccess) e = enqueue(&tb, cand, plan, tb.d_results, c->stream);
                    if (e == cudaSuccess) e = cudaEventRecord(tb.ev1, c->stream);
                    if (e == cudaSuccess) e = cudaEventSynchronize(tb.ev1);
                    float ms = 0.f;
                    if (e == cudaSuccess) cudaEventElapsedTime(&ms, tb.ev0, tb.ev1);
                    if (e == cudaSuccess) t_min = std::min(t_min, ms);
                }
                if (e == cudaSuccess && t_min < best_t) {
                    best_t = t_min;
                    best_o = cand;
                }
            }
    tb.graph = nullptr;
    tb.exec = nullptr;
    free_batch(&tb);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_autotune");
    *best = best_o;
    if (best_ms != nullptr) *best_ms = best_t;
    return SGX_OK;
}

}  // extern "C"
