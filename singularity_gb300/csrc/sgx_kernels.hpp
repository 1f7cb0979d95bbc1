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

// The views one launch traces (a single view for sgx_render, up to
// kMaxLaunchViews for a batch), all device pointers into one layout block:
//   ray_off[n+1]  offsets of each view in the ray-id space (padded pixels x S_v)
//   rec_off[n]    offsets of each view's hit records (pixels x S_v)
//   pix_off[n+1]  offsets of each view's pixels in the packed image/accumulator
//   S[n]          samples of this pass per view
struct ViewSet {
    const void* views;  // View<T>[n]
    const std::uint64_t* ray_off;
    const std::uint64_t* rec_off;
    const std::uint64_t* pix_off;
    const std::uint32_t* S;
    std::uint32_t n;
    std::uint32_t max_S;
    std::uint32_t s0;      // first Halton sample of the pass (progressive single view); 0 for batches
    std::uint32_t tile_w;  // ray-id order: tiles of tile_w x tile_h pixels, samples innermost; 0 = rows
    std::uint32_t tile_h;
    // frame slice of a single view (slice_count > 1): the pass traces the
    // slice_h rows of slice slice_index (bands of slice_band rows dealt
    // round-robin to slice_count slices); its records, pixels and output rows
    // are the slice's, packed
    std::uint32_t slice_count, slice_index, slice_band, slice_h;
    std::uint64_t total_rays;
    std::uint64_t total_pix;
};

// Rows of slice `index` of `count` in a frame of `height` rows (bands of
// `band` rows dealt round-robin), and the frame row of its local row `l`.
__host__ __device__ inline std::uint32_t slice_rows(std::uint32_t height, std::uint32_t band, std::uint32_t count,
                                                    std::uint32_t index) {
    const std::uint32_t bands = (height + band - 1u) / band;
    if (index >= bands) return 0u;
    const std::uint32_t mine = (bands - index + count - 1u) / count;  // bands index, index + count, ...
    const std::uint32_t last = index + (mine - 1u) * count;           // the slice's last band
    return (mine - 1u) * band + (height - last * band < band ? height - last * band : band);
}
__host__ __device__ inline std::uint32_t slice_row(std::uint32_t band, std::uint32_t count, std::uint32_t index,
                                                   std::uint32_t l) {
    const std::uint32_t b = l / band;
    return (b * count + index) * band + (l - b * band);
}

// Launch shape when the caller leaves it to the library.  A refill runs the
// per-ray set-up (camera ray, constants of motion, photon-orbit radius, first
// right-hand side) once per warp for however many lanes are idle, so refilling
// every 128 steps instead of every 32 amortises it over more lanes: on the 4K
// Kerr pass (error-controlled, mixed) the trace kernel takes 47.7 ms at
// 64-thread blocks and refill 128 against 49.7 ms at 256 and 32 (96 and 192:
// within 0.1 ms of 128; 1080p: 12.59 against 13.10 ms; the fixed step 188.6
// against 192.4 ms); 64-thread blocks are 0.3-1 % faster than 128 or 256.
constexpr std::uint32_t kDefaultRefill = 128;
constexpr int kDefaultBlockThreads = 64;
// Multi-view passes copy the whole view table into each block's shared memory
// (64 views: 18 KB), so small blocks run out of shared memory before
// registers: 64 batched views at 64-thread blocks fit 24 warps per SM, at 128
// threads 28 (register-limited); 1866 against 2003 Mrays/s.
constexpr int kDefaultBlockThreadsMulti = 128;
constexpr std::uint32_t kMaxLaunchViews = 128;
constexpr std::uint32_t kMaxPassSamplesHost = 1024;

struct PassDesc {
    ViewSet vs;
    std::uint32_t refill;  // steps between refills
    void* results;         // hit records, record_bytes(precision) each
    PassCounters* counters;
    // adaptive options
    float tol, h_init_frac, h_max_frac, zone;
    std::uint32_t project;  // 1: p_theta projected onto the Carter constant after accepted steps
};

struct LaunchShape {
    int block_threads;
    int blocks_per_sm;
};

// Host plan of a ViewSet: the layout block's contents (to copy to the device
// as one array of 64-bit words) and the totals.  S_pass == 0 -> every view's
// own samples per pixel.
struct SliceSpec {
    std::uint32_t count = 0, index = 0, band = 0;  // count <= 1: the whole frame
};

struct ViewPlan {
    std::uint32_t n = 0, max_S = 0, s0 = 0, tile_w = 0, tile_h = 0;
    SliceSpec slice{};
    std::uint32_t slice_h = 0;
    std::uint64_t total_rays = 0, total_pix = 0, total_recs = 0;
    std::uint64_t words[4 * kMaxLaunchViews + 2] = {};  // ray_off | rec_off | pix_off | S (packed 2 per word)
    std::size_t word_count = 0;
};
// A slice (slice.count > 1) applies to a single view only.
bool plan_views(const sgx_uniforms* u, std::uint32_t n, std::uint32_t s0, std::uint32_t S_pass, std::uint32_t tile_w,
                std::uint32_t tile_h, ViewPlan& plan, SliceSpec slice = {});
// Device ViewSet over a layout block that holds plan.words at d_words and
// the views at d_views.
ViewSet make_view_set(const ViewPlan& plan, const void* d_views, const std::uint64_t* d_words);

// Per-view constants (device) from device copies of the uniforms, one thread each.
cudaError_t launch_setup_views(const sgx_uniforms* d_u, std::uint32_t n, void* d_views, int precision,
                               cudaStream_t st);

// Persistent tracer over a ViewSet.  precision: sgx_precision; integrator: sgx_integrator.
// h_view: for a single-view pass, a host copy of that view's constants
// (view_bytes() from the device slot setup_views wrote), passed to the kernel
// as a parameter; nullptr = every view read from shared memory.
cudaError_t launch_trace(int metric, int precision, int integrator, int rhs_form, const PassDesc& pass,
                         LaunchShape shape, cudaStream_t st, const void* h_view = nullptr);

// Per-sample probe (parity tests) of a single view: n samples, device arrays;
// the integrator options come from opts (tol, h_init_frac, h_max_frac, zone,
// project).
cudaError_t launch_probe(const void* d_view, int metric, int precision, int integrator, int rhs_form,
                         std::uint64_t n, const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s,
                         float* hdr3, std::uint32_t* steps, std::uint32_t* term, const PassDesc& opts,
                         cudaStream_t st);

// Constants of motion (E, L, Q0, Q_end, 2H_end; FP64, 5 per sample) of n
// samples of the error-controlled Kerr form of a single view.
cudaError_t launch_invariants(const void* d_view, int precision, int rhs_form, std::uint64_t n,
                              const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s, double* inv5,
                              std::uint32_t* term, const PassDesc& pass, cudaStream_t st);

// Shades a pass's hit records and adds them in sample order into acc (float4
// per pixel, packed over views); when `finalize`, also writes every view's
// frame in `format` to out (packed like acc; scale 1/spp of each view).
cudaError_t launch_accumulate(int precision, const ViewSet& vs, const void* results, float4* acc, bool first,
                              bool finalize, std::uint32_t format, void* out, cudaStream_t st);

// The last pass of a single-view, unsliced SGX_FORMAT_RGBA16F_HDR frame (W x
// H, W and H >= 2) with the bloom extract fused in: as launch_accumulate with
// finalize, plus ext (W/2 x H/2 half4 texels) = the Karis-weighted, soft-knee
// extract of each 2x2 block of the half-precision frame at `threshold`.
cudaError_t launch_accumulate_hdr_extract(int precision, const ViewSet& vs, const void* results, float4* acc,
                                          bool first, void* out, void* ext, std::uint32_t W, std::uint32_t H,
                                          float threshold, cudaStream_t st);

// Re-encodes an accumulated single-view frame (acc, float4 mean-sum) in another format.
cudaError_t launch_encode(const float4* acc, std::uint32_t npix, float scale, std::uint32_t format, void* out,
                          cudaStream_t st);

// Bytes of one hit record (16 for FP32 and mixed, 32 for FP64).
std::size_t record_bytes(int precision);
// Bytes of one View<T> of the precision (256-aligned slot).
std::size_t view_bytes();
// Bytes of output per pixel in a format.
std::size_t format_bytes(std::uint32_t format);

}  // namespace sgxk
