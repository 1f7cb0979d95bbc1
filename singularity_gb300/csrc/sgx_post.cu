// singularity_gb300/csrc/sgx_post.cu
//
// HDR bloom and display transform of a frame rendered in SGX_FORMAT_RGBA16F_HDR
// — the realtime backends' post-process (render/vulkan/shaders/bloom.hlsl:8-77
// and blit.hlsl:43-57, the same in Metal and WGSL), restated as CUDA kernels
// because the reference's CUDA path has none (geodesic_kernel.cu:12-15):
//   1. extract: each texel of a half-resolution target is the Karis-weighted
//      average (weights 1 / (1 + luma)) of a 2x2 block of the HDR frame,
//      scaled by the soft knee luma^2 / max(luma + threshold, 1e-4) / luma;
//   2. separable blur along x then y with clamp-to-edge addressing: the
//      reference's 7 weights (about sigma = 2 half-resolution texels), or a
//      normalised Gaussian of a requested sigma in full-resolution pixels;
//   3. compose: hdr + bilinear(bloom) * strength, times exposure, ACES
//      (Narkowicz), then sRGB (RGBA8) or kept linear (RGBA32F).
// Intermediate targets are half precision like the reference's rgba16f
// images.  Bilinear filtering uses exact float weights (hardware samplers
// quantise them).

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "sgx.h"
#include "sgx_context.hpp"
#include "sgx_device.cuh"

using sgx_internal::cuda_fail;
using sgx_internal::fail;

namespace {

constexpr int kMaxTaps = 65;

struct Kernel1D {
    int radius;
    float w[kMaxTaps];
};

__device__ __forceinline__ float4 load_h4(const __half2* p, std::uint64_t i) {
    const float2 a = __half22float2(p[2 * i]);
    const float2 b = __half22float2(p[2 * i + 1]);
    return make_float4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ void store_h4(__half2* p, std::uint64_t i, float x, float y, float z) {
    p[2 * i] = __floats2half2_rn(x, y);
    p[2 * i + 1] = __floats2half2_rn(z, 1.0f);
}

// Separate extract from the stored HDR frame: used when sgx_bloom is given a
// threshold of its own, or on a second post-process of the same frame (the
// last accumulation pass fuses the extract at the uniforms' threshold).
__global__ void extract_kernel(const __half2* __restrict__ hdr, int W, __half2* __restrict__ dst, int bw, int bh,
                               float threshold) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= bw || y >= bh) return;
    const int sx = 2 * x, sy = 2 * y;
    const float4 a = load_h4(hdr, std::uint64_t(sy) * W + sx);
    const float4 b = load_h4(hdr, std::uint64_t(sy) * W + sx + 1);
    const float4 c = load_h4(hdr, std::uint64_t(sy + 1) * W + sx);
    const float4 d = load_h4(hdr, std::uint64_t(sy + 1) * W + sx + 1);
    float r, g, bl;
    sgxd::karis_extract(a, b, c, d, threshold, r, g, bl);
    store_h4(dst, std::uint64_t(y) * bw + x, r, g, bl);
}

__global__ void blur_kernel(const __half2* __restrict__ src, __half2* __restrict__ dst, int bw, int bh, int vertical,
                            Kernel1D kw) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= bw || y >= bh) return;
    float r = 0.0f, g = 0.0f, b = 0.0f;
    for (int i = -kw.radius; i <= kw.radius; ++i) {
        int px = x, py = y;
        if (vertical) py = min(max(y + i, 0), bh - 1);
        else px = min(max(x + i, 0), bw - 1);
        const float4 s = load_h4(src, std::uint64_t(py) * bw + px);
        const float w = kw.w[i + kw.radius];
        r += s.x * w;
        g += s.y * w;
        b += s.z * w;
    }
    store_h4(dst, std::uint64_t(y) * bw + x, r, g, b);
}

__global__ void compose_kernel(const __half2* __restrict__ hdr, const __half2* __restrict__ bloom, int W, int H,
                               int bw, int bh, float strength, float exposure, std::uint32_t format, void* out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    // bilinear, clamp to edge, at the full-resolution pixel centre
    const float tx = (float(x) + 0.5f) / float(W) * float(bw) - 0.5f;
    const float ty = (float(y) + 0.5f) / float(H) * float(bh) - 0.5f;
    const float fx0 = floorf(tx), fy0 = floorf(ty);
    const float fx = tx - fx0, fy = ty - fy0;
    const int x0 = min(max(int(fx0), 0), bw - 1), x1 = min(max(int(fx0) + 1, 0), bw - 1);
    const int y0 = min(max(int(fy0), 0), bh - 1), y1 = min(max(int(fy0) + 1, 0), bh - 1);
    const float4 b00 = load_h4(bloom, std::uint64_t(y0) * bw + x0);
    const float4 b10 = load_h4(bloom, std::uint64_t(y0) * bw + x1);
    const float4 b01 = load_h4(bloom, std::uint64_t(y1) * bw + x0);
    const float4 b11 = load_h4(bloom, std::uint64_t(y1) * bw + x1);
    auto lerp2 = [&](float a, float b, float c, float d) {
        const float top = a + fx * (b - a), bot = c + fx * (d - c);
        return top + fy * (bot - top);
    };
    const float4 h = load_h4(hdr, std::uint64_t(y) * W + x);
    float r = (h.x + lerp2(b00.x, b10.x, b01.x, b11.x) * strength) * exposure;
    float g = (h.y + lerp2(b00.y, b10.y, b01.y, b11.y) * strength) * exposure;
    float b = (h.z + lerp2(b00.z, b10.z, b01.z, b11.z) * strength) * exposure;
    r = sgxd::aces1(r);
    g = sgxd::aces1(g);
    b = sgxd::aces1(b);
    const std::uint64_t i = std::uint64_t(y) * W + x;
    if (format == SGX_FORMAT_RGBA8_SRGB) {
        uchar4 o;
        o.x = sgxd::to_u8(r);
        o.y = sgxd::to_u8(g);
        o.z = sgxd::to_u8(b);
        o.w = 255;
        static_cast<uchar4*>(out)[i] = o;
    } else {
        static_cast<float4*>(out)[i] = make_float4(r, g, b, 1.0f);
    }
}

// The reference's 7 taps (bloom.hlsl:8-11) for sigma <= 0; else a
// normalised Gaussian of sigma_px / 2 half-resolution texels, radius
// ceil(3 sigma) (at most 32).
Kernel1D make_kernel(float sigma_px) {
    Kernel1D k{};
    if (!(sigma_px > 0.0f)) {
        const float ref[7] = {0.071303f, 0.131514f, 0.189879f, 0.214607f, 0.189879f, 0.131514f, 0.071303f};
        k.radius = 3;
        for (int i = 0; i < 7; ++i) k.w[i] = ref[i];
        return k;
    }
    const double s = double(sigma_px) * 0.5;
    int r = int(std::ceil(3.0 * s));
    r = r < 1 ? 1 : (r > (kMaxTaps - 1) / 2 ? (kMaxTaps - 1) / 2 : r);
    k.radius = r;
    double sum = 0.0;
    for (int i = -r; i <= r; ++i) sum += std::exp(-0.5 * double(i) * double(i) / (s * s));
    for (int i = -r; i <= r; ++i) k.w[i + r] = float(std::exp(-0.5 * double(i) * double(i) / (s * s)) / sum);
    return k;
}

}  // namespace

sgx_status sgx_internal::ensure_bloom_targets(sgx_context* c, std::uint32_t W, std::uint32_t H) {
    const std::uint32_t bw = W / 2 > 1 ? W / 2 : 1, bh = H / 2 > 1 ? H / 2 : 1;
    const std::size_t half_bytes = std::size_t(bw) * bh * 8;
    if (c->bloom_cap >= half_bytes) return SGX_OK;
    if (c->d_bloom) cudaFree(c->d_bloom);
    c->d_bloom = nullptr;
    c->bloom_cap = 0;
    c->bloom_ext_valid = false;
    cudaError_t e = cudaMalloc(&c->d_bloom, 2 * half_bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "bloom targets: cudaMalloc");
    c->bloom_cap = half_bytes;
    return SGX_OK;
}

extern "C" sgx_status sgx_bloom(sgx_context* c, const sgx_bloom_opts* opts) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (!c->frame_valid || c->frame_format != SGX_FORMAT_RGBA16F_HDR)
        return fail(c, SGX_ERR_NOT_RENDERED, "sgx_bloom needs a complete frame rendered in SGX_FORMAT_RGBA16F_HDR");
    sgx_bloom_opts o{};
    o.struct_size = sizeof(o);
    o.sigma_px = 0.0f;
    o.threshold = -1.0f;
    o.strength = -1.0f;
    o.format = SGX_FORMAT_RGBA8_SRGB;
    if (opts != nullptr) o = *opts;
    if (o.format != SGX_FORMAT_RGBA8_SRGB && o.format != SGX_FORMAT_RGBA32F)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "bloom output must be RGBA8 sRGB or RGBA32F");
    const float threshold = o.threshold >= 0.0f ? o.threshold : c->last_u.bloom_threshold;
    const float strength = o.strength >= 0.0f ? o.strength : c->last_u.bloom_strength;
    const int W = int(c->width), H = int(c->height);
    const int bw = W / 2 > 1 ? W / 2 : 1, bh = H / 2 > 1 ? H / 2 : 1;
    if (W < 2 || H < 2) return fail(c, SGX_ERR_INVALID_ARGUMENT, "bloom needs at least 2x2 pixels");
    cudaSetDevice(c->device);
    const std::size_t half_bytes = std::size_t(bw) * bh * 8;
    const sgx_status st = sgx_internal::ensure_bloom_targets(c, std::uint32_t(W), std::uint32_t(H));
    if (st != SGX_OK) return st;
    if (c->d_post == nullptr) {
        cudaError_t e = cudaMalloc(&c->d_post, std::size_t(W) * H * 16);
        if (e != cudaSuccess) return cuda_fail(c, e, "sgx_bloom: cudaMalloc");
    }
    __half2* a = static_cast<__half2*>(c->d_bloom);
    __half2* b = reinterpret_cast<__half2*>(static_cast<unsigned char*>(c->d_bloom) + half_bytes);
    const __half2* hdr = static_cast<const __half2*>(c->d_image);
    const dim3 blk(16, 16);
    const dim3 gh((bw + 15) / 16, (bh + 15) / 16), gf((W + 15) / 16, (H + 15) / 16);
    const Kernel1D kw = make_kernel(o.sigma_px);
    // the render's last accumulation pass already wrote the extract at the
    // uniforms' threshold into the first target; a threshold of the caller's
    // own, or a second post-process of the frame, extracts again
    const bool fused = o.threshold < 0.0f && c->bloom_ext_valid && c->bloom_ext_threshold == threshold;
    if (!fused) extract_kernel<<<gh, blk, 0, c->stream>>>(hdr, W, a, bw, bh, threshold);
    c->bloom_ext_valid = false;  // the blur below overwrites the first target
    blur_kernel<<<gh, blk, 0, c->stream>>>(a, b, bw, bh, 0, kw);
    blur_kernel<<<gh, blk, 0, c->stream>>>(b, a, bw, bh, 1, kw);
    compose_kernel<<<gf, blk, 0, c->stream>>>(hdr, a, W, H, bw, bh, strength, c->last_u.exposure, o.format, c->d_post);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_bloom");
    c->post_valid = true;
    c->post_format = o.format;
    return SGX_OK;
}
