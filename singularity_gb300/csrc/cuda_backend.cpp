// singularity_gb300/csrc/cuda_backend.cpp
//
// The reference's CudaBackend (render/cuda/cuda_backend.cu:105-166) re-made
// over the C ABI of include/sgx.h.

#include "cuda_backend.hpp"

#include <cstdio>

namespace singularity {

namespace {

// The interface's Scene and CameraState as the C ABI's structs (field for
// field; the C struct keeps bools as 0/1).
sgx_scene scene_to_c(const Scene& s) {
    sgx_scene c{};
    c.metric = static_cast<std::uint32_t>(s.metric);
    c.mass_solar = s.mass_solar;
    c.spin_a_over_M = s.spin_a_over_M;
    c.disc_inner_M = s.disc_inner_M;
    c.disc_outer_M = s.disc_outer_M;
    c.disc_doppler_on = s.disc_doppler_on ? 1u : 0u;
    c.disc_redshift_on = s.disc_redshift_on ? 1u : 0u;
    c.disc_texture_on = s.disc_texture_on ? 1u : 0u;
    c.show_overlay = s.show_overlay ? 1u : 0u;
    c.render_supersample = s.render_supersample;
    c.exposure = s.exposure;
    c.bloom_threshold = s.bloom_threshold;
    c.bloom_strength = s.bloom_strength;
    c.disc_turbulence = s.disc_turbulence;
    c.disc_peak_T_K = s.disc_peak_T_K;
    c.max_steps = s.max_steps;
    c.h_step = s.h_step;
    c.adaptive_step_on = s.adaptive_step_on ? 1u : 0u;
    return c;
}

sgx_camera camera_to_c(const CameraState& cam) {
    sgx_camera c{};
    for (int i = 0; i < 3; ++i) c.position[i] = cam.position[i];
    for (int i = 0; i < 9; ++i) c.basis[i] = cam.basis[i];
    c.fov_y_radians = cam.fov_y_radians;
    return c;
}

}  // namespace

CudaBackend::CudaBackend() = default;

CudaBackend::~CudaBackend() { shutdown(); }

bool CudaBackend::initialize(WindowHandle /*window*/, RenderConfig config) {
    width_ = config.width;
    height_ = config.height;
    frame_time_sec_ = 0.0f;
    rendered_ = false;
    if (ctx_ == nullptr && sgx_create(-1, &ctx_) != SGX_OK) {
        std::fprintf(stderr, "singularity CUDA backend: sgx_create failed (no CUDA device?)\n");
        ctx_ = nullptr;
        return false;
    }
    if (sgx_resize(ctx_, width_, height_) != SGX_OK) {
        std::fprintf(stderr, "singularity CUDA backend: initialize failed: %s\n", sgx_last_error(ctx_));
        sgx_destroy(ctx_);
        ctx_ = nullptr;
        return false;
    }
    return true;
}

void CudaBackend::shutdown() {
    if (ctx_ != nullptr) {
        sgx_destroy(ctx_);
        ctx_ = nullptr;
    }
    width_ = 0;
    height_ = 0;
    rendered_ = false;
}

void CudaBackend::resize(std::uint32_t width, std::uint32_t height) {
    if (width == width_ && height == height_) return;
    shutdown();
    RenderConfig cfg{};
    cfg.width = width;
    cfg.height = height;
    initialize(WindowHandle{}, cfg);
}

void CudaBackend::render_frame(const Scene& scene, const CameraState& camera) {
    if (ctx_ == nullptr) return;
    const sgx_scene sc = scene_to_c(scene);
    const sgx_camera cc = camera_to_c(camera);
    sgx_uniforms u{};
    sgx_pack_uniforms(&sc, &cc, width_, height_, frame_time_sec_, &u);
    sgx_render_opts o;
    if (have_opts_) o = opts_;
    else sgx_render_opts_default(&o);
    if (bloom_) o.format = SGX_FORMAT_RGBA16F_HDR;
    const sgx_status s = sgx_render(ctx_, &u, &o);
    if (s != SGX_OK) {
        std::fprintf(stderr, "singularity CUDA backend: render failed: %s\n", sgx_last_error(ctx_));
    } else {
        rendered_ = true;
    }
    frame_time_sec_ += 1.0f / 30.0f;
}

bool CudaBackend::post_(std::uint32_t format) {
    if (!bloom_) return true;
    sgx_bloom_opts b{};
    b.struct_size = sizeof(b);
    b.sigma_px = bloom_sigma_;
    b.threshold = bloom_threshold_;
    b.strength = bloom_strength_;
    b.format = format;
    if (sgx_bloom(ctx_, &b) != SGX_OK) {
        std::fprintf(stderr, "singularity CUDA backend: bloom failed: %s\n", sgx_last_error(ctx_));
        return false;
    }
    return true;
}

ImageData CudaBackend::capture_frame() {
    ImageData out;
    out.width = width_;
    out.height = height_;
    if (ctx_ == nullptr || !rendered_ || !post_(SGX_FORMAT_RGBA8_SRGB)) return out;
    out.pixels_rgba.resize(std::size_t(width_) * height_ * 4u);
    if (sgx_capture(ctx_, out.pixels_rgba.data(), out.pixels_rgba.size(), SGX_FORMAT_RGBA8_SRGB) != SGX_OK) {
        std::fprintf(stderr, "singularity CUDA backend: capture failed: %s\n", sgx_last_error(ctx_));
        out.pixels_rgba.clear();
    }
    return out;
}

std::vector<float> CudaBackend::capture_frame_float() {
    std::vector<float> out;
    if (ctx_ == nullptr || !rendered_ || !post_(SGX_FORMAT_RGBA32F)) return out;
    out.resize(std::size_t(width_) * height_ * 4u);
    if (sgx_capture(ctx_, out.data(), out.size() * sizeof(float), SGX_FORMAT_RGBA32F) != SGX_OK) out.clear();
    return out;
}

}  // namespace singularity
