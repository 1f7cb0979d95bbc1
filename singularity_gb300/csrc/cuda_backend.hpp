// singularity_gb300/csrc/cuda_backend.hpp
//
// C++20 CudaBackend over the C ABI: the same class, members and behaviour as
// the reference's render/cuda/cuda_backend.hpp:17-46, implementing the
// abstract RenderBackend of render/include/render_backend.hpp:107-132.
//
// The interface types (Scene, CameraState, ImageData, WindowHandle,
// RenderConfig, RenderBackend) come from "render_backend.hpp" on the include
// path, never from this header: the reference's own header when a caller of
// the reference (its cuda_cli/main.cpp, which includes both headers) is
// relinked against this library, or this library's declaration of the same
// interface (csrc/render_api/) in its own build.  Put this directory before
// the reference's render/cuda on the include path so "cuda_backend.hpp"
// resolves here.
//
// Behaviour kept from the reference: initialize() allocates the frame and
// returns false on failure; render_frame() is a no-op without a frame,
// prints CUDA errors to stderr and carries on, and advances a virtual 1/30 s
// clock after every frame (cuda_backend.cu:140-152); capture_frame() returns
// an empty ImageData on failure.
#pragma once

#include <cstdint>
#include <vector>

#include "render_backend.hpp"
#include "sgx.h"

namespace singularity {

class CudaBackend : public RenderBackend {
public:
    CudaBackend();
    ~CudaBackend() override;

    bool initialize(WindowHandle window, RenderConfig config) override;
    void shutdown() override;
    void resize(std::uint32_t width, std::uint32_t height) override;
    void render_frame(const Scene& scene, const CameraState& camera) override;
    ImageData capture_frame() override;
    const char* name() const override { return "CUDA"; }

    // Extension (not in the reference): options of every later render_frame
    // (precision form, integrator, launch shape); defaults = the reference.
    void set_render_options(const sgx_render_opts& opts) { opts_ = opts; have_opts_ = true; }
    // Extension: the last frame as RGBA32F (tone-mapped mean before sRGB).
    std::vector<float> capture_frame_float();
    // Extension: the bloom + blit post-process of the desktop backends on every
    // later frame (frames render to the half-float HDR target; captures return
    // the composite). sigma_px 0 = the reference's 7-tap kernel.
    void set_bloom(float sigma_px, float threshold = -1.0f, float strength = -1.0f) {
        bloom_ = true;
        bloom_sigma_ = sigma_px;
        bloom_threshold_ = threshold;
        bloom_strength_ = strength;
    }
    // Extension: the virtual clock of the next frame (the disc bands' phase).
    void set_frame_time(float seconds) { frame_time_sec_ = seconds; }

private:
    std::uint32_t width_{0};
    std::uint32_t height_{0};
    sgx_context* ctx_{nullptr};
    bool rendered_{false};
    float frame_time_sec_{0.0f};
    sgx_render_opts opts_{};
    bool have_opts_{false};
    bool bloom_{false};
    float bloom_sigma_{0.0f}, bloom_threshold_{-1.0f}, bloom_strength_{-1.0f};
    bool post_(std::uint32_t format);
};

}  // namespace singularity
