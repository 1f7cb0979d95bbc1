// singularity_gb300/csrc/render_api/render_backend.hpp
//
// The reference's render interface (render/include/render_backend.hpp:15-140)
// declared for this library's own C++ build: the namespace, type names,
// members, member order, default values and virtual functions are the
// reference's, because callers of CudaBackend compile against them and the
// shim in ../cuda_backend.hpp implements them.
//
// This directory is on the include path only when this repository builds
// its own CLI and shim.  A caller that already has the reference's
// render/include on its include path (the reference's own cuda_cli, relinked
// against this library) gets the reference's header instead, and
// ../cuda_backend.hpp compiles against either: it includes
// "render_backend.hpp" and defines nothing of its own here.
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

namespace singularity {

// Window and surface handles for initialize(); the CUDA backend has no window
// and ignores all three.
struct WindowHandle {
    void* native_window{nullptr};
    void* native_view{nullptr};
    std::function<void*(void*)> vulkan_create_surface{};
};

struct RenderConfig {
    std::uint32_t width{1280};
    std::uint32_t height{720};
    bool vsync_enabled{true};
};

// Per-frame scene block; the defaults are the reference's (a Kerr a/M = 0.6
// hole, disc from its prograde ISCO to 25 M at 4500 K).
struct Scene {
    enum class MetricType : std::uint32_t {
        Schwarzschild = 0,
        Kerr = 1,
    };

    MetricType metric{MetricType::Kerr};
    float mass_solar{1.0f};
    float spin_a_over_M{0.6f};
    float disc_inner_M{3.83f};
    float disc_outer_M{25.0f};
    bool disc_doppler_on{true};
    bool disc_redshift_on{true};
    bool disc_texture_on{true};
    bool show_overlay{false};

    std::uint32_t render_supersample{1};
    float exposure{1.8f};
    float bloom_threshold{0.8f};
    float bloom_strength{0.55f};
    float disc_turbulence{0.5f};
    float disc_peak_T_K{4500.0f};

    // 0 / 0.0: the backend's own step budget and step size
    std::uint32_t max_steps{0};
    float h_step{0.0f};

    bool adaptive_step_on{false};
};

struct CameraState {
    float position[3]{0.0f, 0.0f, 30.0f};
    float basis[9]{1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};  // row-major rows
    float fov_y_radians{1.047f};
};

struct ImageData {
    std::vector<std::uint8_t> pixels_rgba;
    std::uint32_t width{0};
    std::uint32_t height{0};
};

class RenderBackend {
public:
    virtual ~RenderBackend() = default;

    RenderBackend(const RenderBackend&) = delete;
    RenderBackend& operator=(const RenderBackend&) = delete;
    RenderBackend(RenderBackend&&) = delete;
    RenderBackend& operator=(RenderBackend&&) = delete;

    virtual bool initialize(WindowHandle window, RenderConfig config) = 0;
    virtual void shutdown() = 0;
    virtual void resize(std::uint32_t width, std::uint32_t height) = 0;
    virtual void render_frame(const Scene& scene, const CameraState& camera) = 0;
    virtual ImageData capture_frame() = 0;
    virtual const char* name() const = 0;

protected:
    RenderBackend() = default;
};

// The reference's platform factory (declared there beside the interface; its
// live-app definition never creates a CUDA backend).  Not defined by this
// library.
std::unique_ptr<RenderBackend> create_default_backend();

}  // namespace singularity
