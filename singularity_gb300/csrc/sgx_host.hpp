// singularity_gb300/csrc/sgx_host.hpp
//
// Host-side value types of the drop-in boundary, C++20.  They mirror the
// reference's render-interface structs field for field so a caller of the
// reference's CudaBackend recompiles against these unchanged:
//   Scene        <- render/include/render_backend.hpp:46-82
//   CameraState  <- render/include/render_backend.hpp:84-99
//   ImageData    <- render/include/render_backend.hpp:101-105
//   SceneConfig  <- core/include/scene/scene_config.hpp:39-58 (+ loader statuses)
// and the three pure functions between them:
//   build_orbital_camera  <- cuda_cli/main.cpp:68-109
//   pack_uniforms         <- render/cuda/cuda_backend.cu:45-101
//   load_scene_config     <- core/include/scene/scene_config.hpp:134-199
#pragma once

#include <cstdint>
#include <istream>
#include <string>
#include <vector>

#include "sgx.h"

namespace sgx {

struct Scene {
    enum class MetricType : std::uint32_t { Schwarzschild = 0, Kerr = 1 };
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
    std::uint32_t max_steps{0};
    float h_step{0.0f};
    bool adaptive_step_on{false};
};

struct CameraState {
    float position[3]{0.0f, 0.0f, 30.0f};
    float basis[9]{1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};
    float fov_y_radians{1.047f};
};

struct ImageData {
    std::vector<std::uint8_t> pixels_rgba;
    std::uint32_t width{0};
    std::uint32_t height{0};
};

struct SceneConfig {
    float mass = 1.0f;
    float spin = 0.0f;
    float disc_r_inner = -1.0f;
    float disc_r_outer = 20.0f;
    bool disc_doppler_on = true;
    bool disc_redshift_on = true;
    float camera_fov_deg = 60.0f;
    float camera_distance = 30.0f;
    float camera_elevation = 0.0f;
    float h_step = 0.1f;
    int max_steps = 5000;
};

enum class SceneLoadStatus { Ok, FileNotFound, ParseError, UnknownKey };

struct SceneLoadResult {
    SceneLoadStatus status = SceneLoadStatus::Ok;
    std::string error_line;
    int line_number = 0;
};

SceneLoadResult load_scene_config_from_stream(std::istream& in, SceneConfig& out);
SceneLoadResult load_scene_config_from_file(const std::string& path, SceneConfig& out);

void build_orbital_camera(CameraState& cam, float distance_M, float elevation_rad, float azimuth_rad,
                          float fov_y_deg);

sgx_uniforms pack_uniforms(const Scene& scene, const CameraState& cam, std::uint32_t w, std::uint32_t h,
                           float time_sec);

// Prograde ISCO (core/include/physics/kerr.hpp:85-104), float as the reference.
float kerr_isco_prograde(float mass, float spin);

// C-ABI <-> C++ conversions.
sgx_scene to_c(const Scene& s);
Scene from_c(const sgx_scene& s);

}  // namespace sgx
