// oracle/ref_host_harness.cpp
//
// TEST INFRASTRUCTURE — compiles the reference's own CUDA kernel source
// (render/cuda/kernels/geodesic_kernel.cu, included in place from the
// reference tree; nothing is copied) for the host CPU, so the restatement in
// geodesic_oracle.hpp can be pinned against the reference itself.  Built by
// `make -C oracle ref` into oracle/_ref/ only where the reference sources are
// present; the product never sees it.
//
// The kernel body uses blockIdx/threadIdx/blockDim and the device-side
// unsigned max/min; the shims below give it host definitions.  Its
// __device__ functions compile as plain host functions because the CUDA
// headers define the execution-space keywords to nothing outside nvcc.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <sstream>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#undef __global__
#define __global__

thread_local uint3 blockIdx;
thread_local uint3 threadIdx;
thread_local dim3 blockDim;

#include <cmath>
using std::isfinite;

static inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
static inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }

#include SGX_REFERENCE_KERNEL

static_assert(sizeof(Uniforms) == 160, "reference Uniforms layout");

#include "physics/kerr.hpp"

// The reference CLI translation unit, for its build_orbital_camera and the
// scene loader it includes.  Its main() is renamed and never called; the
// CudaBackend members it references get empty host definitions here.
#define main sgx_ref_cuda_cli_main_unused
#include SGX_REFERENCE_CLI
#undef main
namespace singularity {
CudaBackend::CudaBackend() = default;
CudaBackend::~CudaBackend() = default;
bool CudaBackend::initialize(WindowHandle, RenderConfig) { return false; }
void CudaBackend::shutdown() {}
void CudaBackend::resize(std::uint32_t, std::uint32_t) {}
void CudaBackend::render_frame(const Scene&, const CameraState&) {}
ImageData CudaBackend::capture_frame() { return {}; }
}  // namespace singularity

namespace {

template <class F> void parallel_rows(std::uint32_t n, int threads, F&& body) {
    std::atomic<std::uint32_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const std::uint32_t i = next.fetch_add(1);
            if (i >= n) break;
            body(i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < std::max(1, threads); ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// The reference kernel run for every pixel with the 16x16 launch geometry of
// CudaBackend::render_frame (render/cuda/cuda_backend.cu:145-147).
int ref_render_rgba8(const void* uniforms, std::uint8_t* out, int threads) {
    const Uniforms u = *static_cast<const Uniforms*>(uniforms);
    parallel_rows(u.height, threads, [&](std::uint32_t gy) {
        blockDim = dim3(16, 16, 1);
        for (std::uint32_t gx = 0; gx < u.width; ++gx) {
            blockIdx = make_uint3(gx / 16u, gy / 16u, 0);
            threadIdx = make_uint3(gx % 16u, gy % 16u, 0);
            singularity::singularity_geodesic_kernel(out, u);
        }
    });
    return 0;
}

// One sample through the reference's camera and trace functions: HDR colour
// before exposure and tone mapping (geodesic_kernel.cu:483-501).
int ref_trace_hdr(const void* uniforms, std::int64_t n, const std::uint32_t* gx, const std::uint32_t* gy,
                  const std::uint32_t* s, float* hdr3, int threads) {
    const Uniforms u = *static_cast<const Uniforms*>(uniforms);
    const std::uint32_t spp = max(1u, min(u.supersample, 1024u));
    parallel_rows(std::uint32_t(n), threads, [&](std::uint32_t i) {
        float ox = 0.5f, oy = 0.5f;
        if (spp != 1u) {
            ox = singularity::halton(s[i] + 1u, 2u);
            oy = singularity::halton(s[i] + 1u, 3u);
        }
        const singularity::CameraRay cam = singularity::build_camera_ray_subpixel(gx[i], gy[i], ox, oy, u);
        const float3 hdr = (u.metric_type == SING_METRIC_KERR) ? singularity::trace_kerr(cam, u)
                                                               : singularity::trace_schwarzschild(cam, u);
        hdr3[3 * i + 0] = hdr.x;
        hdr3[3 * i + 1] = hdr.y;
        hdr3[3 * i + 2] = hdr.z;
    });
    return 0;
}

// build_orbital_camera (cuda_cli/main.cpp:68-109): position[3], basis[9], fov.
void ref_build_orbital_camera(float distance, float elevation, float azimuth, float fov_deg, float* out13) {
    singularity::CameraState cam{};
    build_orbital_camera(cam, distance, elevation, azimuth, fov_deg);
    for (int i = 0; i < 3; ++i) out13[i] = cam.position[i];
    for (int i = 0; i < 9; ++i) out13[3 + i] = cam.basis[i];
    out13[12] = cam.fov_y_radians;
}

// The reference's Scene{} defaults (render/include/render_backend.hpp:46-82)
// as the 17 floats ref_pack_uniforms takes.
void ref_scene_default(float* scene17) {
    const singularity::Scene sc{};
    const float f[17] = {sc.metric == singularity::Scene::MetricType::Kerr ? 1.0f : 0.0f, sc.mass_solar,
                         sc.spin_a_over_M, sc.disc_inner_M, sc.disc_outer_M, sc.disc_doppler_on ? 1.0f : 0.0f,
                         sc.disc_redshift_on ? 1.0f : 0.0f, sc.disc_texture_on ? 1.0f : 0.0f,
                         sc.show_overlay ? 1.0f : 0.0f, float(sc.render_supersample), sc.exposure,
                         sc.bloom_threshold, sc.bloom_strength, sc.disc_turbulence, sc.disc_peak_T_K,
                         float(sc.max_steps), sc.h_step};
    for (int i = 0; i < 17; ++i) scene17[i] = f[i];
}

// kerr_isco_prograde (core/include/physics/kerr.hpp:85-104), the reference's own.
float ref_kerr_isco_prograde(float mass, float spin) { return singularity::physics::kerr_isco_prograde(mass, spin); }

// The uniform block CudaBackend::render_frame hands the kernel: the semantics
// of pack_uniforms_cuda (render/cuda/cuda_backend.cu:45-101) restated over the
// reference's own Scene, CameraState and Uniforms types — the camera basis
// rows (right, up, -forward), tan of half the FOV and aspect in float, lengths
// scaled by the mass, the backend's step defaults (h 0.4, 2500 steps) where
// the scene leaves 0, escape at 200 M and capture at 1.02 r_s, the starfield
// always on and the disc / Doppler / redshift bits from the scene.  scene17
// holds the Scene fields in declaration order (bools and integers as floats);
// cam13 the camera's position[3], basis[9] and fov_y_radians.
void ref_pack_uniforms(const float* scene17, const float* cam13, std::uint32_t w, std::uint32_t h, float time_sec,
                       void* out160) {
    singularity::Scene sc{};
    sc.metric = scene17[0] != 0.0f ? singularity::Scene::MetricType::Kerr : singularity::Scene::MetricType::Schwarzschild;
    sc.mass_solar = scene17[1];
    sc.spin_a_over_M = scene17[2];
    sc.disc_inner_M = scene17[3];
    sc.disc_outer_M = scene17[4];
    sc.disc_doppler_on = scene17[5] != 0.0f;
    sc.disc_redshift_on = scene17[6] != 0.0f;
    sc.disc_texture_on = scene17[7] != 0.0f;
    sc.show_overlay = scene17[8] != 0.0f;
    sc.render_supersample = std::uint32_t(scene17[9]);
    sc.exposure = scene17[10];
    sc.bloom_threshold = scene17[11];
    sc.bloom_strength = scene17[12];
    sc.disc_turbulence = scene17[13];
    sc.disc_peak_T_K = scene17[14];
    sc.max_steps = std::uint32_t(scene17[15]);
    sc.h_step = scene17[16];
    singularity::CameraState cam{};
    for (int i = 0; i < 3; ++i) cam.position[i] = cam13[i];
    for (int i = 0; i < 9; ++i) cam.basis[i] = cam13[3 + i];
    cam.fov_y_radians = cam13[12];

    Uniforms u{};
    const float* b = cam.basis;
    u.cam_pos = {cam.position[0], cam.position[1], cam.position[2], 0.0f};
    u.cam_right = {b[0], b[1], b[2], 0.0f};
    u.cam_up = {b[3], b[4], b[5], 0.0f};
    u.cam_fwd = {-b[6], -b[7], -b[8], 0.0f};
    u.tan_half_fov = std::tan(0.5f * cam.fov_y_radians);
    u.aspect = float(w) / float(h);
    const float M = sc.mass_solar;
    u.mass_M = M;
    u.spin_a = sc.spin_a_over_M * M;
    u.rs = 2.0f * M;
    u.disc_r_inner = sc.disc_inner_M * M;
    u.disc_r_outer = sc.disc_outer_M * M;
    u.disc_peak_T = sc.disc_peak_T_K;
    u.h_step = sc.h_step > 0.0f ? sc.h_step : 0.4f;
    u.escape_r = 200.0f * M;
    u.horizon_cut = 1.02f * u.rs;
    u.time_sec = time_sec;
    u.width = w;
    u.height = h;
    u.metric_type = sc.metric == singularity::Scene::MetricType::Kerr ? SING_METRIC_KERR : SING_METRIC_SCHWARZSCHILD;
    u.flags = SING_FLAG_STARFIELD_ON | (sc.disc_texture_on ? SING_FLAG_DISC_ON : 0u) |
              (sc.disc_doppler_on ? SING_FLAG_DOPPLER_ON : 0u) | (sc.disc_redshift_on ? SING_FLAG_REDSHIFT_ON : 0u);
    u.max_steps = sc.max_steps != 0u ? sc.max_steps : 2500u;
    u.frame_index = 0;
    u.supersample = sc.render_supersample == 0u ? 1u : sc.render_supersample;
    u.pad_b = 0;
    u.exposure = sc.exposure;
    u.bloom_threshold = sc.bloom_threshold;
    u.bloom_strength = sc.bloom_strength;
    u.disc_turbulence = sc.disc_turbulence;
    std::memcpy(out160, &u, sizeof(u));
}

// load_scene_config_from_stream (core/include/scene/scene_config.hpp:134-191)
// on a text; fields in declaration order, bools as 0/1, max_steps as float.
int ref_load_scene_text(const char* text, float* out11, int* line) {
    singularity::scene::SceneConfig cfg;
    std::istringstream in{std::string(text)};
    const auto r = singularity::scene::load_scene_config_from_stream(in, cfg);
    const float f[11] = {cfg.mass, cfg.spin, cfg.disc_r_inner, cfg.disc_r_outer, cfg.disc_doppler_on ? 1.0f : 0.0f,
                         cfg.disc_redshift_on ? 1.0f : 0.0f, cfg.camera_fov_deg, cfg.camera_distance,
                         cfg.camera_elevation, cfg.h_step, float(cfg.max_steps)};
    for (int i = 0; i < 11; ++i) out11[i] = f[i];
    *line = r.line_number;
    return int(r.status);
}

}  // extern "C"
