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
