// singularity_gb300/csrc/sgx_host.cpp
//
// Host-only half of the boundary: the .scene loader, the orbital camera and
// the uniform packing.  Each function keeps the reference's semantics and its
// float arithmetic order (the packed uniform bytes must equal the
// reference's), written in this library's own structure.

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "sgx_host.hpp"

namespace sgx {

namespace {

// Whitespace trim and typed parsers with the reference's acceptance rules
// (scene_config.hpp:76-131): bools true/on/yes/1 and false/off/no/0 in any
// case; numbers must be followed by nothing but whitespace.
std::string trimmed(const std::string& s) {
    std::size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    return s.substr(b, e - b);
}

bool only_space(const char* p) {
    for (; p != nullptr && *p != '\0'; ++p)
        if (!std::isspace(static_cast<unsigned char>(*p))) return false;
    return true;
}

bool read_bool(const std::string& v, bool& out) {
    std::string k;
    for (char c : v) k.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(c))));
    if (k == "true" || k == "on" || k == "yes" || k == "1") {
        out = true;
        return true;
    }
    if (k == "false" || k == "off" || k == "no" || k == "0") {
        out = false;
        return true;
    }
    return false;
}

bool read_float(const std::string& v, float& out) {
    if (v.empty()) return false;
    char* end = nullptr;
    const float x = std::strtof(v.c_str(), &end);
    if (end == v.c_str() || !only_space(end)) return false;
    out = x;
    return true;
}

bool read_int(const std::string& v, int& out) {
    if (v.empty()) return false;
    char* end = nullptr;
    const long x = std::strtol(v.c_str(), &end, 10);
    if (end == v.c_str() || !only_space(end)) return false;
    out = static_cast<int>(x);
    return true;
}

}  // namespace

SceneLoadResult load_scene_config_from_stream(std::istream& in, SceneConfig& out) {
    std::string raw;
    int n = 0;
    while (std::getline(in, raw)) {
        ++n;
        std::string line = raw.substr(0, raw.find('#'));
        line = trimmed(line);
        if (line.empty()) continue;
        const auto eq = line.find('=');
        if (eq == std::string::npos) return {SceneLoadStatus::ParseError, line, n};
        const std::string key = trimmed(line.substr(0, eq));
        const std::string val = trimmed(line.substr(eq + 1));
        if (key.empty() || val.empty()) return {SceneLoadStatus::ParseError, line, n};
        bool ok;
        if (key == "mass") ok = read_float(val, out.mass);
        else if (key == "spin") ok = read_float(val, out.spin);
        else if (key == "disc_r_inner") ok = read_float(val, out.disc_r_inner);
        else if (key == "disc_r_outer") ok = read_float(val, out.disc_r_outer);
        else if (key == "disc_doppler_on") ok = read_bool(val, out.disc_doppler_on);
        else if (key == "disc_redshift_on") ok = read_bool(val, out.disc_redshift_on);
        else if (key == "camera_fov_deg") ok = read_float(val, out.camera_fov_deg);
        else if (key == "camera_distance") ok = read_float(val, out.camera_distance);
        else if (key == "camera_elevation") ok = read_float(val, out.camera_elevation);
        else if (key == "h_step") ok = read_float(val, out.h_step);
        else if (key == "max_steps") ok = read_int(val, out.max_steps);
        else return {SceneLoadStatus::UnknownKey, key, n};
        if (!ok) return {SceneLoadStatus::ParseError, line, n};
    }
    return {SceneLoadStatus::Ok, {}, n};
}

SceneLoadResult load_scene_config_from_file(const std::string& path, SceneConfig& out) {
    std::ifstream f(path);
    if (!f) return {SceneLoadStatus::FileNotFound, path, 0};
    return load_scene_config_from_stream(f, out);
}

// Orbit camera looking at the origin; basis rows right, up, -forward.
void build_orbital_camera(CameraState& cam, float distance_M, float elevation_rad, float azimuth_rad,
                          float fov_y_deg) {
    const float ce = std::cos(elevation_rad);
    const float se = std::sin(elevation_rad);
    const float ca = std::cos(azimuth_rad);
    const float sa = std::sin(azimuth_rad);
    cam.position[0] = distance_M * ce * ca;
    cam.position[1] = distance_M * ce * sa;
    cam.position[2] = distance_M * se;
    const float inv = 1.0f / distance_M;
    const float f0 = -cam.position[0] * inv, f1 = -cam.position[1] * inv, f2 = -cam.position[2] * inv;
    float r0 = f1, r1 = -f0, r2 = 0.0f;
    const float rl = std::sqrt(r0 * r0 + r1 * r1 + r2 * r2);
    const float ir = (rl > 1e-6f) ? 1.0f / rl : 1.0f;
    r0 *= ir;
    r1 *= ir;
    r2 *= ir;
    // up = forward x right
    const float u0 = f1 * r2 - f2 * r1;
    const float u1 = f2 * r0 - f0 * r2;
    const float u2 = f0 * r1 - f1 * r0;
    const float rows[9] = {r0, r1, r2, u0, u1, u2, -f0, -f1, -f2};
    std::memcpy(cam.basis, rows, sizeof(rows));
    cam.fov_y_radians = fov_y_deg * (3.14159265358979323846f / 180.0f);
}

sgx_uniforms pack_uniforms(const Scene& scene, const CameraState& cam, std::uint32_t w, std::uint32_t h,
                           float time_sec) {
    // Backend defaults when the scene leaves them at 0 (cuda_backend.cu:35-36).
    constexpr std::uint32_t kMaxSteps = 2500;
    constexpr float kHStep = 0.4f;
    sgx_uniforms u{};
    u.cam_pos = {cam.position[0], cam.position[1], cam.position[2], 0.0f};
    u.cam_right = {cam.basis[0], cam.basis[1], cam.basis[2], 0.0f};
    u.cam_up = {cam.basis[3], cam.basis[4], cam.basis[5], 0.0f};
    u.cam_fwd = {-cam.basis[6], -cam.basis[7], -cam.basis[8], 0.0f};
    u.tan_half_fov = std::tan(0.5f * cam.fov_y_radians);
    u.aspect = float(w) / float(h);
    u.mass_M = scene.mass_solar;
    u.spin_a = scene.spin_a_over_M * scene.mass_solar;
    u.rs = 2.0f * scene.mass_solar;
    u.disc_r_inner = scene.disc_inner_M * scene.mass_solar;
    u.disc_r_outer = scene.disc_outer_M * scene.mass_solar;
    u.disc_peak_T = scene.disc_peak_T_K;
    u.h_step = scene.h_step > 0.0f ? scene.h_step : kHStep;
    u.escape_r = 200.0f * scene.mass_solar;
    u.horizon_cut = 1.02f * u.rs;
    u.time_sec = time_sec;
    u.width = w;
    u.height = h;
    u.metric_type = scene.metric == Scene::MetricType::Kerr ? SGX_METRIC_KERR : SGX_METRIC_SCHWARZSCHILD;
    std::uint32_t flags = SGX_FLAG_STARFIELD_ON;
    if (scene.disc_texture_on) flags |= SGX_FLAG_DISC_ON;
    if (scene.disc_doppler_on) flags |= SGX_FLAG_DOPPLER_ON;
    if (scene.disc_redshift_on) flags |= SGX_FLAG_REDSHIFT_ON;
    // adaptive_step_on (render_backend.hpp:78-81) is honoured as the WebGPU
    // backend does (webgpu_backend.cpp:159-160); the reference CUDA backend
    // drops it.  Off by default, so default scenes pack identically.
    if (scene.adaptive_step_on) flags |= SGX_FLAG_ADAPTIVE_STEP;
    u.flags = flags;
    u.max_steps = scene.max_steps != 0 ? scene.max_steps : kMaxSteps;
    u.frame_index = 0;
    u.supersample = scene.render_supersample == 0 ? 1u : scene.render_supersample;
    u.pad_b = 0;
    u.exposure = scene.exposure;
    u.bloom_threshold = scene.bloom_threshold;
    u.bloom_strength = scene.bloom_strength;
    u.disc_turbulence = scene.disc_turbulence;
    return u;
}

float kerr_isco_prograde(float mass, float spin) {
    const float x = spin / mass;
    const float x2 = x * x;
    const float z1 = 1.0f + std::cbrt(1.0f - x2) * (std::cbrt(1.0f + x) + std::cbrt(1.0f - x));
    const float z2 = std::sqrt(3.0f * x2 + z1 * z1);
    const float rad = (3.0f - z1) * (3.0f + z1 + 2.0f * z2);
    return mass * (3.0f + z2 - std::sqrt(rad > 0.0f ? rad : 0.0f));
}

sgx_scene to_c(const Scene& s) {
    sgx_scene c{};
    c.metric = static_cast<std::uint32_t>(s.metric);
    c.mass_solar = s.mass_solar;
    c.spin_a_over_M = s.spin_a_over_M;
    c.disc_inner_M = s.disc_inner_M;
    c.disc_outer_M = s.disc_outer_M;
    c.disc_doppler_on = s.disc_doppler_on;
    c.disc_redshift_on = s.disc_redshift_on;
    c.disc_texture_on = s.disc_texture_on;
    c.show_overlay = s.show_overlay;
    c.render_supersample = s.render_supersample;
    c.exposure = s.exposure;
    c.bloom_threshold = s.bloom_threshold;
    c.bloom_strength = s.bloom_strength;
    c.disc_turbulence = s.disc_turbulence;
    c.disc_peak_T_K = s.disc_peak_T_K;
    c.max_steps = s.max_steps;
    c.h_step = s.h_step;
    c.adaptive_step_on = s.adaptive_step_on;
    return c;
}

Scene from_c(const sgx_scene& c) {
    Scene s;
    s.metric = c.metric == SGX_METRIC_KERR ? Scene::MetricType::Kerr : Scene::MetricType::Schwarzschild;
    s.mass_solar = c.mass_solar;
    s.spin_a_over_M = c.spin_a_over_M;
    s.disc_inner_M = c.disc_inner_M;
    s.disc_outer_M = c.disc_outer_M;
    s.disc_doppler_on = c.disc_doppler_on != 0;
    s.disc_redshift_on = c.disc_redshift_on != 0;
    s.disc_texture_on = c.disc_texture_on != 0;
    s.show_overlay = c.show_overlay != 0;
    s.render_supersample = c.render_supersample;
    s.exposure = c.exposure;
    s.bloom_threshold = c.bloom_threshold;
    s.bloom_strength = c.bloom_strength;
    s.disc_turbulence = c.disc_turbulence;
    s.disc_peak_T_K = c.disc_peak_T_K;
    s.max_steps = c.max_steps;
    s.h_step = c.h_step;
    s.adaptive_step_on = c.adaptive_step_on != 0;
    return s;
}

}  // namespace sgx

// ---------------------------------------------------------------------------
// C ABI: host helpers
// ---------------------------------------------------------------------------
namespace {

void copy_err(char* buf, std::size_t len, const std::string& s) {
    if (buf == nullptr || len == 0) return;
    const std::size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
}

sgx_scene_config cfg_to_c(const sgx::SceneConfig& c) {
    sgx_scene_config o{};
    o.mass = c.mass;
    o.spin = c.spin;
    o.disc_r_inner = c.disc_r_inner;
    o.disc_r_outer = c.disc_r_outer;
    o.disc_doppler_on = c.disc_doppler_on;
    o.disc_redshift_on = c.disc_redshift_on;
    o.camera_fov_deg = c.camera_fov_deg;
    o.camera_distance = c.camera_distance;
    o.camera_elevation = c.camera_elevation;
    o.h_step = c.h_step;
    o.max_steps = c.max_steps;
    return o;
}

sgx::SceneConfig cfg_from_c(const sgx_scene_config& o) {
    sgx::SceneConfig c;
    c.mass = o.mass;
    c.spin = o.spin;
    c.disc_r_inner = o.disc_r_inner;
    c.disc_r_outer = o.disc_r_outer;
    c.disc_doppler_on = o.disc_doppler_on != 0;
    c.disc_redshift_on = o.disc_redshift_on != 0;
    c.camera_fov_deg = o.camera_fov_deg;
    c.camera_distance = o.camera_distance;
    c.camera_elevation = o.camera_elevation;
    c.h_step = o.h_step;
    c.max_steps = o.max_steps;
    return c;
}

sgx_scene_status finish_load(const sgx::SceneLoadResult& r, const sgx::SceneConfig& c, sgx_scene_config* out,
                             int* line, char* errbuf, std::size_t errlen) {
    if (line != nullptr) *line = r.line_number;
    copy_err(errbuf, errlen, r.error_line);
    // Keys parsed before an error stay applied, as in the reference loader.
    *out = cfg_to_c(c);
    switch (r.status) {
        case sgx::SceneLoadStatus::Ok: return SGX_SCENE_OK;
        case sgx::SceneLoadStatus::FileNotFound: return SGX_SCENE_FILE_NOT_FOUND;
        case sgx::SceneLoadStatus::UnknownKey: return SGX_SCENE_UNKNOWN_KEY;
        default: return SGX_SCENE_PARSE_ERROR;
    }
}

}  // namespace

extern "C" {

void sgx_scene_default(sgx_scene* out) {
    if (out != nullptr) *out = sgx::to_c(sgx::Scene{});
}

void sgx_build_orbital_camera(sgx_camera* cam, float distance_M, float elevation_rad, float azimuth_rad,
                              float fov_y_deg) {
    if (cam == nullptr) return;
    sgx::CameraState c;
    sgx::build_orbital_camera(c, distance_M, elevation_rad, azimuth_rad, fov_y_deg);
    std::memcpy(cam->position, c.position, sizeof(c.position));
    std::memcpy(cam->basis, c.basis, sizeof(c.basis));
    cam->fov_y_radians = c.fov_y_radians;
}

void sgx_pack_uniforms(const sgx_scene* scene, const sgx_camera* cam, uint32_t width, uint32_t height,
                       float time_sec, sgx_uniforms* out) {
    if (scene == nullptr || cam == nullptr || out == nullptr) return;
    sgx::CameraState c;
    std::memcpy(c.position, cam->position, sizeof(c.position));
    std::memcpy(c.basis, cam->basis, sizeof(c.basis));
    c.fov_y_radians = cam->fov_y_radians;
    *out = sgx::pack_uniforms(sgx::from_c(*scene), c, width, height, time_sec);
}

void sgx_scene_config_default(sgx_scene_config* out) {
    if (out != nullptr) *out = cfg_to_c(sgx::SceneConfig{});
}

sgx_scene_status sgx_scene_config_load_file(const char* path, sgx_scene_config* out, int* line, char* errbuf,
                                            size_t errbuf_len) {
    if (path == nullptr || out == nullptr) return SGX_SCENE_FILE_NOT_FOUND;
    sgx::SceneConfig c = cfg_from_c(*out);
    const sgx::SceneLoadResult r = sgx::load_scene_config_from_file(path, c);
    return finish_load(r, c, out, line, errbuf, errbuf_len);
}

sgx_scene_status sgx_scene_config_load_string(const char* text, sgx_scene_config* out, int* line, char* errbuf,
                                              size_t errbuf_len) {
    if (text == nullptr || out == nullptr) return SGX_SCENE_PARSE_ERROR;
    sgx::SceneConfig c = cfg_from_c(*out);
    std::istringstream in{std::string(text)};
    const sgx::SceneLoadResult r = sgx::load_scene_config_from_stream(in, c);
    return finish_load(r, c, out, line, errbuf, errbuf_len);
}

float sgx_kerr_isco_prograde(float mass, float spin) { return sgx::kerr_isco_prograde(mass, spin); }

}  // extern "C"
