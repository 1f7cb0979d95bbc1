// singularity_gb300/csrc/cli_main.cpp
//
// singularity_cuda_cli: the offline renderer's command line, drop-in for the
// reference's cuda_cli/main.cpp — the same flags, defaults, scene mapping,
// messages and exit codes (2 for usage and scene errors, 1 for runtime
// errors), over the GB300 library.
//
// Kept from the reference on purpose (cuda_cli/main.cpp:193-237): without
// --scene the scene is the render_backend.hpp default (Kerr a/M = 0.6); from
// a .scene file only mass, spin, disc_r_inner/outer, Doppler and redshift are
// used, metric = Kerr iff spin > 0; the scene's camera, h_step and max_steps
// keys are ignored unless --use-scene-camera / --use-scene-integrator ask.
//
// Additions (all off by default): integrator and precision forms, tolerance,
// peak temperature, exposure, turbulence, step/budget overrides, disc inner
// edge at the ISCO, and a float output (.pfm).  PNG encoding and file writes
// of frame k run on a writer thread while frame k+1 renders.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <string>
#include <string_view>
#include <vector>

#include "cuda_backend.hpp"
#include "sgx_host.hpp"

namespace {

void print_help() {
    std::puts(
        "singularity_cuda_cli - offline geodesic renderer (GB300)\n"
        "\n"
        "Usage:\n"
        "  singularity_cuda_cli [--scene PATH] [--output PATH] [--res WxH]\n"
        "                       [--samples-per-pixel N]\n"
        "                       [--camera-distance M] [--camera-elevation R]\n"
        "                       [--camera-azimuth R] [--fov-y-deg D]\n"
        "                       [--frames N --output-pattern PATTERN]\n"
        "\n"
        "Options:\n"
        "  --scene PATH           Scene config (key = value; mass, spin, disc_r_inner, ...).\n"
        "  --output PATH          PNG written for a single frame (default cuda_render.png).\n"
        "  --res WxH              Image size (default 1280x720).\n"
        "  --samples-per-pixel N  Halton(2,3) samples per pixel, 1..1024 (default 1).\n"
        "  --camera-distance M    Orbit radius in M (default 30).\n"
        "  --camera-elevation R   Elevation above the equator, radians (default 0.15).\n"
        "  --camera-azimuth R     Starting azimuth, radians (default 0).\n"
        "  --fov-y-deg D          Vertical field of view in degrees (default 60).\n"
        "  --frames N             N frames orbiting 2 pi in azimuth (default 1).\n"
        "  --output-pattern P     printf pattern with one %d / %0Nd for the frame index;\n"
        "                         required when --frames > 1.\n"
        "  --encode-mp4 PATH      After the last frame, run ffmpeg (libx264, yuv420p, crf 18)\n"
        "                         on the sequence; needs --frames > 1 and ffmpeg on PATH.\n"
        "  --mp4-fps N            Frame rate for --encode-mp4 (default 30).\n"
        "\n"
        "Extensions (defaults reproduce the options above exactly):\n"
        "  --integrator fixed|adaptive   fixed-step RK4 (default) or error-controlled RK4\n"
        "  --precision fp32|mixed|fp64   arithmetic form (mixed: adaptive only)\n"
        "  --tolerance T                 adaptive error tolerance (default 1e-6)\n"
        "  --rhs-form 0|1|2              Kerr right-hand side: 0 separated form (default),\n"
        "                                1 the reference's divisions, 2 form 0 with sin/cos of\n"
        "                                theta carried in the fixed-step state (FP32)\n"
        "  --peak-temp K                 disc peak temperature (default 4500)\n"
        "  --exposure X                  exposure before tone mapping (default 1.8)\n"
        "  --turbulence X                disc band amplitude (default 0.5)\n"
        "  --h-step H / --max-steps N    integrator step and budget (default 0.4 / 2500)\n"
        "  --adaptive-step               radius-adaptive fixed step h * clamp(r / 6M, 1, 40)\n"
        "  --turbulence-seed N           disc band phase of seed N (first frame at time N/30 s)\n"
        "  --bloom                       bloom + blit post-process (half-float HDR, the 7-tap kernel)\n"
        "  --bloom-sigma PX              ... with a Gaussian of PX pixels instead\n"
        "  --disc-inner-isco             disc inner edge at the prograde ISCO of the spin\n"
        "  --use-scene-camera            take camera_distance/elevation/fov from the scene file\n"
        "  --use-scene-integrator        take h_step/max_steps from the scene file\n"
        "  --pfm                         also write the float image (LDR mean) as .pfm\n"
        "\n"
        "Manual encode (same as --encode-mp4):\n"
        "  ffmpeg -framerate 30 -i frames/frame_%04d.png -c:v libx264 \\\n"
        "         -pix_fmt yuv420p -crf 18 kerr.mp4\n");
}

// --- PNG (stored deflate blocks, no compression library) -------------------
// CRC-32 (reflected, polynomial 0xEDB88320) by slicing-by-8: eight 256-entry
// tables, eight input bytes per iteration.
struct Crc32 {
    std::uint32_t t[8][256];
    Crc32() {
        for (std::uint32_t i = 0; i < 256; ++i) {
            std::uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1u) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            t[0][i] = v;
        }
        for (std::uint32_t i = 0; i < 256; ++i)
            for (int k = 1; k < 8; ++k) t[k][i] = (t[k - 1][i] >> 8) ^ t[0][t[k - 1][i] & 0xFFu];
    }
    // c: running value (start 0xFFFFFFFF; the stored CRC is c ^ 0xFFFFFFFF)
    std::uint32_t update(std::uint32_t c, const unsigned char* p, std::size_t n) const {
        while (n >= 8) {
            const std::uint32_t lo = c ^ (std::uint32_t(p[0]) | std::uint32_t(p[1]) << 8 | std::uint32_t(p[2]) << 16 |
                                          std::uint32_t(p[3]) << 24);
            const std::uint32_t hi =
                std::uint32_t(p[4]) | std::uint32_t(p[5]) << 8 | std::uint32_t(p[6]) << 16 | std::uint32_t(p[7]) << 24;
            c = t[7][lo & 0xFFu] ^ t[6][(lo >> 8) & 0xFFu] ^ t[5][(lo >> 16) & 0xFFu] ^ t[4][lo >> 24] ^
                t[3][hi & 0xFFu] ^ t[2][(hi >> 8) & 0xFFu] ^ t[1][(hi >> 16) & 0xFFu] ^ t[0][hi >> 24];
            p += 8;
            n -= 8;
        }
        while (n-- > 0) c = t[0][(c ^ *p++) & 0xFFu] ^ (c >> 8);
        return c;
    }
};

const Crc32& crc_tables() {
    static const Crc32 t;
    return t;
}

// Adler-32 with the modulo deferred over runs of 5552 bytes (the longest run
// whose sums cannot overflow 32 bits).
void adler_update(std::uint32_t& a, std::uint32_t& b, const unsigned char* p, std::size_t n) {
    while (n > 0) {
        std::size_t k = n < 5552 ? n : 5552;
        n -= k;
        while (k-- > 0) {
            a += *p++;
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
    }
}

void put32(std::vector<unsigned char>& o, std::uint32_t v) {
    o.push_back(static_cast<unsigned char>(v >> 24));
    o.push_back(static_cast<unsigned char>(v >> 16));
    o.push_back(static_cast<unsigned char>(v >> 8));
    o.push_back(static_cast<unsigned char>(v));
}

void chunk(std::vector<unsigned char>& o, const char* type, const std::vector<unsigned char>& body) {
    put32(o, std::uint32_t(body.size()));
    const std::size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), body.begin(), body.end());
    put32(o, crc_tables().update(0xFFFFFFFFu, o.data() + start, o.size() - start) ^ 0xFFFFFFFFu);
}

// RGBA8 image as a PNG: filter 0 on every row, the zlib stream as stored
// (uncompressed) deflate blocks of at most 65535 bytes; the IDAT chunk is
// assembled in one buffer (one copy of the pixels) and checksummed once.
bool write_png_rgba8(const char* path, const std::uint8_t* px, std::uint32_t w, std::uint32_t h) {
    const std::size_t rowb = std::size_t(w) * 4;
    const std::size_t raw_n = (rowb + 1) * h;  // filter byte + pixels, per row
    const std::size_t nblk = raw_n == 0 ? 1 : (raw_n + 65534) / 65535;
    const std::size_t idat_n = 2 + 5 * nblk + raw_n + 4;
    if (idat_n > 0x7FFFFFFFu) return false;  // a PNG chunk holds at most 2^31 - 1 bytes
    std::vector<unsigned char> idat(8 + idat_n + 4);
    unsigned char* q = idat.data();
    auto be32 = [](unsigned char* d, std::uint32_t v) {
        d[0] = static_cast<unsigned char>(v >> 24);
        d[1] = static_cast<unsigned char>(v >> 16);
        d[2] = static_cast<unsigned char>(v >> 8);
        d[3] = static_cast<unsigned char>(v);
    };
    be32(q, std::uint32_t(idat_n));
    q[4] = 'I';
    q[5] = 'D';
    q[6] = 'A';
    q[7] = 'T';
    unsigned char* d = q + 8;
    *d++ = 0x78;
    *d++ = 0x01;
    // the raw stream (row r: filter byte 0, then rowb pixel bytes) cut into blocks
    std::uint32_t a = 1, b = 0;
    std::size_t left = raw_n, row = 0, in_row = 0;  // in_row 0: the filter byte is next
    const unsigned char zero = 0;
    do {
        const std::size_t n = left < 65535 ? left : 65535;
        left -= n;
        *d++ = left == 0 ? 1 : 0;
        *d++ = static_cast<unsigned char>(n & 0xFF);
        *d++ = static_cast<unsigned char>(n >> 8);
        *d++ = static_cast<unsigned char>(~n & 0xFF);
        *d++ = static_cast<unsigned char>((~n >> 8) & 0xFF);
        for (std::size_t k = n; k > 0;) {
            if (in_row == 0) {
                *d++ = 0;
                adler_update(a, b, &zero, 1);
                in_row = 1;
                --k;
                continue;
            }
            const std::size_t take = std::min(k, rowb - (in_row - 1));
            const unsigned char* src = px + row * rowb + (in_row - 1);
            std::memcpy(d, src, take);
            adler_update(a, b, src, take);
            d += take;
            k -= take;
            in_row += take;
            if (in_row == rowb + 1) {
                in_row = 0;
                ++row;
            }
        }
    } while (left > 0);
    be32(d, (b << 16) | a);
    d += 4;
    be32(d, crc_tables().update(0xFFFFFFFFu, q + 4, 4 + idat_n) ^ 0xFFFFFFFFu);
    std::vector<unsigned char> head = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<unsigned char> ihdr;
    put32(ihdr, w);
    put32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    chunk(head, "IHDR", ihdr);
    std::vector<unsigned char> tail;
    chunk(tail, "IEND", {});
    std::FILE* f = std::fopen(path, "wb");
    if (f == nullptr) return false;
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    ok = ok && std::fwrite(idat.data(), 1, idat.size(), f) == idat.size();
    ok = ok && std::fwrite(tail.data(), 1, tail.size(), f) == tail.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok;
}

bool write_pfm(const char* path, const std::vector<float>& rgba, std::uint32_t w, std::uint32_t h) {
    std::FILE* f = std::fopen(path, "wb");
    if (f == nullptr) return false;
    std::fprintf(f, "PF\n%u %u\n-1.0\n", w, h);
    std::vector<float> row(std::size_t(w) * 3);
    bool ok = true;
    for (std::uint32_t y = h; y-- > 0;) {  // PFM rows run bottom to top
        for (std::uint32_t x = 0; x < w; ++x)
            for (int c = 0; c < 3; ++c) row[std::size_t(x) * 3 + c] = rgba[(std::size_t(y) * w + x) * 4 + c];
        ok = ok && std::fwrite(row.data(), sizeof(float), row.size(), f) == row.size();
    }
    return (std::fclose(f) == 0) && ok;
}

}  // namespace

int main(int argc, char** argv) {
    std::string scene_path;
    std::string output_path = "cuda_render.png";
    std::uint32_t width = 1280, height = 720;
    float camera_distance = 30.0f, camera_elevation = 0.15f, camera_azimuth = 0.0f, fov_y_deg = 60.0f;
    std::uint32_t samples_per_pixel = 1, frames = 1, mp4_fps = 30;
    std::string output_pattern, encode_mp4_path;
    // extensions
    sgx_render_opts opts;
    sgx_render_opts_default(&opts);
    bool have_opts = false, isco_inner = false, scene_camera = false, scene_integrator = false, pfm = false, adaptive_step = false;
    bool bloom = false, have_seed = false;
    float bloom_sigma = 0.0f;
    long turbulence_seed = 0;
    float peak_temp = -1.0f, exposure = -1.0f, turbulence = -1.0f, h_step = 0.0f;
    std::uint32_t max_steps = 0;

    for (int i = 1; i < argc; ++i) {
        const std::string_view a = argv[i];
        const bool has_val = i + 1 < argc;
        if (a == "--help" || a == "-h") {
            print_help();
            return 0;
        }
        if (a == "--scene" && has_val) {
            scene_path = argv[++i];
        } else if (a == "--output" && has_val) {
            output_path = argv[++i];
        } else if (a == "--res" && has_val) {
            const char* v = argv[++i];
            const char* x = std::strchr(v, 'x');
            if (x == nullptr) {
                std::fprintf(stderr, "singularity_cuda_cli: --res expects WxH, got %s\n", v);
                return 2;
            }
            width = static_cast<std::uint32_t>(std::strtoul(v, nullptr, 10));
            height = static_cast<std::uint32_t>(std::strtoul(x + 1, nullptr, 10));
            if (width < 4 || height < 4) {
                std::fprintf(stderr, "singularity_cuda_cli: --res too small\n");
                return 2;
            }
        } else if (a == "--camera-distance" && has_val) {
            camera_distance = std::strtof(argv[++i], nullptr);
        } else if (a == "--camera-elevation" && has_val) {
            camera_elevation = std::strtof(argv[++i], nullptr);
        } else if (a == "--camera-azimuth" && has_val) {
            camera_azimuth = std::strtof(argv[++i], nullptr);
        } else if (a == "--fov-y-deg" && has_val) {
            fov_y_deg = std::strtof(argv[++i], nullptr);
        } else if (a == "--samples-per-pixel" && has_val) {
            const unsigned long v = std::strtoul(argv[++i], nullptr, 10);
            if (v < 1ul || v > 1024ul) {
                std::fprintf(stderr, "singularity_cuda_cli: --samples-per-pixel must be in [1, 1024]\n");
                return 2;
            }
            samples_per_pixel = static_cast<std::uint32_t>(v);
        } else if (a == "--frames" && has_val) {
            const unsigned long v = std::strtoul(argv[++i], nullptr, 10);
            if (v < 1ul || v > 100000ul) {
                std::fprintf(stderr, "singularity_cuda_cli: --frames must be in [1, 100000]\n");
                return 2;
            }
            frames = static_cast<std::uint32_t>(v);
        } else if (a == "--output-pattern" && has_val) {
            output_pattern = argv[++i];
        } else if (a == "--encode-mp4" && has_val) {
            encode_mp4_path = argv[++i];
        } else if (a == "--mp4-fps" && has_val) {
            const unsigned long v = std::strtoul(argv[++i], nullptr, 10);
            if (v < 1ul || v > 240ul) {
                std::fprintf(stderr, "singularity_cuda_cli: --mp4-fps must be in [1, 240]\n");
                return 2;
            }
            mp4_fps = static_cast<std::uint32_t>(v);
        } else if (a == "--integrator" && has_val) {
            const std::string_view v = argv[++i];
            if (v != "fixed" && v != "adaptive") {
                std::fprintf(stderr, "singularity_cuda_cli: --integrator must be fixed or adaptive\n");
                return 2;
            }
            opts.integrator = v == "adaptive" ? SGX_INTEGRATOR_ADAPTIVE : SGX_INTEGRATOR_FIXED;
            have_opts = true;
        } else if (a == "--precision" && has_val) {
            const std::string_view v = argv[++i];
            if (v == "fp32") opts.precision = SGX_PRECISION_FP32;
            else if (v == "mixed") opts.precision = SGX_PRECISION_MIXED;
            else if (v == "fp64") opts.precision = SGX_PRECISION_FP64;
            else {
                std::fprintf(stderr, "singularity_cuda_cli: --precision must be fp32, mixed or fp64\n");
                return 2;
            }
            have_opts = true;
        } else if (a == "--tolerance" && has_val) {
            opts.tolerance = std::strtof(argv[++i], nullptr);
            have_opts = true;
        } else if (a == "--rhs-form" && has_val) {
            const std::string_view v = argv[++i];
            if (v != "0" && v != "1" && v != "2") {
                std::fprintf(stderr, "singularity_cuda_cli: --rhs-form must be 0, 1 or 2\n");
                return 2;
            }
            opts.rhs_form = std::uint32_t(v[0] - '0');
            have_opts = true;
        } else if (a == "--peak-temp" && has_val) {
            peak_temp = std::strtof(argv[++i], nullptr);
        } else if (a == "--exposure" && has_val) {
            exposure = std::strtof(argv[++i], nullptr);
        } else if (a == "--turbulence" && has_val) {
            turbulence = std::strtof(argv[++i], nullptr);
        } else if (a == "--h-step" && has_val) {
            h_step = std::strtof(argv[++i], nullptr);
        } else if (a == "--max-steps" && has_val) {
            max_steps = static_cast<std::uint32_t>(std::strtoul(argv[++i], nullptr, 10));
        } else if (a == "--adaptive-step") {
            adaptive_step = true;
        } else if (a == "--turbulence-seed" && has_val) {
            turbulence_seed = std::strtol(argv[++i], nullptr, 10);
            have_seed = true;
        } else if (a == "--bloom") {
            bloom = true;
        } else if (a == "--bloom-sigma" && has_val) {
            bloom = true;
            bloom_sigma = std::strtof(argv[++i], nullptr);
        } else if (a == "--disc-inner-isco") {
            isco_inner = true;
        } else if (a == "--use-scene-camera") {
            scene_camera = true;
        } else if (a == "--use-scene-integrator") {
            scene_integrator = true;
        } else if (a == "--pfm") {
            pfm = true;
        } else {
            std::fprintf(stderr, "singularity_cuda_cli: unknown argument: %.*s\n", int(a.size()), a.data());
            print_help();
            return 2;
        }
    }

    singularity::Scene scene{};
    if (!scene_path.empty()) {
        sgx::SceneConfig cfg;
        const auto res = sgx::load_scene_config_from_file(scene_path, cfg);
        using S = sgx::SceneLoadStatus;
        if (res.status != S::Ok) {
            const char* reason = res.status == S::FileNotFound  ? "file-not-found"
                                 : res.status == S::UnknownKey ? "unknown-key"
                                                               : "parse-error";
            std::fprintf(stderr, "singularity_cuda_cli: scene load failed (%s, line %d): %s\n", reason,
                         res.line_number, res.error_line.c_str());
            return 2;
        }
        scene.mass_solar = cfg.mass;
        scene.spin_a_over_M = cfg.spin;
        scene.disc_inner_M = cfg.disc_r_inner;
        scene.disc_outer_M = cfg.disc_r_outer;
        scene.disc_doppler_on = cfg.disc_doppler_on;
        scene.disc_redshift_on = cfg.disc_redshift_on;
        scene.metric = (cfg.spin > 0.0f) ? singularity::Scene::MetricType::Kerr
                                         : singularity::Scene::MetricType::Schwarzschild;
        if (scene_camera) {
            camera_distance = cfg.camera_distance;
            camera_elevation = cfg.camera_elevation;
            fov_y_deg = cfg.camera_fov_deg;
        }
        if (scene_integrator) {
            scene.h_step = cfg.h_step;
            scene.max_steps = cfg.max_steps > 0 ? std::uint32_t(cfg.max_steps) : 0u;
        }
        if (cfg.disc_r_inner < 0.0f && isco_inner) scene.disc_inner_M = sgx::kerr_isco_prograde(1.0f, cfg.spin);
    }
    scene.render_supersample = samples_per_pixel;
    if (isco_inner) scene.disc_inner_M = sgx::kerr_isco_prograde(1.0f, scene.spin_a_over_M);
    if (peak_temp > 0.0f) scene.disc_peak_T_K = peak_temp;
    if (exposure >= 0.0f) scene.exposure = exposure;
    if (turbulence >= 0.0f) scene.disc_turbulence = turbulence;
    if (h_step > 0.0f) scene.h_step = h_step;
    if (adaptive_step) scene.adaptive_step_on = true;
    if (max_steps > 0) scene.max_steps = max_steps;

    if (bloom && !(bloom_sigma >= 0.0f && bloom_sigma <= 64.0f)) {
        std::fprintf(stderr, "singularity_cuda_cli: --bloom-sigma must be in [0, 64]\n");
        return 2;
    }
    if (frames > 1 && output_pattern.empty()) {
        std::fprintf(stderr,
                     "singularity_cuda_cli: --frames > 1 requires --output-pattern with a "
                     "printf-style %%d placeholder, e.g. frames/frame_%%04d.png\n");
        return 2;
    }
    if (frames > 1 && output_pattern.find('%') == std::string::npos) {
        std::fprintf(stderr,
                     "singularity_cuda_cli: --output-pattern must contain a printf placeholder "
                     "(%%d / %%04d)\n");
        return 2;
    }
    if (!encode_mp4_path.empty() && frames < 2) {
        std::fprintf(stderr,
                     "singularity_cuda_cli: --encode-mp4 requires --frames > 1 (a sequence to "
                     "encode)\n");
        return 2;
    }

    singularity::RenderConfig rcfg{};
    rcfg.width = width;
    rcfg.height = height;
    singularity::CudaBackend backend;
    if (!backend.initialize(singularity::WindowHandle{}, rcfg)) {
        std::fprintf(stderr, "singularity_cuda_cli: backend initialize failed\n");
        return 1;
    }
    if (have_opts) backend.set_render_options(opts);
    if (bloom) backend.set_bloom(bloom_sigma);
    if (have_seed) backend.set_frame_time(float(turbulence_seed) / 30.0f);

    constexpr float kTwoPi = 6.28318530717958647693f;
    std::future<bool> pending;
    std::string pending_path;
    auto finish_pending = [&]() -> bool {
        if (!pending.valid()) return true;
        if (!pending.get()) {
            std::fprintf(stderr, "singularity_cuda_cli: failed to write '%s'\n", pending_path.c_str());
            return false;
        }
        return true;
    };

    for (std::uint32_t f = 0; f < frames; ++f) {
        const float az = camera_azimuth + (frames > 1 ? (kTwoPi * float(f) / float(frames)) : 0.0f);
        sgx_camera cc{};
        sgx_build_orbital_camera(&cc, camera_distance, camera_elevation, az, fov_y_deg);
        singularity::CameraState camera{};
        for (int i = 0; i < 3; ++i) camera.position[i] = cc.position[i];
        for (int i = 0; i < 9; ++i) camera.basis[i] = cc.basis[i];
        camera.fov_y_radians = cc.fov_y_radians;
        backend.render_frame(scene, camera);  // overlaps the previous frame's write
        auto img = std::make_shared<singularity::ImageData>(backend.capture_frame());
        if (img->pixels_rgba.empty() || img->width == 0 || img->height == 0) {
            std::fprintf(stderr, "singularity_cuda_cli: empty capture (frame %u)\n", f);
            finish_pending();
            backend.shutdown();
            return 1;
        }
        if (!finish_pending()) {
            backend.shutdown();
            return 1;
        }
        char path_buf[1024];
        if (frames > 1) std::snprintf(path_buf, sizeof(path_buf), output_pattern.c_str(), int(f));
        else std::snprintf(path_buf, sizeof(path_buf), "%s", output_path.c_str());
        pending_path = path_buf;
        if (pfm) {
            // The same frame's tone-mapped mean before sRGB, as floats.
            const std::vector<float> fimg = backend.capture_frame_float();
            std::string fpath = pending_path;
            const auto dot = fpath.rfind('.');
            fpath = (dot == std::string::npos ? fpath : fpath.substr(0, dot)) + ".pfm";
            if (fimg.empty() || !write_pfm(fpath.c_str(), fimg, width, height)) {
                std::fprintf(stderr, "singularity_cuda_cli: failed to write '%s'\n", fpath.c_str());
                backend.shutdown();
                return 1;
            }
        }
        pending = std::async(std::launch::async, [img, path = pending_path, f, frames]() {
            if (!write_png_rgba8(path.c_str(), img->pixels_rgba.data(), img->width, img->height)) return false;
            if (frames > 1) {
                std::printf("wrote %s (%ux%u, frame %u/%u, CUDA)\n", path.c_str(), img->width, img->height, f + 1,
                            frames);
                std::fflush(stdout);
            } else {
                std::printf("wrote %s (%ux%u, CUDA)\n", path.c_str(), img->width, img->height);
            }
            return true;
        });
    }
    if (!finish_pending()) {
        backend.shutdown();
        return 1;
    }
    backend.shutdown();

    if (!encode_mp4_path.empty()) {
        char cmd[2048];
        const int written = std::snprintf(cmd, sizeof(cmd),
                                          "ffmpeg -y -hide_banner -loglevel warning -framerate %u -i \"%s\" "
                                          "-c:v libx264 -pix_fmt yuv420p -crf 18 \"%s\"",
                                          mp4_fps, output_pattern.c_str(), encode_mp4_path.c_str());
        if (written < 0 || written >= int(sizeof(cmd))) {
            std::fprintf(stderr, "singularity_cuda_cli: ffmpeg command exceeded buffer (paths too long)\n");
            return 1;
        }
        std::printf("encoding: %s\n", cmd);
        std::fflush(stdout);
        const int rc = std::system(cmd);
        if (rc != 0) {
            std::fprintf(stderr,
                         "singularity_cuda_cli: ffmpeg exited %d -- is `ffmpeg` on PATH? "
                         "(see manual one-liner in --help)\n",
                         rc);
            return 1;
        }
        std::printf("wrote %s (%u frames at %u fps, libx264 crf=18 yuv420p)\n", encode_mp4_path.c_str(), frames,
                    mp4_fps);
    }
    return 0;
}
