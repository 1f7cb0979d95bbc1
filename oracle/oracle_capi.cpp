// oracle/oracle_capi.cpp
//
// TEST INFRASTRUCTURE — C entry points of the CPU oracle, loaded with ctypes
// by tests/, the smoke check and bench.py's CPU-baseline leg.  Never linked
// into the product.
//
// Every entry takes the 160-byte uniform block of the reference
// (shared_shader/uniforms.h:54-95) and runs the restatement in
// geodesic_oracle.hpp (FP32, FP64 or op-counting) across `threads` host
// threads, pixels or rays handed out through an atomic counter the way the
// reference CPU renderer hands out rows (cli/main.cpp:739-872).

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <thread>
#include <vector>

#include "adaptive_oracle.hpp"
#include "diff_oracle.hpp"
#include "geodesic_oracle.hpp"

namespace {

template <class F> void parallel_for(std::int64_t n, int threads, F&& body) {
    if (threads <= 1 || n < 64) {
        for (std::int64_t i = 0; i < n; ++i) body(i);
        return;
    }
    std::atomic<std::int64_t> next{0};
    const std::int64_t chunk = 16;
    auto worker = [&]() {
        for (;;) {
            const std::int64_t b = next.fetch_add(chunk);
            if (b >= n) break;
            const std::int64_t e = std::min(n, b + chunk);
            for (std::int64_t i = b; i < e; ++i) body(i);
        }
    };
    std::vector<std::thread> pool;
    const int nt = std::max(1, threads);
    pool.reserve(nt);
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

template <class T>
oracle::V3<T> pixel_ldr(std::uint32_t gx, std::uint32_t gy, const oracle::Params<T>& p,
                        const oracle::AdaptiveOpts* ad) {
    if (ad == nullptr) return oracle::shade_pixel(gx, gy, p);
    return oracle::shade_pixel_adaptive(gx, gy, p, *ad);
}

template <class T, class Out>
int render_pixels(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* pix, std::uint8_t* rgba8,
                  Out* ldr3, int threads, const oracle::AdaptiveOpts* ad) {
    if (u == nullptr || u->width == 0 || u->height == 0) return 1;
    const oracle::Params<T> p = oracle::promote<T>(*u);
    const std::int64_t npix = std::int64_t(u->width) * u->height;
    const std::int64_t count = (pix == nullptr) ? npix : n;
    parallel_for(count, threads, [&](std::int64_t i) {
        const std::int64_t idx = (pix == nullptr) ? i : std::int64_t(pix[i]);
        if (idx < 0 || idx >= npix) return;
        const std::uint32_t gx = std::uint32_t(idx % u->width);
        const std::uint32_t gy = std::uint32_t(idx / u->width);
        const oracle::V3<T> l = pixel_ldr(gx, gy, p, ad);
        if (rgba8 != nullptr) {
            rgba8[4 * i + 0] = oracle::to_u8(l.x);
            rgba8[4 * i + 1] = oracle::to_u8(l.y);
            rgba8[4 * i + 2] = oracle::to_u8(l.z);
            rgba8[4 * i + 3] = 255;
        }
        if (ldr3 != nullptr) {
            ldr3[3 * i + 0] = Out(l.x);
            ldr3[3 * i + 1] = Out(l.y);
            ldr3[3 * i + 2] = Out(l.z);
        }
    });
    return 0;
}

template <class T, class Out>
int trace_samples(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* gx, const std::uint32_t* gy,
                  const std::uint32_t* s, Out* hdr3, std::uint32_t* steps, std::uint32_t* term, int threads,
                  const oracle::AdaptiveOpts* ad, oracle::RayDiag* diag) {
    if (u == nullptr || gx == nullptr || gy == nullptr || s == nullptr) return 1;
    const oracle::Params<T> p = oracle::promote<T>(*u);
    parallel_for(n, threads, [&](std::int64_t i) {
        oracle::TraceOut<T> o;
        if (ad == nullptr) {
            o = oracle::trace_sample(gx[i], gy[i], s[i], p);
        } else {
            o = oracle::trace_sample_adaptive(gx[i], gy[i], s[i], p, *ad, diag ? &diag[i] : nullptr);
        }
        if (hdr3 != nullptr) {
            hdr3[3 * i + 0] = Out(o.hdr.x);
            hdr3[3 * i + 1] = Out(o.hdr.y);
            hdr3[3 * i + 2] = Out(o.hdr.z);
        }
        if (steps != nullptr) steps[i] = o.steps;
        if (term != nullptr) term[i] = o.term;
    });
    return 0;
}

}  // namespace

extern "C" {

int oracle_abi_version(void) { return 2; }

// Full-image or pixel-subset render (pix == nullptr -> every pixel, row-major).
int oracle_render_f32(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* pix, std::uint8_t* rgba8,
                      float* ldr3, int threads) {
    return render_pixels<float, float>(u, n, pix, rgba8, ldr3, threads, nullptr);
}
int oracle_render_f64(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* pix, std::uint8_t* rgba8,
                      double* ldr3, int threads) {
    return render_pixels<double, double>(u, n, pix, rgba8, ldr3, threads, nullptr);
}

// Individual samples (gx, gy, sample index) -> HDR colour, steps, termination.
int oracle_trace_f32(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* gx, const std::uint32_t* gy,
                     const std::uint32_t* s, float* hdr3, std::uint32_t* steps, std::uint32_t* term,
                     int threads) {
    return trace_samples<float, float>(u, n, gx, gy, s, hdr3, steps, term, threads, nullptr, nullptr);
}
int oracle_trace_f64(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* gx, const std::uint32_t* gy,
                     const std::uint32_t* s, double* hdr3, std::uint32_t* steps, std::uint32_t* term,
                     int threads) {
    return trace_samples<double, double>(u, n, gx, gy, s, hdr3, steps, term, threads, nullptr, nullptr);
}

// Algorithmic FP32 operation count of the reference formulas, per sample.
int oracle_count_ops(const sgx_uniforms* u, std::int64_t n, const std::uint32_t* gx, const std::uint32_t* gy,
                     const std::uint32_t* s, std::uint64_t* ops, std::uint32_t* steps, std::uint32_t* term,
                     const oracle::AdaptiveOpts* ad) {
    if (u == nullptr) return 1;
    const oracle::Params<oracle::Counted> p = oracle::promote<oracle::Counted>(*u);
    for (std::int64_t i = 0; i < n; ++i) {
        oracle::g_ops = 0;
        oracle::TraceOut<oracle::Counted> o;
        if (ad == nullptr) {
            o = oracle::trace_sample(gx[i], gy[i], s[i], p);
        } else {
            o = oracle::trace_sample_adaptive(gx[i], gy[i], s[i], p, *ad, nullptr);
        }
        // Per-sample display work: exposure scale + ACES (3 channels).
        (void)oracle::aces(oracle::vmul(o.hdr, p.exposure));
        ops[i] = oracle::g_ops;
        if (steps) steps[i] = o.steps;
        if (term) term[i] = o.term;
    }
    return 0;
}

// Adaptive-integrator variants (the extension in adaptive_oracle.hpp).
int oracle_render_adaptive_f32(const sgx_uniforms* u, const oracle::AdaptiveOpts* ad, std::int64_t n,
                               const std::uint32_t* pix, std::uint8_t* rgba8, float* ldr3, int threads) {
    if (ad == nullptr) return 1;
    return render_pixels<float, float>(u, n, pix, rgba8, ldr3, threads, ad);
}
int oracle_render_adaptive_f64(const sgx_uniforms* u, const oracle::AdaptiveOpts* ad, std::int64_t n,
                               const std::uint32_t* pix, std::uint8_t* rgba8, double* ldr3, int threads) {
    if (ad == nullptr) return 1;
    return render_pixels<double, double>(u, n, pix, rgba8, ldr3, threads, ad);
}
int oracle_trace_adaptive_f32(const sgx_uniforms* u, const oracle::AdaptiveOpts* ad, std::int64_t n,
                              const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s,
                              float* hdr3, std::uint32_t* steps, std::uint32_t* term, oracle::RayDiag* diag,
                              int threads) {
    if (ad == nullptr) return 1;
    return trace_samples<float, float>(u, n, gx, gy, s, hdr3, steps, term, threads, ad, diag);
}
int oracle_trace_adaptive_f64(const sgx_uniforms* u, const oracle::AdaptiveOpts* ad, std::int64_t n,
                              const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s,
                              double* hdr3, std::uint32_t* steps, std::uint32_t* term, oracle::RayDiag* diag,
                              int threads) {
    if (ad == nullptr) return 1;
    return trace_samples<double, double>(u, n, gx, gy, s, hdr3, steps, term, threads, ad, diag);
}

// ---- per-function entry points for the known-answer tests ----
// State layout: Kerr (t, r, theta, phi, p_r, p_theta); constants (E, L, Q, a, M).
#define ORACLE_KERR_FN(T, SUF)                                                                     \
    void oracle_kerr_rhs_##SUF(const T* y6, const T* c5, T* d6) {                                 \
        const oracle::KState<T> y{y6[0], y6[1], y6[2], y6[3], y6[4], y6[5]};                      \
        const oracle::KConst<T> c{c5[0], c5[1], c5[2], c5[3], c5[4]};                             \
        const oracle::KState<T> d = oracle::kerr_rhs(y, c);                                      \
        d6[0] = d.t; d6[1] = d.r; d6[2] = d.theta; d6[3] = d.phi; d6[4] = d.p_r; d6[5] = d.p_theta; \
    }                                                                                              \
    T oracle_kerr_two_H_##SUF(T r, T th, T pr, T pth, const T* c5) {                              \
        const oracle::KConst<T> c{c5[0], c5[1], c5[2], c5[3], c5[4]};                             \
        return oracle::kerr_two_H(r, th, pr, pth, c);                                            \
    }                                                                                              \
    void oracle_kerr_rk4_n_##SUF(T* y6, T h, const T* c5, std::int64_t n) {                       \
        oracle::KState<T> y{y6[0], y6[1], y6[2], y6[3], y6[4], y6[5]};                            \
        const oracle::KConst<T> c{c5[0], c5[1], c5[2], c5[3], c5[4]};                             \
        for (std::int64_t i = 0; i < n; ++i) y = oracle::kerr_rk4(y, h, c);                       \
        y6[0] = y.t; y6[1] = y.r; y6[2] = y.theta; y6[3] = y.phi; y6[4] = y.p_r; y6[5] = y.p_theta; \
    }
ORACLE_KERR_FN(float, f32)
ORACLE_KERR_FN(double, f64)

// Schwarzschild (t, r, theta, phi, u^t, u^r, u^theta, u^phi): n RK4 steps of h.
void oracle_schw_rk4_n_f32(float* y8, float h, float rs, std::int64_t n) {
    oracle::SState<float> y{y8[0], y8[1], y8[2], y8[3], y8[4], y8[5], y8[6], y8[7]};
    for (std::int64_t i = 0; i < n; ++i) y = oracle::schw_rk4(y, h, rs);
    const float o[8] = {y.t, y.r, y.theta, y.phi, y.ut, y.ur, y.utheta, y.uphi};
    for (int i = 0; i < 8; ++i) y8[i] = o[i];
}
void oracle_schw_rhs_f64(const double* y8, double rs, double* d8) {
    const oracle::SState<double> y{y8[0], y8[1], y8[2], y8[3], y8[4], y8[5], y8[6], y8[7]};
    const oracle::SState<double> d = oracle::schw_rhs(y, rs);
    const double o[8] = {d.t, d.r, d.theta, d.phi, d.ut, d.ur, d.utheta, d.uphi};
    for (int i = 0; i < 8; ++i) d8[i] = o[i];
}

// Integrates a Schwarzschild state with fixed h or the radius-adaptive step
// until r > r_out (test_adaptive_step.cpp:71-80); returns the steps taken, -1 if
// the budget ran out.  max_e / max_l get the largest relative drift of
// E = (1 - rs/r) u^t and L = r^2 sin^2(theta) u^phi along the way.
int oracle_schw_integrate_f32(float* y8, float h_base, float rs, float r_out, int adaptive, int budget,
                              float* max_e, float* max_l) {
    oracle::SState<float> y{y8[0], y8[1], y8[2], y8[3], y8[4], y8[5], y8[6], y8[7]};
    auto energy = [&](const oracle::SState<float>& s) { return (1.0f - rs / s.r) * s.ut; };
    auto ang = [&](const oracle::SState<float>& s) {
        const float st = std::sin(s.theta);
        return s.r * s.r * st * st * s.uphi;
    };
    const float E0 = energy(y), L0 = ang(y);
    float me = 0.0f, ml = 0.0f;
    int steps = -1;
    for (int i = 0; i < budget; ++i) {
        const float h = adaptive ? oracle::radius_adaptive_h(h_base, y.r, 0.5f * rs) : h_base;
        y = oracle::schw_rk4(y, h, rs);
        me = std::max(me, std::fabs(energy(y) - E0) / std::fabs(E0));
        ml = std::max(ml, std::fabs(ang(y) - L0) / std::fabs(L0));
        if (y.r > r_out) {
            steps = i + 1;
            break;
        }
    }
    const float o[8] = {y.t, y.r, y.theta, y.phi, y.ut, y.ur, y.utheta, y.uphi};
    for (int i = 0; i < 8; ++i) y8[i] = o[i];
    if (max_e) *max_e = me;
    if (max_l) *max_l = ml;
    return steps;
}

// Equatorial crossing (disc_intersection.h:30-55): returns crossed, writes frac.
int oracle_crossing_f32(float th_prev, float th_curr, float* frac) {
    const oracle::Crossing<float> x = oracle::equatorial_crossing(th_prev, th_curr);
    *frac = x.frac;
    return x.crossed ? 1 : 0;
}

// Spherical photon orbit radius for xi = L/E (adaptive_oracle.hpp).
double oracle_photon_orbit_radius(double a, double M, double xi) { return oracle::photon_orbit_radius<double>(a, M, xi); }

// Differentiable render form (diff_oracle.hpp): the LDR mean image, H*W*3.
int oracle_diff_render_f32(const sgx_uniforms* u, const oracle::DiffParams* p, const oracle::DiffOpts* o,
                           float* ldr3, int threads) {
    if (u == nullptr || p == nullptr || o == nullptr || ldr3 == nullptr) return 1;
    const std::int64_t npix = std::int64_t(u->width) * u->height;
    parallel_for(npix, threads, [&](std::int64_t i) {
        const auto l = oracle::diff_pixel<float>(*u, *p, *o, std::uint32_t(i % u->width), std::uint32_t(i / u->width));
        ldr3[3 * i] = l.x;
        ldr3[3 * i + 1] = l.y;
        ldr3[3 * i + 2] = l.z;
    });
    return 0;
}
int oracle_diff_render_f64(const sgx_uniforms* u, const oracle::DiffParams* p, const oracle::DiffOpts* o,
                           double* ldr3, int threads) {
    if (u == nullptr || p == nullptr || o == nullptr || ldr3 == nullptr) return 1;
    const std::int64_t npix = std::int64_t(u->width) * u->height;
    parallel_for(npix, threads, [&](std::int64_t i) {
        const auto l = oracle::diff_pixel<double>(*u, *p, *o, std::uint32_t(i % u->width), std::uint32_t(i / u->width));
        ldr3[3 * i] = l.x;
        ldr3[3 * i + 1] = l.y;
        ldr3[3 * i + 2] = l.z;
    });
    return 0;
}
// Per-sample HDR, steps and crossing count of the form.
int oracle_diff_trace_f64(const sgx_uniforms* u, const oracle::DiffParams* p, const oracle::DiffOpts* o,
                          std::int64_t n, const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s,
                          double* hdr3, std::uint32_t* steps, std::uint32_t* crossings, int threads) {
    if (u == nullptr || p == nullptr || o == nullptr) return 1;
    parallel_for(n, threads, [&](std::int64_t i) {
        const auto t = oracle::diff_trace<double>(*u, *p, *o, gx[i], gy[i], s[i]);
        if (hdr3) {
            hdr3[3 * i] = t.hdr.x;
            hdr3[3 * i + 1] = t.hdr.y;
            hdr3[3 * i + 2] = t.hdr.z;
        }
        if (steps) steps[i] = t.steps;
        if (crossings) crossings[i] = t.crossings;
    });
    return 0;
}

// Gradient of sum_px dL/dI . I with respect to (spin, incl, r_in, t_scale),
// I the form's LDR image, by forward-mode dual numbers over diff_trace
// (FP64).  dLdI is H*W*3; per-pixel terms are summed in pixel order.
int oracle_diff_grad_f64(const sgx_uniforms* u, const oracle::DiffParams* p, const oracle::DiffOpts* o,
                         const double* dLdI, double* grad4, double* ldr3, int threads) {
    if (u == nullptr || p == nullptr || o == nullptr || dLdI == nullptr || grad4 == nullptr) return 1;
    const std::int64_t npix = std::int64_t(u->width) * u->height;
    std::vector<double> part(std::size_t(npix) * 4, 0.0);
    parallel_for(npix, threads, [&](std::int64_t i) {
        double l[3], dl[3][4];
        oracle::diff_pixel_grad(*u, *p, *o, std::uint32_t(i % u->width), std::uint32_t(i / u->width), l, dl);
        for (int q = 0; q < 4; ++q)
            part[std::size_t(i) * 4 + q] = dLdI[3 * i] * dl[0][q] + dLdI[3 * i + 1] * dl[1][q] + dLdI[3 * i + 2] * dl[2][q];
        if (ldr3) {
            ldr3[3 * i] = l[0];
            ldr3[3 * i + 1] = l[1];
            ldr3[3 * i + 2] = l[2];
        }
    });
    for (int q = 0; q < 4; ++q) grad4[q] = 0.0;
    for (std::int64_t i = 0; i < npix; ++i)
        for (int q = 0; q < 4; ++q) grad4[q] += part[std::size_t(i) * 4 + q];
    return 0;
}

}  // extern "C"
