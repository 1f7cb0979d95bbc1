// oracle/geodesic_oracle.hpp
//
// TEST INFRASTRUCTURE — the CPU oracle of the geodesic tracer.  Nothing in the
// product (the CUDA library, the host mirror, the CLI) includes, links or
// calls this file; only tests/, the smoke check and bench.py's CPU-baseline
// leg load the shared library built from it, and only as the checker.
//
// A restatement, templated on the scalar type T, of the reference's per-pixel
// hot path:
//   * camera ray:      render/cuda/kernels/geodesic_kernel.cu:188-223
//   * Schwarzschild:   geodesic_kernel.cu:229-297 with the RHS and RK4 of
//                      shared_shader/geodesic_math.h:101-134
//   * Kerr:            geodesic_kernel.cu:303-403 with the Hamiltonian RHS and
//                      RK4 of shared_shader/kerr_hamilton.h:67-178
//   * disc crossing:   shared_shader/disc_intersection.h:30-55
//   * shading:         geodesic_kernel.cu:77-171 (blackbody, NT temperature,
//                      band mask, starfield hash)
//   * tone map + AA:   geodesic_kernel.cu:413-510 (ACES, sRGB, Halton(2,3))
//
// With T = float every expression keeps the reference's operand order, so a
// host build of this file reproduces a host build of the reference bit for bit
// (pinned against oracle/_ref by tests/test_oracle_pins.py).  With T = double
// it is the FP64 oracle.  With T = Counted it counts the floating-point
// operations of the reference formulas (add/sub/mul/div/sqrt/min/max and each
// transcendental count 1) — the algorithmic work per ray used by the roofline.
//
// The error-controlled adaptive integrator (an extension that the reference
// does not have) lives in oracle/adaptive_oracle.hpp and reuses the pieces
// defined here.

#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/sgx_uniforms.h"

namespace oracle {

// ---------------------------------------------------------------------------
// Operation-counting scalar.  Wraps a float so that a Counted run follows the
// same branch decisions (step counts, terminations) as the FP32 run.
// ---------------------------------------------------------------------------
inline thread_local std::uint64_t g_ops = 0;

struct Counted {
    float v;
    Counted() = default;
    constexpr Counted(float x) : v(x) {}
    explicit operator int() const { return int(v); }
    explicit operator float() const { return v; }
    explicit operator double() const { return double(v); }
};
inline Counted operator+(Counted a, Counted b) { ++g_ops; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { ++g_ops; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { ++g_ops; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { ++g_ops; return Counted(a.v / b.v); }
inline Counted operator-(Counted a) { return Counted(-a.v); }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { return a.v >= b.v; }

// Scalar math, dispatched on T.  float -> the C float functions, double -> the
// double ones, Counted -> float functions plus one count each.
template <class T> struct M;
template <> struct M<float> {
    static float sqrt(float x) { return ::sqrtf(x); }
    static float exp(float x) { return ::expf(x); }
    static float sin(float x) { return ::sinf(x); }
    static float cos(float x) { return ::cosf(x); }
    static float acos(float x) { return ::acosf(x); }
    static float atan2(float y, float x) { return ::atan2f(y, x); }
    static float pow(float x, float y) { return ::powf(x, y); }
    static float log(float x) { return ::logf(x); }
    static float fmin(float a, float b) { return ::fminf(a, b); }
    static float fmax(float a, float b) { return ::fmaxf(a, b); }
    static float copysign(float m, float s) { return std::copysign(m, s); }
    static bool isfinite(float x) { return std::isfinite(x); }
    static float lit(float f, double) { return f; }
};
template <> struct M<double> {
    static double sqrt(double x) { return std::sqrt(x); }
    static double exp(double x) { return std::exp(x); }
    static double sin(double x) { return std::sin(x); }
    static double cos(double x) { return std::cos(x); }
    static double acos(double x) { return std::acos(x); }
    static double atan2(double y, double x) { return std::atan2(y, x); }
    static double pow(double x, double y) { return std::pow(x, y); }
    static double log(double x) { return std::log(x); }
    static double fmin(double a, double b) { return std::fmin(a, b); }
    static double fmax(double a, double b) { return std::fmax(a, b); }
    static double copysign(double m, double s) { return std::copysign(m, s); }
    static bool isfinite(double x) { return std::isfinite(x); }
    static double lit(float, double d) { return d; }
};
template <> struct M<Counted> {
    using C = Counted;
    static C sqrt(C x) { ++g_ops; return C(::sqrtf(x.v)); }
    static C sin(C x) { ++g_ops; return C(::sinf(x.v)); }
    static C cos(C x) { ++g_ops; return C(::cosf(x.v)); }
    static C acos(C x) { ++g_ops; return C(::acosf(x.v)); }
    static C atan2(C y, C x) { ++g_ops; return C(::atan2f(y.v, x.v)); }
    static C pow(C x, C y) { ++g_ops; return C(::powf(x.v, y.v)); }
    static C log(C x) { ++g_ops; return C(::logf(x.v)); }
    static C fmin(C a, C b) { ++g_ops; return C(::fminf(a.v, b.v)); }
    static C fmax(C a, C b) { ++g_ops; return C(::fmaxf(a.v, b.v)); }
    static C copysign(C m, C s) { return C(std::copysign(m.v, s.v)); }  // a sign transfer, no arithmetic
    static bool isfinite(C x) { return std::isfinite(x.v); }
    static C lit(float f, double) { return C(f); }
};

// A literal written once, rounded directly from its decimal text to T
// (float literal for float and Counted, double literal for double).
#define OLIT(x) (M<T>::lit(x##f, x))

template <class T> struct V3 {
    T x, y, z;
};

template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> vadd(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> vmul(V3<T> a, T k) { return {a.x * k, a.y * k, a.z * k}; }
template <class T> inline V3<T> vdiv(V3<T> a, T k) {
    const T ik = OLIT(1.0) / k;
    return vmul(a, ik);
}
template <class T> inline T vdot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T vlength(V3<T> a) { return M<T>::sqrt(vdot(a, a)); }
template <class T> inline V3<T> vnormalize(V3<T> a) {
    return vdiv(a, M<T>::fmax(vlength(a), OLIT(1e-20)));
}
template <class T> inline T vclamp(T x, T lo, T hi) { return M<T>::fmin(M<T>::fmax(x, lo), hi); }
template <class T> inline T vmix(T a, T b, T t) { return a + t * (b - a); }

template <class T> inline T pi_() { return OLIT(3.14159265358979323846); }

// ---------------------------------------------------------------------------
// Shading helpers (geodesic_kernel.cu:77-171)
// ---------------------------------------------------------------------------

// Tanner-Helland blackbody fit in centikelvin (geodesic_kernel.cu:77-97).
template <class T> inline V3<T> blackbody_srgb(T temp) {
    temp = vclamp(temp, OLIT(1000.0), OLIT(40000.0)) * OLIT(0.01);
    T r, g, b;
    if (temp <= OLIT(66.0)) {
        r = OLIT(1.0);
        g = vclamp(OLIT(0.39008157876901960784) * M<T>::log(temp) - OLIT(0.63184144378862745098),
                   OLIT(0.0), OLIT(1.0));
    } else {
        const T t1 = temp - OLIT(60.0);
        r = vclamp(OLIT(1.29293618606274509804) * M<T>::pow(t1, OLIT(-0.1332047592)), OLIT(0.0),
                   OLIT(1.0));
        g = vclamp(OLIT(1.12989086089529411765) * M<T>::pow(t1, OLIT(-0.0755148492)), OLIT(0.0),
                   OLIT(1.0));
    }
    if (temp >= OLIT(66.0)) {
        b = OLIT(1.0);
    } else if (temp <= OLIT(19.0)) {
        b = OLIT(0.0);
    } else {
        const T t1 = temp - OLIT(10.0);
        b = vclamp(OLIT(0.54320678911019607843) * M<T>::log(t1) - OLIT(1.19625408914), OLIT(0.0),
                   OLIT(1.0));
    }
    return v3(r, g, b);
}

// Novikov-Thorne-shaped temperature (geodesic_kernel.cu:99-107).
template <class T> inline T disc_temperature(T r_cross, T r_inner, T peak_T) {
    if (r_cross < r_inner) return OLIT(0.0);
    const T ratio = r_inner / r_cross;
    const T q = M<T>::pow(ratio, OLIT(0.75));
    const T edge = OLIT(1.0) - M<T>::sqrt(ratio);
    const T raw = q * M<T>::fmax(edge, OLIT(0.0));
    return peak_T * raw / OLIT(0.186);
}

// Spiral band modulation (geodesic_kernel.cu:109-121).
template <class T> inline T disc_band_mask(T r_cross, T phi_cross, T r_inner, T turbulence, T time_sec) {
    const T rho = M<T>::log(M<T>::fmax(r_cross / r_inner, OLIT(0.1)));
    const T shear = OLIT(4.0) / M<T>::fmax(M<T>::pow(r_cross / r_inner, OLIT(1.5)), OLIT(0.25));
    const T omega = M<T>::pow(M<T>::fmax(r_cross / r_inner, OLIT(0.1)), OLIT(-1.5));
    const T phi_anim = phi_cross - OLIT(0.8) * time_sec * omega;
    const T band1 = OLIT(0.5) + OLIT(0.5) * M<T>::cos(OLIT(10.0) * rho + OLIT(3.0) * phi_anim + shear);
    const T band2 = OLIT(0.5) + OLIT(0.5) * M<T>::cos(OLIT(22.0) * rho - OLIT(1.7) * phi_anim);
    const T combined = vmix(OLIT(0.8), band1 * band1 * band2, turbulence);
    return vclamp(OLIT(0.65) + OLIT(0.55) * combined, OLIT(0.0), OLIT(1.3));
}

// Integer hash of the starfield (geodesic_kernel.cu:123-131): bit-exact work.
inline std::uint32_t xorshift32(std::uint32_t x) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return x;
}
inline std::uint32_t mix32(std::uint32_t a, std::uint32_t b) { return xorshift32(a * 0x9E3779B9u + b); }

// Equirectangular 768x384 star cells (geodesic_kernel.cu:135-171).
template <class T> inline V3<T> starfield_color(V3<T> dir) {
    const T len = vlength(dir);
    if (len < OLIT(1e-6)) return v3(OLIT(0.0), OLIT(0.0), OLIT(0.005));
    const V3<T> n = vdiv(dir, len);
    const T theta = M<T>::acos(vclamp(n.z, OLIT(-1.0), OLIT(1.0)));
    const T phi = M<T>::atan2(n.y, n.x) + pi_<T>();
    const int NX = 768;
    const int NY = 384;
    const T two_pi = OLIT(2.0) * pi_<T>();
    int ix = int(phi / two_pi * T(float(NX))) % NX;
    int iy = int(theta / pi_<T>() * T(float(NY))) % NY;
    if (ix < 0) ix += NX;
    if (iy < 0) iy += NY;
    const std::uint32_t seed = mix32(std::uint32_t(ix), std::uint32_t(iy));
    const bool has_star = (seed & 0xFFu) < 4u;
    T r = OLIT(0.0015);
    T g = OLIT(0.002);
    T b = OLIT(0.005);
    if (has_star) {
        const T bright_raw = T(float((seed >> 8) & 0xFFu)) / OLIT(255.0);
        const T brightness = M<T>::pow(bright_raw, OLIT(4.0));
        const T hue = T(float((seed >> 16) & 0xFFu)) / OLIT(255.0);
        const T star_r = OLIT(1.0) - OLIT(0.5) * hue;
        const T star_g = OLIT(0.8) + OLIT(0.2) * hue * (OLIT(1.0) - hue) * OLIT(4.0);
        const T star_b = OLIT(0.4) + OLIT(0.6) * hue;
        r = M<T>::fmin(OLIT(1.0), r + brightness * star_r);
        g = M<T>::fmin(OLIT(1.0), g + brightness * star_g);
        b = M<T>::fmin(OLIT(1.0), b + brightness * star_b);
    }
    return vmul(v3(r, g, b), OLIT(0.6));
}

template <class T> inline V3<T> sky_color_sc(T sin_theta, T cos_theta, T phi) {
    const T sx = sin_theta * M<T>::cos(phi);
    const T sy = sin_theta * M<T>::sin(phi);
    return starfield_color(v3(sx, sy, cos_theta));
}
template <class T> inline V3<T> sky_color(T theta, T phi) {
    return sky_color_sc(M<T>::sin(theta), M<T>::cos(theta), phi);
}

// ---------------------------------------------------------------------------
// Parameters, promoted from the uniform block to T once per render.
// ---------------------------------------------------------------------------
template <class T> struct Params {
    V3<T> cam_pos, cam_fwd, cam_right, cam_up;
    T mass_M, spin_a, rs, tan_half_fov;
    T r_in, r_out, peak_T, aspect;
    T h_step, escape_r, horizon_cut, time_sec;
    T exposure, turbulence;
    std::uint32_t width, height, metric, flags, max_steps, spp;
};

template <class T> inline Params<T> promote(const sgx_uniforms& u) {
    Params<T> p;
    p.cam_pos = v3(T(u.cam_pos.x), T(u.cam_pos.y), T(u.cam_pos.z));
    p.cam_fwd = v3(T(u.cam_fwd.x), T(u.cam_fwd.y), T(u.cam_fwd.z));
    p.cam_right = v3(T(u.cam_right.x), T(u.cam_right.y), T(u.cam_right.z));
    p.cam_up = v3(T(u.cam_up.x), T(u.cam_up.y), T(u.cam_up.z));
    p.mass_M = T(u.mass_M);
    p.spin_a = T(u.spin_a);
    p.rs = T(u.rs);
    p.tan_half_fov = T(u.tan_half_fov);
    p.r_in = T(u.disc_r_inner);
    p.r_out = T(u.disc_r_outer);
    p.peak_T = T(u.disc_peak_T);
    p.aspect = T(u.aspect);
    p.h_step = T(u.h_step);
    p.escape_r = T(u.escape_r);
    p.horizon_cut = T(u.horizon_cut);
    p.time_sec = T(u.time_sec);
    p.exposure = T(u.exposure);
    p.turbulence = T(u.disc_turbulence);
    p.width = u.width;
    p.height = u.height;
    p.metric = u.metric_type;
    p.flags = u.flags;
    p.max_steps = u.max_steps;
    const std::uint32_t ss = u.supersample;
    p.spp = ss < 1u ? 1u : (ss > 1024u ? 1024u : ss);
    return p;
}

// ---------------------------------------------------------------------------
// Camera ray (geodesic_kernel.cu:177-223)
// ---------------------------------------------------------------------------
template <class T> struct CamRay {
    V3<T> cart;
    T ur, utheta, uphi;
    T cam_r, cam_theta, cam_phi, sin_th;
};

template <class T>
inline CamRay<T> camera_ray(std::uint32_t gx, std::uint32_t gy, T ox, T oy, const Params<T>& u) {
    const T fx = T(float(gx)) + ox;
    const T fy = T(float(gy)) + oy;
    const T u_ndc = (OLIT(2.0) * fx / T(float(u.width)) - OLIT(1.0)) * u.aspect * u.tan_half_fov;
    const T v_ndc = -(OLIT(2.0) * fy / T(float(u.height)) - OLIT(1.0)) * u.tan_half_fov;
    const V3<T> dir = vnormalize(vadd(u.cam_fwd, vadd(vmul(u.cam_right, u_ndc), vmul(u.cam_up, v_ndc))));
    CamRay<T> r;
    r.cart = dir;
    const V3<T> p = u.cam_pos;
    r.cam_r = vlength(p);
    r.cam_theta = M<T>::acos(vclamp(p.z / M<T>::fmax(r.cam_r, OLIT(1e-6)), OLIT(-1.0), OLIT(1.0)));
    r.cam_phi = M<T>::atan2(p.y, p.x);
    r.sin_th = M<T>::sin(r.cam_theta);
    const T cos_th = M<T>::cos(r.cam_theta);
    const T cos_phi = M<T>::cos(r.cam_phi);
    const T sin_phi = M<T>::sin(r.cam_phi);
    const V3<T> rhat = v3(r.sin_th * cos_phi, r.sin_th * sin_phi, cos_th);
    const V3<T> that = v3(cos_th * cos_phi, cos_th * sin_phi, -r.sin_th);
    const V3<T> phat = v3(-sin_phi, cos_phi, OLIT(0.0));
    const T ur_ortho = vdot(dir, rhat);
    const T uth_ortho = vdot(dir, that);
    const T uphi_ortho = vdot(dir, phat);
    r.ur = ur_ortho;
    r.utheta = uth_ortho / r.cam_r;
    r.uphi = uphi_ortho / (r.cam_r * M<T>::fmax(r.sin_th, OLIT(1e-6)));
    return r;
}

// ---------------------------------------------------------------------------
// Disc crossing (shared_shader/disc_intersection.h:30-55)
// ---------------------------------------------------------------------------
template <class T> struct Crossing {
    bool crossed;
    T frac;
};
template <class T> inline Crossing<T> equatorial_crossing(T theta_prev, T theta_curr) {
    const T mid = OLIT(1.5707963267948966);
    const T dp = theta_prev - mid;
    const T dc = theta_curr - mid;
    Crossing<T> x;
    x.crossed = (dp * dc) < OLIT(0.0);
    const T denom = theta_curr - theta_prev;
    x.frac = x.crossed ? (mid - theta_prev) / denom : OLIT(0.0);
    return x;
}
template <class T> inline T lerp_s(T prev, T curr, T frac) { return prev + frac * (curr - prev); }
template <class T> inline bool in_annulus(T r, T r_in, T r_out) { return (r >= r_in) && (r <= r_out); }

// How a ray ended; diagnostics only (the reference returns a colour).
enum Term : std::uint32_t {
    TERM_HORIZON = 0,   // captured or non-finite radius
    TERM_ESCAPE = 1,    // reached escape_r
    TERM_DISC = 2,      // hit the emitting annulus
    TERM_BUDGET = 3,    // max_steps exhausted
    TERM_DISC_COLD = 4, // crossed the annulus where T <= 0
    TERM_NO_ROOT = 5,   // Kerr u^t quadratic has no real root
};

template <class T> struct TraceOut {
    V3<T> hdr;
    std::uint32_t steps;
    std::uint32_t term;
};

// ---------------------------------------------------------------------------
// Schwarzschild (geodesic_math.h:25-28,101-134; geodesic_kernel.cu:229-297)
// ---------------------------------------------------------------------------
template <class T> struct SState {
    T t, r, theta, phi, ut, ur, utheta, uphi;
};

template <class T> inline SState<T> s_add_scaled(SState<T> y, SState<T> k, T f) {
    SState<T> o;
    o.t = y.t + k.t * f;
    o.r = y.r + k.r * f;
    o.theta = y.theta + k.theta * f;
    o.phi = y.phi + k.phi * f;
    o.ut = y.ut + k.ut * f;
    o.ur = y.ur + k.ur * f;
    o.utheta = y.utheta + k.utheta * f;
    o.uphi = y.uphi + k.uphi * f;
    return o;
}

template <class T> inline SState<T> schw_rhs(const SState<T>& s, T rs) {
    const T f = OLIT(1.0) - rs / s.r;
    const T r2 = s.r * s.r;
    const T sin_t = M<T>::sin(s.theta);
    const T cos_t = M<T>::cos(s.theta);
    SState<T> d;
    d.t = s.ut;
    d.r = s.ur;
    d.theta = s.utheta;
    d.phi = s.uphi;
    d.ut = -(rs / (r2 * f)) * s.ut * s.ur;
    d.ur = -(rs * f / (OLIT(2.0) * r2)) * s.ut * s.ut + (rs / (OLIT(2.0) * r2 * f)) * s.ur * s.ur
           + s.r * f * (s.utheta * s.utheta + sin_t * sin_t * s.uphi * s.uphi);
    d.utheta = OLIT(-2.0) * s.ur * s.utheta / s.r + sin_t * cos_t * s.uphi * s.uphi;
    d.uphi = OLIT(-2.0) * s.ur * s.uphi / s.r - OLIT(2.0) * (cos_t / sin_t) * s.utheta * s.uphi;
    return d;
}

// sum = (k1 + 2 k2) + (2 k3 + k4); y + sum * (h/6), component by component.
template <class T>
inline T rk4_combine(T y, T k1, T k2, T k3, T k4, T h6) {
    return y + ((k1 + k2 * OLIT(2.0)) + (k3 * OLIT(2.0) + k4)) * h6;
}

template <class T> inline SState<T> schw_rk4(const SState<T>& y, T h, T rs) {
    const SState<T> k1 = schw_rhs(y, rs);
    const SState<T> k2 = schw_rhs(s_add_scaled(y, k1, OLIT(0.5) * h), rs);
    const SState<T> k3 = schw_rhs(s_add_scaled(y, k2, OLIT(0.5) * h), rs);
    const SState<T> k4 = schw_rhs(s_add_scaled(y, k3, h), rs);
    const T h6 = h / OLIT(6.0);
    SState<T> o;
    o.t = rk4_combine(y.t, k1.t, k2.t, k3.t, k4.t, h6);
    o.r = rk4_combine(y.r, k1.r, k2.r, k3.r, k4.r, h6);
    o.theta = rk4_combine(y.theta, k1.theta, k2.theta, k3.theta, k4.theta, h6);
    o.phi = rk4_combine(y.phi, k1.phi, k2.phi, k3.phi, k4.phi, h6);
    o.ut = rk4_combine(y.ut, k1.ut, k2.ut, k3.ut, k4.ut, h6);
    o.ur = rk4_combine(y.ur, k1.ur, k2.ur, k3.ur, k4.ur, h6);
    o.utheta = rk4_combine(y.utheta, k1.utheta, k2.utheta, k3.utheta, k4.utheta, h6);
    o.uphi = rk4_combine(y.uphi, k1.uphi, k2.uphi, k3.uphi, k4.uphi, h6);
    return o;
}

// Shading shared by both metrics once the crossing radius is known.
template <class T>
inline V3<T> disc_shade(const Params<T>& u, T r_cross, T phi_cross, T T_local, T g) {
    const V3<T> col = blackbody_srgb(g * T_local);
    const T flux = vclamp(M<T>::pow(u.r_in / r_cross, OLIT(3.0)), OLIT(0.05), OLIT(1.5));
    const T bands = disc_band_mask(r_cross, phi_cross, u.r_in, u.turbulence, u.time_sec);
    const T g2 = g * g;
    return vmul(col, flux * bands * g2 * g2);
}

// Radius-adaptive step (geodesic_math.h:91-96), gated by SING_FLAG_ADAPTIVE_STEP:
// h = h_base * clamp(r / 6M, 1, 40).  The reference applies it in its WebGPU
// kernel for both metrics (geodesic_kernel.wgsl:117-122,486,591); its CUDA
// kernel ignores the flag.
template <class T> inline T radius_adaptive_h(T h_base, T r, T mass_M) {
    T mult = r / (OLIT(6.0) * mass_M);
    mult = (mult < OLIT(1.0)) ? OLIT(1.0) : mult;
    mult = (mult > OLIT(40.0)) ? OLIT(40.0) : mult;
    return h_base * mult;
}
template <class T> inline T step_h(const Params<T>& u, T r) {
    return (u.flags & SGX_FLAG_ADAPTIVE_STEP) ? radius_adaptive_h(u.h_step, r, u.mass_M) : u.h_step;
}

template <class T> inline TraceOut<T> trace_schwarzschild(const CamRay<T>& cam, const Params<T>& u) {
    SState<T> s;
    s.t = OLIT(0.0);
    s.r = cam.cam_r;
    s.theta = cam.cam_theta;
    s.phi = cam.cam_phi;
    s.ur = cam.ur;
    s.utheta = cam.utheta;
    s.uphi = cam.uphi;
    const T f_cam = OLIT(1.0) - u.rs / cam.cam_r;
    const T kin = (cam.ur * cam.ur) / f_cam + cam.utheta * cam.utheta * cam.cam_r * cam.cam_r
                  + cam.uphi * cam.uphi * cam.cam_r * cam.cam_r * cam.sin_th * cam.sin_th;
    s.ut = M<T>::sqrt(M<T>::fmax(kin / f_cam, OLIT(0.0)));

    T prev_theta = s.theta;
    T prev_r = s.r;
    T prev_uphi = s.uphi;
    const V3<T> black = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    for (std::uint32_t step = 0; step < u.max_steps; ++step) {
        if (!M<T>::isfinite(s.r) || s.r < u.horizon_cut) return {black, step, TERM_HORIZON};
        if (s.r > u.escape_r) {
            if (u.flags & SGX_FLAG_STARFIELD_ON) return {sky_color(s.theta, s.phi), step, TERM_ESCAPE};
            return {black, step, TERM_ESCAPE};
        }
        const Crossing<T> x = equatorial_crossing(prev_theta, s.theta);
        if ((u.flags & SGX_FLAG_DISC_ON) && x.crossed) {
            const T r_cross = lerp_s(prev_r, s.r, x.frac);
            const T uphi_cross = lerp_s(prev_uphi, s.uphi, x.frac);
            if (in_annulus(r_cross, u.r_in, u.r_out)) {
                const T T_local = disc_temperature(r_cross, u.r_in, u.peak_T);
                if (T_local > OLIT(0.0)) {
                    const T f_emit = OLIT(1.0) - u.rs / r_cross;
                    const T g_grav = (u.flags & SGX_FLAG_REDSHIFT_ON)
                                         ? M<T>::sqrt(M<T>::fmax(f_emit / f_cam, OLIT(0.0)))
                                         : OLIT(1.0);
                    T g_dop = OLIT(1.0);
                    if (u.flags & SGX_FLAG_DOPPLER_ON) {
                        const T omega = M<T>::sqrt(u.mass_M / (r_cross * r_cross * r_cross));
                        const T v = r_cross * omega / M<T>::sqrt(M<T>::fmax(f_emit, OLIT(1e-6)));
                        const T cos_psi = vclamp(-uphi_cross * r_cross, OLIT(-1.0), OLIT(1.0));
                        g_dop = M<T>::sqrt(M<T>::fmax(OLIT(1.0) - v * v, OLIT(0.0)))
                                / M<T>::fmax(OLIT(1.0) - v * cos_psi, OLIT(1e-4));
                    }
                    const T g = g_grav * g_dop;
                    // The reference interpolates phi between two identical
                    // endpoints (geodesic_kernel.cu:282); kept as written.
                    const T phi_cross = lerp_s(s.phi, s.phi, x.frac);
                    return {disc_shade(u, r_cross, phi_cross, T_local, g), step, TERM_DISC};
                }
                return {black, step, TERM_DISC_COLD};
            }
        }
        prev_theta = s.theta;
        prev_r = s.r;
        prev_uphi = s.uphi;
        s = schw_rk4(s, step_h(u, s.r), u.rs);
    }
    return {black, u.max_steps, TERM_BUDGET};
}

// ---------------------------------------------------------------------------
// Kerr, Hamiltonian form (kerr_hamilton.h:37-178; geodesic_kernel.cu:303-403)
// ---------------------------------------------------------------------------
template <class T> struct KState {
    T t, r, theta, phi, p_r, p_theta;
};
template <class T> struct KConst {
    T E, L, Q, a, M;
};

template <class T> inline KState<T> k_add_scaled(const KState<T>& y, const KState<T>& k, T f) {
    return {y.t + k.t * f, y.r + k.r * f, y.theta + k.theta * f,
            y.phi + k.phi * f, y.p_r + k.p_r * f, y.p_theta + k.p_theta * f};
}

// 2H with E, L_z substituted (kerr_hamilton.h:67-94).
template <class T> inline T kerr_two_H(T r, T theta, T p_r, T p_theta, const KConst<T>& c) {
    const T st = M<T>::sin(theta);
    const T s2 = st * st;
    const T safe_s2 = (s2 < OLIT(1e-10)) ? OLIT(1e-10) : s2;
    const T ct = M<T>::cos(theta);
    const T c2 = ct * ct;
    const T r2 = r * r;
    const T a2 = c.a * c.a;
    const T Sigma = r2 + a2 * c2;
    const T Delta = r2 - OLIT(2.0) * c.M * r + a2;
    const T A = (r2 + a2) * (r2 + a2) - a2 * Delta * s2;
    const T SD = Sigma * Delta;
    const T t_tt = -A * c.E * c.E / SD;
    const T t_tp = OLIT(4.0) * c.M * r * c.a * c.E * c.L / SD;
    const T t_pp = (Delta - a2 * safe_s2) * c.L * c.L / (SD * safe_s2);
    const T t_rr = Delta * p_r * p_r / Sigma;
    const T t_th = p_theta * p_theta / Sigma;
    return t_tt + t_tp + t_pp + t_rr + t_th;
}

// Hamilton's equations with the analytic partials (kerr_hamilton.h:97-155),
// with sin(theta) and cos(theta) given (the theta slot of s is not read).
// WITH_T = false leaves dt/dlambda out (the error-controlled form drops t).
template <class T, bool WITH_T = true>
inline KState<T> kerr_rhs_sc(const KState<T>& s, T st, T ct, const KConst<T>& c) {
    const T r = s.r;
    const T s2 = st * st;
    const T safe_s2 = (s2 < OLIT(1e-10)) ? OLIT(1e-10) : s2;
    const T c2 = ct * ct;
    const T r2 = r * r;
    const T a = c.a;
    const T Mm = c.M;
    const T a2 = a * a;
    const T Sigma = r2 + a2 * c2;
    const T Delta = r2 - OLIT(2.0) * Mm * r + a2;
    const T A = (r2 + a2) * (r2 + a2) - a2 * Delta * s2;
    const T SD = Sigma * Delta;
    KState<T> d;
    if constexpr (WITH_T) d.t = (A * c.E - OLIT(2.0) * Mm * r * a * c.L) / SD;
    else d.t = OLIT(0.0);
    d.phi = (OLIT(2.0) * Mm * r * a * c.E * s2 + (Delta - a2 * s2) * c.L) / (SD * safe_s2);
    d.r = Delta * s.p_r / Sigma;
    d.theta = s.p_theta / Sigma;
    const T E = c.E;
    const T L = c.L;
    const T L2 = L * L;
    const T B = -A * E * E + OLIT(4.0) * Mm * r * a * E * L - a2 * L2;
    const T Sig_r = OLIT(2.0) * r;
    const T Del_r = OLIT(2.0) * r - OLIT(2.0) * Mm;
    const T A_r = OLIT(4.0) * r * (r2 + a2) - a2 * Del_r * s2;
    const T B_r = -A_r * E * E + OLIT(4.0) * Mm * a * E * L;
    const T sin2t = OLIT(2.0) * st * ct;
    const T Sig_t = -a2 * sin2t;
    const T B_t = a2 * Delta * sin2t * E * E;
    const T Sigma2 = Sigma * Sigma;
    const T Dp2 = Delta * s.p_r * s.p_r + s.p_theta * s.p_theta;
    const T dH_dr = B_r / SD - B * (Sig_r * Delta + Sigma * Del_r) / (SD * SD)
                    - L2 * Sig_r / (Sigma2 * safe_s2) + Del_r * s.p_r * s.p_r / Sigma
                    - Dp2 * Sig_r / Sigma2;
    const T dH_dth = B_t / SD - B * Sig_t / (Sigma2 * Delta)
                     - L2 * (Sig_t * safe_s2 + Sigma * sin2t) / (Sigma2 * safe_s2 * safe_s2)
                     - Dp2 * Sig_t / Sigma2;
    d.p_r = OLIT(-0.5) * dH_dr;
    d.p_theta = OLIT(-0.5) * dH_dth;
    return d;
}

template <class T> inline KState<T> kerr_rhs(const KState<T>& s, const KConst<T>& c) {
    const T st = M<T>::sin(s.theta);
    const T ct = M<T>::cos(s.theta);
    return kerr_rhs_sc(s, st, ct, c);
}

// Near-pole step damping: h * clamp(5|sin theta|, 0.05, 1) (kerr_hamilton.h:165-170).
template <class T> inline T pole_scaled_h(T h, T theta) {
    T st_abs = M<T>::sin(theta);
    st_abs = (st_abs < OLIT(0.0)) ? -st_abs : st_abs;
    T ps = st_abs * OLIT(5.0);
    ps = (ps > OLIT(1.0)) ? OLIT(1.0) : ((ps < OLIT(0.05)) ? OLIT(0.05) : ps);
    return h * ps;
}

template <class T> inline KState<T> kerr_rk4(const KState<T>& y, T h, const KConst<T>& c) {
    h = pole_scaled_h(h, y.theta);
    const KState<T> k1 = kerr_rhs(y, c);
    const KState<T> k2 = kerr_rhs(k_add_scaled(y, k1, OLIT(0.5) * h), c);
    const KState<T> k3 = kerr_rhs(k_add_scaled(y, k2, OLIT(0.5) * h), c);
    const KState<T> k4 = kerr_rhs(k_add_scaled(y, k3, h), c);
    const T h6 = h / OLIT(6.0);
    KState<T> o;
    o.t = rk4_combine(y.t, k1.t, k2.t, k3.t, k4.t, h6);
    o.r = rk4_combine(y.r, k1.r, k2.r, k3.r, k4.r, h6);
    o.theta = rk4_combine(y.theta, k1.theta, k2.theta, k3.theta, k4.theta, h6);
    o.phi = rk4_combine(y.phi, k1.phi, k2.phi, k3.phi, k4.phi, h6);
    o.p_r = rk4_combine(y.p_r, k1.p_r, k2.p_r, k3.p_r, k4.p_r, h6);
    o.p_theta = rk4_combine(y.p_theta, k1.p_theta, k2.p_theta, k3.p_theta, k4.p_theta, h6);
    return o;
}

// Initial canonical state and constants of motion from a camera ray
// (geodesic_kernel.cu:304-344).  Returns false when the u^t quadratic has no
// real root (the reference then returns black).
template <class T>
inline bool kerr_init(const CamRay<T>& cam, const Params<T>& u, KState<T>& s, KConst<T>& c) {
    const T Mm = u.mass_M;
    const T a = u.spin_a;
    const T sin_th = cam.sin_th;
    const T cos_th = M<T>::cos(cam.cam_theta);
    const T cam_r = cam.cam_r;
    const T Sigma_c = cam_r * cam_r + a * a * cos_th * cos_th;
    const T Delta_c = cam_r * cam_r - OLIT(2.0) * Mm * cam_r + a * a;
    const T s2_c = sin_th * sin_th;
    const T g_tt = -(OLIT(1.0) - OLIT(2.0) * Mm * cam_r / Sigma_c);
    const T g_tp = OLIT(-2.0) * Mm * cam_r * a * s2_c / Sigma_c;
    const T g_rr = Sigma_c / Delta_c;
    const T g_thth = Sigma_c;
    const T g_pp = s2_c * ((cam_r * cam_r + a * a) * (cam_r * cam_r + a * a) - a * a * Delta_c * s2_c)
                   / Sigma_c;
    const T A_q = g_tt;
    const T B_q = OLIT(2.0) * g_tp * cam.uphi;
    const T C_q = g_rr * cam.ur * cam.ur + g_thth * cam.utheta * cam.utheta + g_pp * cam.uphi * cam.uphi;
    const T disc_q = B_q * B_q - OLIT(4.0) * A_q * C_q;
    if (disc_q < OLIT(0.0)) return false;
    const T ut = (-B_q - M<T>::sqrt(disc_q)) / (OLIT(2.0) * A_q);
    c.a = a;
    c.M = Mm;
    c.E = -(g_tt * ut + g_tp * cam.uphi);
    c.L = g_tp * ut + g_pp * cam.uphi;
    const T p_theta_init = g_thth * cam.utheta;
    c.Q = p_theta_init * p_theta_init
          + cos_th * cos_th * (c.L * c.L / M<T>::fmax(s2_c, OLIT(1e-6)) - a * a * c.E * c.E);
    s.t = OLIT(0.0);
    s.r = cam_r;
    s.theta = cam.cam_theta;
    s.phi = cam.cam_phi;
    s.p_r = g_rr * cam.ur;
    s.p_theta = g_thth * cam.utheta;
    return true;
}

template <class T> inline T kerr_horizon_cut(T Mm, T a) {
    return OLIT(1.02) * (Mm + M<T>::sqrt(M<T>::fmax(Mm * Mm - a * a, OLIT(0.0))));
}

// Disc colour at a Kerr crossing (geodesic_kernel.cu:368-393).
template <class T>
inline V3<T> kerr_disc_colour(const Params<T>& u, const KConst<T>& c, T cam_r, T r_cross, T phi_cross,
                              T T_local) {
    const T Mm = u.mass_M;
    const T a = u.spin_a;
    const T f_emit = OLIT(1.0) - OLIT(2.0) * Mm / r_cross;
    const T f_obs = OLIT(1.0) - OLIT(2.0) * Mm / cam_r;
    const T g_grav = (u.flags & SGX_FLAG_REDSHIFT_ON)
                         ? M<T>::sqrt(M<T>::fmax(f_emit, OLIT(1e-6)) / M<T>::fmax(f_obs, OLIT(1e-6)))
                         : OLIT(1.0);
    T g_dop = OLIT(1.0);
    if (u.flags & SGX_FLAG_DOPPLER_ON) {
        const T om0 = M<T>::sqrt(Mm / (r_cross * r_cross * r_cross));
        const T omega_K = om0 / (OLIT(1.0) + a * om0);
        const T v = r_cross * omega_K / M<T>::sqrt(M<T>::fmax(f_emit, OLIT(1e-6)));
        const T cos_psi = vclamp(c.L / r_cross, OLIT(-1.0), OLIT(1.0));
        const T v2 = v * v;
        g_dop = M<T>::sqrt(M<T>::fmax(OLIT(1.0) - v2, OLIT(0.0))) / M<T>::fmax(OLIT(1.0) - v * cos_psi, OLIT(1e-4));
    }
    const T g = g_grav * g_dop;
    return disc_shade(u, r_cross, phi_cross, T_local, g);
}

template <class T> inline TraceOut<T> trace_kerr(const CamRay<T>& cam, const Params<T>& u) {
    const V3<T> black = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    KState<T> s;
    KConst<T> c;
    if (!kerr_init(cam, u, s, c)) return {black, 0u, TERM_NO_ROOT};
    T prev_theta = s.theta;
    T prev_r = s.r;
    const T hcut = kerr_horizon_cut(u.mass_M, u.spin_a);
    for (std::uint32_t step = 0; step < u.max_steps; ++step) {
        if (!M<T>::isfinite(s.r) || s.r < hcut) return {black, step, TERM_HORIZON};
        if (s.r > u.escape_r) {
            if (u.flags & SGX_FLAG_STARFIELD_ON) return {sky_color(s.theta, s.phi), step, TERM_ESCAPE};
            return {black, step, TERM_ESCAPE};
        }
        const Crossing<T> x = equatorial_crossing(prev_theta, s.theta);
        if ((u.flags & SGX_FLAG_DISC_ON) && x.crossed) {
            const T r_cross = lerp_s(prev_r, s.r, x.frac);
            if (in_annulus(r_cross, u.r_in, u.r_out)) {
                const T T_local = disc_temperature(r_cross, u.r_in, u.peak_T);
                if (T_local > OLIT(0.0))
                    return {kerr_disc_colour(u, c, cam.cam_r, r_cross, s.phi, T_local), step, TERM_DISC};
                return {black, step, TERM_DISC_COLD};
            }
        }
        prev_theta = s.theta;
        prev_r = s.r;
        s = kerr_rk4(s, step_h(u, s.r), c);
    }
    return {black, u.max_steps, TERM_BUDGET};
}

// ---------------------------------------------------------------------------
// Display transform (geodesic_kernel.cu:413-451)
// ---------------------------------------------------------------------------
template <class T> inline T aces1(T x) {
    const T a = OLIT(2.51), b = OLIT(0.03), c = OLIT(2.43), d = OLIT(0.59), e = OLIT(0.14);
    return vclamp((x * (a * x + b)) / (x * (c * x + d) + e), OLIT(0.0), OLIT(1.0));
}
template <class T> inline V3<T> aces(V3<T> x) { return v3(aces1(x.x), aces1(x.y), aces1(x.z)); }

template <class T> inline T linear_to_srgb(T c) {
    c = vclamp(c, OLIT(0.0), OLIT(1.0));
    return c <= OLIT(0.0031308) ? OLIT(12.92) * c
                                : OLIT(1.055) * M<T>::pow(c, OLIT(1.0) / OLIT(2.4)) - OLIT(0.055);
}
// Truncating conversion to a byte, as the reference's (std::uint8_t) cast.
template <class T> inline std::uint8_t to_u8(T c) {
    const T v = vclamp(linear_to_srgb(c) * OLIT(255.0) + OLIT(0.5), OLIT(0.0), OLIT(255.0));
    return std::uint8_t(int(v));
}

// Radical inverse of i in the given base, in T (geodesic_kernel.cu:442-451).
template <class T> inline T halton(std::uint32_t i, std::uint32_t base) {
    T f = OLIT(1.0);
    T r = OLIT(0.0);
    while (i > 0u) {
        f = f / T(float(base));
        r = r + f * T(float(i % base));
        i /= base;
    }
    return r;
}

// One camera sample: jitter -> ray -> trace (geodesic_kernel.cu:483-501).
template <class T>
inline TraceOut<T> trace_sample(std::uint32_t gx, std::uint32_t gy, std::uint32_t s, const Params<T>& u) {
    T ox, oy;
    if (u.spp == 1u) {
        ox = OLIT(0.5);
        oy = OLIT(0.5);
    } else {
        ox = halton<T>(s + 1u, 2u);
        oy = halton<T>(s + 1u, 3u);
    }
    const CamRay<T> cam = camera_ray(gx, gy, ox, oy, u);
    return (u.metric == SGX_METRIC_KERR) ? trace_kerr(cam, u) : trace_schwarzschild(cam, u);
}

// The per-pixel body of the reference kernel: average of per-sample ACES
// values (geodesic_kernel.cu:482-503).  Returns the LDR mean before sRGB.
template <class T> inline V3<T> shade_pixel(std::uint32_t gx, std::uint32_t gy, const Params<T>& u) {
    V3<T> ldr = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    if (u.spp == 1u) {
        const TraceOut<T> o = trace_sample(gx, gy, 0u, u);
        ldr = aces(vmul(o.hdr, u.exposure));
    } else {
        for (std::uint32_t s = 0; s < u.spp; ++s) {
            const TraceOut<T> o = trace_sample(gx, gy, s, u);
            ldr = vadd(ldr, aces(vmul(o.hdr, u.exposure)));
        }
        ldr = vmul(ldr, OLIT(1.0) / T(float(u.spp)));
    }
    return ldr;
}

}  // namespace oracle
