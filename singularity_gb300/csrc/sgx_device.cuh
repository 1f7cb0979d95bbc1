// singularity_gb300/csrc/sgx_device.cuh
//
// Device-side physics of the tracer, templated on the arithmetic type T
// (float for the FP32 and mixed forms, double for the FP64 form).
//
// The formulas are the reference's (cited per function); the structure is
// this library's own:
//   * everything that depends only on the view (camera spherical position and
//     its orthonormal frame, the Kerr metric at the camera, horizon radius,
//     f(r_cam)) is evaluated once per view by `make_view` instead of once per
//     sample, with the same float expressions, so the values are the ones the
//     reference recomputes for every sample;
//   * the per-ray state is the minimum the output depends on: the reference
//     also integrates t, which nothing reads, so it is dropped;
//   * the Kerr right-hand side comes in two algebraically equal forms: REF
//     keeps the reference's fourteen IEEE divisions (kerr_hamilton.h:97-155);
//     FAST shares three reciprocals 1/Sigma, 1/Delta, 1/sin^2 and folds the
//     per-ray products E^2, 4MaEL, a^2 L^2 into constants.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include <type_traits>

#include "sgx_uniforms.h"

namespace sgxd {

// ---------------------------------------------------------------------------
// Scalar traits
// ---------------------------------------------------------------------------
template <class T> struct DM;
template <> struct DM<float> {
    static __device__ __forceinline__ float lit(float f, double) { return f; }
    static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float sin_(float x) { return sinf(x); }
    static __device__ __forceinline__ float cos_(float x) { return cosf(x); }
    static __device__ __forceinline__ void sincos_(float x, float* s, float* c) { sincosf(x, s, c); }
    static __device__ __forceinline__ float acos_(float x) { return acosf(x); }
    static __device__ __forceinline__ float atan2_(float y, float x) { return atan2f(y, x); }
    static __device__ __forceinline__ float pow_(float x, float y) { return powf(x, y); }
    static __device__ __forceinline__ float log_(float x) { return logf(x); }
    static __device__ __forceinline__ float exp_(float x) { return expf(x); }
    static __device__ __forceinline__ float fmin_(float a, float b) { return fminf(a, b); }
    static __device__ __forceinline__ float fmax_(float a, float b) { return fmaxf(a, b); }
    static __device__ __forceinline__ float rcp_(float x) { return 1.0f / x; }
    // PTX rcp.approx.ftz.f32: one MUFU op, at most 1 ulp from 1/x.
    static __device__ __forceinline__ float rcp_fast(float x) {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        return r;
    }
};
template <> struct DM<double> {
    static __device__ __forceinline__ double lit(float, double d) { return d; }
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double sin_(double x) { return sin(x); }
    static __device__ __forceinline__ double cos_(double x) { return cos(x); }
    static __device__ __forceinline__ void sincos_(double x, double* s, double* c) { sincos(x, s, c); }
    static __device__ __forceinline__ double acos_(double x) { return acos(x); }
    static __device__ __forceinline__ double atan2_(double y, double x) { return atan2(y, x); }
    static __device__ __forceinline__ double pow_(double x, double y) { return pow(x, y); }
    static __device__ __forceinline__ double log_(double x) { return log(x); }
    static __device__ __forceinline__ double exp_(double x) { return exp(x); }
    static __device__ __forceinline__ double fmin_(double a, double b) { return fmin(a, b); }
    static __device__ __forceinline__ double fmax_(double a, double b) { return fmax(a, b); }
    static __device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double rcp_fast(double x) { return 1.0 / x; }
};

#define DLIT(x) (::sgxd::DM<T>::lit(x##f, x))

template <class T> __device__ __forceinline__ T clampv(T x, T lo, T hi) {
    return DM<T>::fmin_(DM<T>::fmax_(x, lo), hi);
}

template <class T> struct V3 {
    T x, y, z;
};
template <class T> __device__ __forceinline__ V3<T> mk3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> __device__ __forceinline__ T dot3(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// How a ray ended (diagnostic; the image only sees the colour).
enum : std::uint32_t {
    TERM_HORIZON = 0,
    TERM_ESCAPE = 1,
    TERM_DISC = 2,
    TERM_BUDGET = 3,
    TERM_DISC_COLD = 4,
    TERM_NO_ROOT = 5,
};

// ---------------------------------------------------------------------------
// Per-view constants
// ---------------------------------------------------------------------------
template <class T> struct View {
    // camera frame (build_camera_ray_subpixel, geodesic_kernel.cu:188-223)
    V3<T> fwd, right, up;
    V3<T> rhat, that, phat;
    T aspect, tan_half_fov, width_f, height_f;
    T cam_r, cam_theta, cam_phi, sin_th, cos_th;
    T uphi_den;  // cam_r * max(sin_th, 1e-6)
    // scene
    T M, a, a2, rs, r_in, r_out, peak_T, h, escape_r, time_sec, exposure, turbulence;
    T twoM;   // 2 M
    T hcut;   // capture radius: 1.02 r_+ (Kerr) or u.horizon_cut (Schwarzschild)
    T f_cam;  // Schwarzschild 1 - rs/r_cam
    T f_obs;  // Kerr shading 1 - 2M/r_cam
    T r_plus;             // outer horizon M + sqrt(M^2 - a^2)
    T r_ph_pro, r_ph_ret; // equatorial prograde / retrograde photon orbits
    // Kerr metric at the camera (geodesic_kernel.cu:310-319)
    T g_tt, g_tp, g_rr, g_thth, g_pp, s2_c;
    // the same in FP64 (from the T camera values) for the mixed form's FP64
    // constants of motion, and 1 / (2 g_tt)
    double g_tt_d, g_tp_d, g_rr_d, g_thth_d, g_pp_d, inv_2gtt_d;
    std::uint32_t width, height, flags, max_steps, spp, metric;
};

template <class T> __device__ inline View<T> make_view(const sgx_uniforms& u) {
    View<T> v;
    v.fwd = mk3(T(u.cam_fwd.x), T(u.cam_fwd.y), T(u.cam_fwd.z));
    v.right = mk3(T(u.cam_right.x), T(u.cam_right.y), T(u.cam_right.z));
    v.up = mk3(T(u.cam_up.x), T(u.cam_up.y), T(u.cam_up.z));
    v.aspect = T(u.aspect);
    v.tan_half_fov = T(u.tan_half_fov);
    v.width_f = T(float(u.width));
    v.height_f = T(float(u.height));
    const V3<T> p = mk3(T(u.cam_pos.x), T(u.cam_pos.y), T(u.cam_pos.z));
    v.cam_r = DM<T>::sqrt_(dot3(p, p));
    v.cam_theta = DM<T>::acos_(clampv(p.z / DM<T>::fmax_(v.cam_r, DLIT(1e-6)), DLIT(-1.0), DLIT(1.0)));
    v.cam_phi = DM<T>::atan2_(p.y, p.x);
    v.sin_th = DM<T>::sin_(v.cam_theta);
    v.cos_th = DM<T>::cos_(v.cam_theta);
    const T cos_phi = DM<T>::cos_(v.cam_phi);
    const T sin_phi = DM<T>::sin_(v.cam_phi);
    v.rhat = mk3(v.sin_th * cos_phi, v.sin_th * sin_phi, v.cos_th);
    v.that = mk3(v.cos_th * cos_phi, v.cos_th * sin_phi, -v.sin_th);
    v.phat = mk3(-sin_phi, cos_phi, DLIT(0.0));
    v.uphi_den = v.cam_r * DM<T>::fmax_(v.sin_th, DLIT(1e-6));

    v.M = T(u.mass_M);
    v.a = T(u.spin_a);
    v.a2 = v.a * v.a;
    v.twoM = DLIT(2.0) * v.M;
    v.rs = T(u.rs);
    v.r_in = T(u.disc_r_inner);
    v.r_out = T(u.disc_r_outer);
    v.peak_T = T(u.disc_peak_T);
    v.h = T(u.h_step);
    v.escape_r = T(u.escape_r);
    v.time_sec = T(u.time_sec);
    v.exposure = T(u.exposure);
    v.turbulence = T(u.disc_turbulence);
    v.width = u.width;
    v.height = u.height;
    v.flags = u.flags;
    v.max_steps = u.max_steps;
    v.spp = u.supersample < 1u ? 1u : (u.supersample > 1024u ? 1024u : u.supersample);
    v.metric = u.metric_type;

    v.f_cam = DLIT(1.0) - v.rs / v.cam_r;
    v.f_obs = DLIT(1.0) - DLIT(2.0) * v.M / v.cam_r;
    const T r = v.cam_r, a = v.a, Mm = v.M;
    const T Sigma_c = r * r + a * a * v.cos_th * v.cos_th;
    const T Delta_c = r * r - DLIT(2.0) * Mm * r + a * a;
    v.s2_c = v.sin_th * v.sin_th;
    v.g_tt = -(DLIT(1.0) - DLIT(2.0) * Mm * r / Sigma_c);
    v.g_tp = DLIT(-2.0) * Mm * r * a * v.s2_c / Sigma_c;
    v.g_rr = Sigma_c / Delta_c;
    v.g_thth = Sigma_c;
    v.g_pp = v.s2_c * ((r * r + a * a) * (r * r + a * a) - a * a * Delta_c * v.s2_c) / Sigma_c;
    {
        const double Md = v.M, ad = v.a, rd = v.cam_r, ct = v.cos_th, st = v.sin_th;
        const double Sg = rd * rd + ad * ad * ct * ct, Dl = rd * rd - 2.0 * Md * rd + ad * ad, s2 = st * st;
        v.g_tt_d = -(1.0 - 2.0 * Md * rd / Sg);
        v.g_tp_d = -2.0 * Md * rd * ad * s2 / Sg;
        v.g_rr_d = Sg / Dl;
        v.g_thth_d = Sg;
        v.g_pp_d = s2 * ((rd * rd + ad * ad) * (rd * rd + ad * ad) - ad * ad * Dl * s2) / Sg;
        v.inv_2gtt_d = 1.0 / (2.0 * v.g_tt_d);
    }
    if (v.metric == SGX_METRIC_KERR) {
        v.hcut = DLIT(1.02) * (Mm + DM<T>::sqrt_(DM<T>::fmax_(Mm * Mm - a * a, DLIT(0.0))));
    } else {
        v.hcut = T(u.horizon_cut);
    }
    v.r_plus = Mm + DM<T>::sqrt_(DM<T>::fmax_(Mm * Mm - a * a, DLIT(0.0)));
    v.r_ph_pro = DLIT(2.0) * Mm * (DLIT(1.0) + DM<T>::cos_(DLIT(2.0) / DLIT(3.0) * DM<T>::acos_(-a / Mm)));
    v.r_ph_ret = DLIT(2.0) * Mm * (DLIT(1.0) + DM<T>::cos_(DLIT(2.0) / DLIT(3.0) * DM<T>::acos_(a / Mm)));
    return v;
}

// ---------------------------------------------------------------------------
// Camera sample (geodesic_kernel.cu:188-223, 442-451, 483-501)
// ---------------------------------------------------------------------------
template <class T> __device__ __forceinline__ T halton(std::uint32_t i, std::uint32_t base) {
    T f = DLIT(1.0);
    T r = DLIT(0.0);
    const T b = T(float(base));
    while (i > 0u) {
        f = f / b;
        r = r + f * T(float(i % base));
        i /= base;
    }
    return r;
}

template <class T> struct CamDir {
    T ur, utheta, uphi;
};

// Sub-pixel offset of sample s (geodesic_kernel.cu:483-497): the pixel centre
// for spp == 1, else Halton(s + 1) in bases 2 and 3.
template <class T> __device__ __forceinline__ void sample_offset(std::uint32_t spp, std::uint32_t s, T& ox, T& oy) {
    if (spp == 1u) {
        ox = DLIT(0.5);
        oy = DLIT(0.5);
    } else {
        ox = halton<T>(s + 1u, 2u);
        oy = halton<T>(s + 1u, 3u);
    }
}

// Camera direction for pixel (gx, gy) and sub-pixel offset (ox, oy): the
// per-sample part of build_camera_ray_subpixel (geodesic_kernel.cu:188-223).
template <class T>
__device__ __forceinline__ CamDir<T> camera_dir(const View<T>& v, std::uint32_t gx, std::uint32_t gy, T ox, T oy) {
    const T fx = T(float(gx)) + ox;
    const T fy = T(float(gy)) + oy;
    const T u_ndc = (DLIT(2.0) * fx / v.width_f - DLIT(1.0)) * v.aspect * v.tan_half_fov;
    const T v_ndc = -(DLIT(2.0) * fy / v.height_f - DLIT(1.0)) * v.tan_half_fov;
    V3<T> d = mk3(v.fwd.x + (v.right.x * u_ndc + v.up.x * v_ndc), v.fwd.y + (v.right.y * u_ndc + v.up.y * v_ndc),
                  v.fwd.z + (v.right.z * u_ndc + v.up.z * v_ndc));
    const T len = DM<T>::fmax_(DM<T>::sqrt_(dot3(d, d)), DLIT(1e-20));
    const T ik = DLIT(1.0) / len;
    d = mk3(d.x * ik, d.y * ik, d.z * ik);
    CamDir<T> c;
    c.ur = dot3(d, v.rhat);
    c.utheta = dot3(d, v.that) / v.cam_r;
    c.uphi = dot3(d, v.phat) / v.uphi_den;
    return c;
}

// ---------------------------------------------------------------------------
// Shading (geodesic_kernel.cu:77-171), evaluated once per terminated ray.
// ---------------------------------------------------------------------------
template <class T> __device__ inline V3<T> blackbody_srgb(T temp) {
    temp = clampv(temp, DLIT(1000.0), DLIT(40000.0)) * DLIT(0.01);
    T r, g, b;
    if (temp <= DLIT(66.0)) {
        r = DLIT(1.0);
        g = clampv(DLIT(0.39008157876901960784) * DM<T>::log_(temp) - DLIT(0.63184144378862745098), DLIT(0.0),
                   DLIT(1.0));
    } else {
        const T t1 = temp - DLIT(60.0);
        r = clampv(DLIT(1.29293618606274509804) * DM<T>::pow_(t1, DLIT(-0.1332047592)), DLIT(0.0), DLIT(1.0));
        g = clampv(DLIT(1.12989086089529411765) * DM<T>::pow_(t1, DLIT(-0.0755148492)), DLIT(0.0), DLIT(1.0));
    }
    if (temp >= DLIT(66.0)) {
        b = DLIT(1.0);
    } else if (temp <= DLIT(19.0)) {
        b = DLIT(0.0);
    } else {
        const T t1 = temp - DLIT(10.0);
        b = clampv(DLIT(0.54320678911019607843) * DM<T>::log_(t1) - DLIT(1.19625408914), DLIT(0.0), DLIT(1.0));
    }
    return mk3(r, g, b);
}

template <class T> __device__ __forceinline__ T disc_temperature(T r_cross, T r_inner, T peak_T) {
    if (r_cross < r_inner) return DLIT(0.0);
    const T ratio = r_inner / r_cross;
    const T q = DM<T>::pow_(ratio, DLIT(0.75));
    const T edge = DLIT(1.0) - DM<T>::sqrt_(ratio);
    const T raw = q * DM<T>::fmax_(edge, DLIT(0.0));
    return peak_T * raw / DLIT(0.186);
}

template <class T> __device__ inline T disc_band_mask(T r_cross, T phi_cross, T r_inner, T turbulence, T time_sec) {
    const T rho = DM<T>::log_(DM<T>::fmax_(r_cross / r_inner, DLIT(0.1)));
    const T shear = DLIT(4.0) / DM<T>::fmax_(DM<T>::pow_(r_cross / r_inner, DLIT(1.5)), DLIT(0.25));
    const T omega = DM<T>::pow_(DM<T>::fmax_(r_cross / r_inner, DLIT(0.1)), DLIT(-1.5));
    const T phi_anim = phi_cross - DLIT(0.8) * time_sec * omega;
    const T band1 = DLIT(0.5) + DLIT(0.5) * DM<T>::cos_(DLIT(10.0) * rho + DLIT(3.0) * phi_anim + shear);
    const T band2 = DLIT(0.5) + DLIT(0.5) * DM<T>::cos_(DLIT(22.0) * rho - DLIT(1.7) * phi_anim);
    const T combined = DLIT(0.8) + turbulence * (band1 * band1 * band2 - DLIT(0.8));
    return clampv(DLIT(0.65) + DLIT(0.55) * combined, DLIT(0.0), DLIT(1.3));
}

__device__ __forceinline__ std::uint32_t star_hash(std::uint32_t ix, std::uint32_t iy) {
    std::uint32_t x = ix * 0x9E3779B9u + iy;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return x;
}

// Sky colour for an escaped ray with (sin theta, cos theta, phi) at its last
// state: the starfield of geodesic_kernel.cu:135-171 in that direction.
template <class T> __device__ inline V3<T> sky_color_sc(T st, T ct, T phi) {
    const V3<T> dir = mk3(st * DM<T>::cos_(phi), st * DM<T>::sin_(phi), ct);
    const T len = DM<T>::sqrt_(dot3(dir, dir));
    if (len < DLIT(1e-6)) return mk3(DLIT(0.0), DLIT(0.0), DLIT(0.005));
    const T ik = DLIT(1.0) / len;
    const V3<T> n = mk3(dir.x * ik, dir.y * ik, dir.z * ik);
    const T pi = DLIT(3.14159265358979323846);
    const T th = DM<T>::acos_(clampv(n.z, DLIT(-1.0), DLIT(1.0)));
    const T ph = DM<T>::atan2_(n.y, n.x) + pi;
    int ix = int(ph / (DLIT(2.0) * pi) * T(768.0f)) % 768;
    int iy = int(th / pi * T(384.0f)) % 384;
    if (ix < 0) ix += 768;
    if (iy < 0) iy += 384;
    const std::uint32_t seed = star_hash(std::uint32_t(ix), std::uint32_t(iy));
    T r = DLIT(0.0015), g = DLIT(0.002), b = DLIT(0.005);
    if ((seed & 0xFFu) < 4u) {
        const T bright_raw = T(float((seed >> 8) & 0xFFu)) / DLIT(255.0);
        const T brightness = DM<T>::pow_(bright_raw, DLIT(4.0));
        const T hue = T(float((seed >> 16) & 0xFFu)) / DLIT(255.0);
        const T star_r = DLIT(1.0) - DLIT(0.5) * hue;
        const T star_g = DLIT(0.8) + DLIT(0.2) * hue * (DLIT(1.0) - hue) * DLIT(4.0);
        const T star_b = DLIT(0.4) + DLIT(0.6) * hue;
        r = DM<T>::fmin_(DLIT(1.0), r + brightness * star_r);
        g = DM<T>::fmin_(DLIT(1.0), g + brightness * star_g);
        b = DM<T>::fmin_(DLIT(1.0), b + brightness * star_b);
    }
    return mk3(r * DLIT(0.6), g * DLIT(0.6), b * DLIT(0.6));
}

template <class T>
__device__ __forceinline__ V3<T> disc_shade(const View<T>& v, T r_cross, T phi_cross, T T_local, T g) {
    const V3<T> col = blackbody_srgb(g * T_local);
    const T flux = clampv(DM<T>::pow_(v.r_in / r_cross, DLIT(3.0)), DLIT(0.05), DLIT(1.5));
    const T bands = disc_band_mask(r_cross, phi_cross, v.r_in, v.turbulence, v.time_sec);
    const T g2 = g * g;
    const T k = flux * bands * g2 * g2;
    return mk3(col.x * k, col.y * k, col.z * k);
}

// Kerr disc colour (geodesic_kernel.cu:368-393).
template <class T> __device__ inline V3<T> kerr_disc(const View<T>& v, T L, T r_cross, T phi_cross, T T_local) {
    const T f_emit = DLIT(1.0) - DLIT(2.0) * v.M / r_cross;
    const T g_grav = (v.flags & SGX_FLAG_REDSHIFT_ON)
                         ? DM<T>::sqrt_(DM<T>::fmax_(f_emit, DLIT(1e-6)) / DM<T>::fmax_(v.f_obs, DLIT(1e-6)))
                         : DLIT(1.0);
    T g_dop = DLIT(1.0);
    if (v.flags & SGX_FLAG_DOPPLER_ON) {
        const T om0 = DM<T>::sqrt_(v.M / (r_cross * r_cross * r_cross));
        const T omega_K = om0 / (DLIT(1.0) + v.a * om0);
        const T vel = r_cross * omega_K / DM<T>::sqrt_(DM<T>::fmax_(f_emit, DLIT(1e-6)));
        const T cos_psi = clampv(L / r_cross, DLIT(-1.0), DLIT(1.0));
        g_dop = DM<T>::sqrt_(DM<T>::fmax_(DLIT(1.0) - vel * vel, DLIT(0.0)))
                / DM<T>::fmax_(DLIT(1.0) - vel * cos_psi, DLIT(1e-4));
    }
    return disc_shade(v, r_cross, phi_cross, T_local, g_grav * g_dop);
}

// Schwarzschild disc colour (geodesic_kernel.cu:266-287).
template <class T> __device__ inline V3<T> schw_disc(const View<T>& v, T uphi_cross, T r_cross, T phi, T T_local) {
    const T f_emit = DLIT(1.0) - v.rs / r_cross;
    const T g_grav = (v.flags & SGX_FLAG_REDSHIFT_ON) ? DM<T>::sqrt_(DM<T>::fmax_(f_emit / v.f_cam, DLIT(0.0)))
                                                      : DLIT(1.0);
    T g_dop = DLIT(1.0);
    if (v.flags & SGX_FLAG_DOPPLER_ON) {
        const T omega = DM<T>::sqrt_(v.M / (r_cross * r_cross * r_cross));
        const T vel = r_cross * omega / DM<T>::sqrt_(DM<T>::fmax_(f_emit, DLIT(1e-6)));
        const T cos_psi = clampv(-uphi_cross * r_cross, DLIT(-1.0), DLIT(1.0));
        g_dop = DM<T>::sqrt_(DM<T>::fmax_(DLIT(1.0) - vel * vel, DLIT(0.0)))
                / DM<T>::fmax_(DLIT(1.0) - vel * cos_psi, DLIT(1e-4));
    }
    return disc_shade(v, r_cross, phi, T_local, g_grav * g_dop);
}

// ACES (Narkowicz) of hdr * exposure (geodesic_kernel.cu:413-422).
template <class T> __device__ __forceinline__ T aces1(T x) {
    return clampv((x * (DLIT(2.51) * x + DLIT(0.03))) / (x * (DLIT(2.43) * x + DLIT(0.59)) + DLIT(0.14)), DLIT(0.0),
                  DLIT(1.0));
}

__device__ __forceinline__ float linear_to_srgb(float c) {
    c = fminf(fmaxf(c, 0.0f), 1.0f);
    return c <= 0.0031308f ? 12.92f * c : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ std::uint8_t to_u8(float c) {
    return (std::uint8_t)fminf(fmaxf(linear_to_srgb(c) * 255.0f + 0.5f, 0.0f), 255.0f);
}

// ---------------------------------------------------------------------------
// Kerr Hamiltonian right-hand side (kerr_hamilton.h:97-155), t dropped.
// ---------------------------------------------------------------------------
template <class T> struct KS {
    T r, th, ph, pr, pth;
};

// Per-ray constants of motion and the products the separated form folds.
template <class T> struct KC {
    T E, L;
    T aE, aL;          // a E, a L
    T twoaE, twoE;     // 2 a E, 2 E
};

template <class T> __device__ __forceinline__ KC<T> make_kc(const View<T>& v, T E, T L) {
    KC<T> c;
    c.E = E;
    c.L = L;
    c.aE = v.a * E;
    c.aL = v.a * L;
    c.twoaE = DLIT(2.0) * c.aE;
    c.twoE = DLIT(2.0) * E;
    return c;
}

// The reference's expression, division for division, with sin(theta) and
// cos(theta) given.
template <class T>
__device__ __forceinline__ KS<T> kerr_rhs_ref_sc(const KS<T>& s, T st, T ct, const View<T>& v, const KC<T>& c) {
    const T r = s.r;
    const T s2 = st * st;
    const T safe_s2 = (s2 < DLIT(1e-10)) ? DLIT(1e-10) : s2;
    const T c2 = ct * ct;
    const T r2 = r * r;
    const T a = v.a, Mm = v.M, a2 = v.a2;
    const T Sigma = r2 + a2 * c2;
    const T Delta = r2 - DLIT(2.0) * Mm * r + a2;
    const T A = (r2 + a2) * (r2 + a2) - a2 * Delta * s2;
    const T SD = Sigma * Delta;
    const T E = c.E, L = c.L, L2 = L * L;
    KS<T> d;
    d.ph = (DLIT(2.0) * Mm * r * a * E * s2 + (Delta - a2 * s2) * L) / (SD * safe_s2);
    d.r = Delta * s.pr / Sigma;
    d.th = s.pth / Sigma;
    const T B = -A * E * E + DLIT(4.0) * Mm * r * a * E * L - a2 * L2;
    const T Sig_r = DLIT(2.0) * r;
    const T Del_r = DLIT(2.0) * r - DLIT(2.0) * Mm;
    const T A_r = DLIT(4.0) * r * (r2 + a2) - a2 * Del_r * s2;
    const T B_r = -A_r * E * E + DLIT(4.0) * Mm * a * E * L;
    const T sin2t = DLIT(2.0) * st * ct;
    const T Sig_t = -a2 * sin2t;
    const T B_t = a2 * Delta * sin2t * E * E;
    const T Sigma2 = Sigma * Sigma;
    const T Dp2 = Delta * s.pr * s.pr + s.pth * s.pth;
    const T dH_dr = B_r / SD - B * (Sig_r * Delta + Sigma * Del_r) / (SD * SD) - L2 * Sig_r / (Sigma2 * safe_s2)
                    + Del_r * s.pr * s.pr / Sigma - Dp2 * Sig_r / Sigma2;
    const T dH_dth = B_t / SD - B * Sig_t / (Sigma2 * Delta)
                     - L2 * (Sig_t * safe_s2 + Sigma * sin2t) / (Sigma2 * safe_s2 * safe_s2) - Dp2 * Sig_t / Sigma2;
    d.pr = DLIT(-0.5) * dH_dr;
    d.pth = DLIT(-0.5) * dH_dth;
    return d;
}

template <class T> __device__ __forceinline__ KS<T> kerr_rhs_ref(const KS<T>& s, const View<T>& v, const KC<T>& c) {
    T st, ct;
    DM<T>::sincos_(s.th, &st, &ct);
    return kerr_rhs_ref_sc(s, st, ct, v, c);
}

// Packed FP32 pairs (PTX .f32x2, sm_100 and later): one instruction performs
// the operation on both lanes with the scalar instruction's rounding, so a
// component-wise update of the state costs half the issue slots.
struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 f2(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unf2(F2 x, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v)); }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}

// The same Hamiltonian in Carter's separated form (Carter 1968), with three
// reciprocals.  With s2 = sin^2(theta), P = (r^2 + a^2) E - a L and
// W = L - a E s2,
//   2 Sigma H = N = Delta p_r^2 + p_th^2 - P^2 / Delta + W^2 / s2,
// which equals the reference's grouping identically: -P^2/Delta + W^2/s2 =
// B/Delta + L^2/s2 with B = -A E^2 + 4 M a r E L - a^2 L^2 (expand and use
// r^2 + a^2 - Delta = 2 M r).  With Q = P/Delta and U = W/s2:
//   dr = Delta p_r / Sigma,   dth = p_th / Sigma,   dphi = (a Q + U) / Sigma
//   dp_r  = -(N_r  - N Sigma_r  / Sigma) / (2 Sigma) = (r N/Sigma + (M - r)(p_r^2 + Q^2) + 2 E r Q) / Sigma
//   dp_th = -(N_th - N Sigma_th / Sigma) / (2 Sigma) = -sin(th) cos(th) (a^2 N/Sigma - U (2 a E + U)) / Sigma
// using N_r = 2 (r - M)(p_r^2 + Q^2) - 4 r E Q, Sigma_r = 2 r,
// N_th = -sin(2 th) U (2 a E + U), Sigma_th = -a^2 sin(2 th).  About 41
// operations against the reference grouping's ~75; the 1/sin^2 guard (1e-10)
// applies to U as it does to the reference's L^2/s2 terms.
template <class T>
__device__ __forceinline__ KS<T> kerr_rhs_sep_sc(const KS<T>& s, T st, T ct, const View<T>& v, const KC<T>& c) {
    if constexpr (std::is_same_v<T, float>) {
        // the same operations with independent pairs packed (.f32x2)
        const float r = s.r, a2 = v.a2;
        float s2, c2, pr2, pth2;
        unf2(mul2(f2(st, ct), f2(st, ct)), s2, c2);
        unf2(mul2(f2(s.pr, s.pth), f2(s.pr, s.pth)), pr2, pth2);
        const float safe_s2 = fmaxf(s2, 1e-10f);
        const float r2 = r * r;
        const float r2a2 = r2 + a2;
        const float Sigma = r2 + a2 * c2;
        const float Delta = r2a2 - v.twoM * r;
        const float P = r2a2 * c.E - c.aL;
        const float W = c.L - c.aE * s2;
        const float iS = DM<float>::rcp_fast(Sigma);
        const float iD = DM<float>::rcp_fast(Delta);
        const float is2 = DM<float>::rcp_fast(safe_s2);
        float Q, U;
        unf2(mul2(f2(P, W), f2(iD, is2)), Q, U);
        KS<T> d;
        d.th = s.pth * iS;
        unf2(mul2(f2(Delta * s.pr, v.a * Q + U), f2(iS, iS)), d.r, d.ph);
        const float N = ((Delta * pr2 + pth2) - P * Q) + W * U;
        const float NiS = N * iS;
        const float A3 = r * NiS + ((v.M - r) * (Q * Q + pr2) + (c.twoE * r) * Q);
        const float B4 = a2 * NiS - U * (c.twoaE + U);
        unf2(mul2(f2(A3, B4), f2(iS, -(iS * (st * ct)))), d.pr, d.pth);
        return d;
    }
    const T r = s.r;
    const T a2 = v.a2;
    const T s2 = st * st;
    const T safe_s2 = DM<T>::fmax_(s2, DLIT(1e-10));
    const T r2 = r * r;
    const T r2a2 = r2 + a2;
    const T Sigma = r2 + a2 * (ct * ct);
    const T Delta = r2a2 - v.twoM * r;
    const T P = r2a2 * c.E - c.aL;
    const T W = c.L - c.aE * s2;
    const T iS = DM<T>::rcp_fast(Sigma);
    const T iD = DM<T>::rcp_fast(Delta);
    const T is2 = DM<T>::rcp_fast(safe_s2);
    const T Q = P * iD;
    const T U = W * is2;
    KS<T> d;
    d.r = Delta * s.pr * iS;
    d.th = s.pth * iS;
    d.ph = (v.a * Q + U) * iS;
    const T pr2 = s.pr * s.pr;
    const T N = ((Delta * pr2 + s.pth * s.pth) - P * Q) + W * U;
    const T NiS = N * iS;
    d.pr = (r * NiS + ((v.M - r) * (Q * Q + pr2) + (c.twoE * r) * Q)) * iS;
    d.pth = -(iS * (st * ct)) * (a2 * NiS - U * (c.twoaE + U));
    return d;
}

// Kerr RHS forms: 0 = the reference's divisions, 1 = the separated form.
constexpr int RHS_REF = 0, RHS_SEP = 1;

template <class T, int FORM> __device__ __forceinline__ void rhs_sincos(T x, T* s, T* c) {
    DM<T>::sincos_(x, s, c);
}

template <class T, int FORM = RHS_SEP>
__device__ __forceinline__ KS<T> kerr_rhs_fast(const KS<T>& s, const View<T>& v, const KC<T>& c) {
    T st, ct;
    rhs_sincos<T, FORM>(s.th, &st, &ct);
    return kerr_rhs_sep_sc(s, st, ct, v, c);
}

template <class T, int FORM>
__device__ __forceinline__ KS<T> kerr_rhs(const KS<T>& s, const View<T>& v, const KC<T>& c) {
    if constexpr (FORM != RHS_REF) return kerr_rhs_fast<T, FORM>(s, v, c);
    else return kerr_rhs_ref(s, v, c);
}

template <class T> __device__ __forceinline__ KS<T> ks_axpy(const KS<T>& y, const KS<T>& k, T f) {
    return KS<T>{y.r + k.r * f, y.th + k.th * f, y.ph + k.ph * f, y.pr + k.pr * f, y.pth + k.pth * f};
}

// Step of the fixed-step integrators: h_step, or with SGX_FLAG_ADAPTIVE_STEP
// the radius-adaptive h_step * clamp(r / 6M, 1, 40) (geodesic_math.h:91-96,
// applied by the reference's WebGPU kernel, geodesic_kernel.wgsl:117-122).
template <class T> __device__ __forceinline__ T fixed_step_h(const View<T>& v, T r) {
    if (!(v.flags & SGX_FLAG_ADAPTIVE_STEP)) return v.h;
    T mult = r / (DLIT(6.0) * v.M);
    mult = (mult < DLIT(1.0)) ? DLIT(1.0) : mult;
    mult = (mult > DLIT(40.0)) ? DLIT(40.0) : mult;
    return v.h * mult;
}

// Fixed-step RK4 with the reference's near-pole damping (kerr_hamilton.h:165-178).
template <class T, int FORM>
__device__ __forceinline__ KS<T> kerr_rk4(const KS<T>& y, T h, const View<T>& v, const KC<T>& c) {
    // sin(theta) of the step's start serves both the pole damping and k1.
    T s0, c0;
    rhs_sincos<T, FORM>(y.th, &s0, &c0);
    T st = (s0 < DLIT(0.0)) ? -s0 : s0;
    T ps = st * DLIT(5.0);
    ps = (ps > DLIT(1.0)) ? DLIT(1.0) : ((ps < DLIT(0.05)) ? DLIT(0.05) : ps);
    h = h * ps;
    const T hh = DLIT(0.5) * h;
    KS<T> k1;
    if constexpr (FORM != RHS_REF) k1 = kerr_rhs_sep_sc(y, s0, c0, v, c);
    else k1 = kerr_rhs_ref(y, v, c);
    const KS<T> k2 = kerr_rhs<T, FORM>(ks_axpy(y, k1, hh), v, c);
    const KS<T> k3 = kerr_rhs<T, FORM>(ks_axpy(y, k2, hh), v, c);
    const KS<T> k4 = kerr_rhs<T, FORM>(ks_axpy(y, k3, h), v, c);
    const T h6 = h / DLIT(6.0);
    KS<T> o;
    o.r = y.r + ((k1.r + k2.r * DLIT(2.0)) + (k3.r * DLIT(2.0) + k4.r)) * h6;
    o.th = y.th + ((k1.th + k2.th * DLIT(2.0)) + (k3.th * DLIT(2.0) + k4.th)) * h6;
    o.ph = y.ph + ((k1.ph + k2.ph * DLIT(2.0)) + (k3.ph * DLIT(2.0) + k4.ph)) * h6;
    o.pr = y.pr + ((k1.pr + k2.pr * DLIT(2.0)) + (k3.pr * DLIT(2.0) + k4.pr)) * h6;
    o.pth = y.pth + ((k1.pth + k2.pth * DLIT(2.0)) + (k3.pth * DLIT(2.0) + k4.pth)) * h6;
    return o;
}

// The same step with sin(theta), cos(theta) carried alongside the state
// (st, ct: in and out): the stages read them instead of evaluating sin and
// cos (ds = cos dtheta, dc = -sin dtheta), and the pair is put back on the unit
// circle after the step by n = 3/2 - (s^2 + c^2)/2; theta itself is still
// integrated for the reference's crossing test.  Separated right-hand side.
template <class T>
__device__ __forceinline__ KS<T> kerr_rk4_sc(const KS<T>& y, T& st, T& ct, T h, const View<T>& v, const KC<T>& c) {
    T ps = DM<T>::fmin_(DM<T>::fmax_((st < DLIT(0.0) ? -st : st) * DLIT(5.0), DLIT(0.05)), DLIT(1.0));
    h = h * ps;
    const T hh = DLIT(0.5) * h;
    const KS<T> k1 = kerr_rhs_sep_sc(y, st, ct, v, c);
    const T s1 = st + (ct * k1.th) * hh, c1 = ct - (st * k1.th) * hh;
    const KS<T> k2 = kerr_rhs_sep_sc(ks_axpy(y, k1, hh), s1, c1, v, c);
    const T s2 = st + (c1 * k2.th) * hh, c2 = ct - (s1 * k2.th) * hh;
    const KS<T> k3 = kerr_rhs_sep_sc(ks_axpy(y, k2, hh), s2, c2, v, c);
    const T s3 = st + (c2 * k3.th) * h, c3 = ct - (s2 * k3.th) * h;
    const KS<T> k4 = kerr_rhs_sep_sc(ks_axpy(y, k3, h), s3, c3, v, c);
    const T h6 = h / DLIT(6.0);
    auto comb = [&](T y0, T a1, T a2, T a3, T a4) { return y0 + ((a1 + a2 * DLIT(2.0)) + (a3 * DLIT(2.0) + a4)) * h6; };
    KS<T> o;
    o.r = comb(y.r, k1.r, k2.r, k3.r, k4.r);
    o.th = comb(y.th, k1.th, k2.th, k3.th, k4.th);
    o.ph = comb(y.ph, k1.ph, k2.ph, k3.ph, k4.ph);
    o.pr = comb(y.pr, k1.pr, k2.pr, k3.pr, k4.pr);
    o.pth = comb(y.pth, k1.pth, k2.pth, k3.pth, k4.pth);
    const T sn = comb(st, ct * k1.th, c1 * k2.th, c2 * k3.th, c3 * k4.th);
    const T cn = comb(ct, -(st * k1.th), -(s1 * k2.th), -(s2 * k3.th), -(s3 * k4.th));
    const T n = DLIT(1.5) - DLIT(0.5) * (sn * sn + cn * cn);
    st = sn * n;
    ct = cn * n;
    return o;
}

// Initial canonical state from a camera direction (geodesic_kernel.cu:320-344).
// Returns false when the u^t quadratic has no real root.
template <class T>
__device__ __forceinline__ bool kerr_init(const View<T>& v, const CamDir<T>& cd, KS<T>& y, T& E, T& L) {
    const T A_q = v.g_tt;
    const T B_q = DLIT(2.0) * v.g_tp * cd.uphi;
    const T C_q = v.g_rr * cd.ur * cd.ur + v.g_thth * cd.utheta * cd.utheta + v.g_pp * cd.uphi * cd.uphi;
    const T disc_q = B_q * B_q - DLIT(4.0) * A_q * C_q;
    if (disc_q < DLIT(0.0)) return false;
    const T ut = (-B_q - DM<T>::sqrt_(disc_q)) / (DLIT(2.0) * A_q);
    E = -(v.g_tt * ut + v.g_tp * cd.uphi);
    L = v.g_tp * ut + v.g_pp * cd.uphi;
    y.r = v.cam_r;
    y.th = v.cam_theta;
    y.ph = v.cam_phi;
    y.pr = v.g_rr * cd.ur;
    y.pth = v.g_thth * cd.utheta;
    return true;
}

// FP64 constants of motion from the FP32 camera direction (mixed form).
__device__ __forceinline__ bool kerr_init_fp64_constants(const View<float>& v, const CamDir<float>& cd, double& E,
                                                         double& L, double& pr, double& pth) {
    // the metric at the camera is per view (View::*_d); per ray one FP64 sqrt
    const double ur = cd.ur, uth = cd.utheta, uph = cd.uphi;
    const double B = 2.0 * v.g_tp_d * uph, C = v.g_rr_d * ur * ur + v.g_thth_d * uth * uth + v.g_pp_d * uph * uph;
    const double disc = B * B - 4.0 * v.g_tt_d * C;
    if (disc < 0.0) return false;
    const double ut = (-B - sqrt(disc)) * v.inv_2gtt_d;
    E = -(v.g_tt_d * ut + v.g_tp_d * uph);
    L = v.g_tp_d * ut + v.g_pp_d * uph;
    pr = v.g_rr_d * ur;
    pth = v.g_thth_d * uth;
    return true;
}

// ---------------------------------------------------------------------------
// Schwarzschild (geodesic_math.h:101-134), t dropped.
// ---------------------------------------------------------------------------
template <class T> struct SS {
    T r, th, ph, ut, ur, uth, uph;
};

template <class T> __device__ __forceinline__ SS<T> schw_rhs(const SS<T>& s, T rs) {
    const T f = DLIT(1.0) - rs / s.r;
    const T r2 = s.r * s.r;
    T sin_t, cos_t;
    DM<T>::sincos_(s.th, &sin_t, &cos_t);
    SS<T> d;
    d.r = s.ur;
    d.th = s.uth;
    d.ph = s.uph;
    d.ut = -(rs / (r2 * f)) * s.ut * s.ur;
    d.ur = -(rs * f / (DLIT(2.0) * r2)) * s.ut * s.ut + (rs / (DLIT(2.0) * r2 * f)) * s.ur * s.ur
           + s.r * f * (s.uth * s.uth + sin_t * sin_t * s.uph * s.uph);
    d.uth = DLIT(-2.0) * s.ur * s.uth / s.r + sin_t * cos_t * s.uph * s.uph;
    d.uph = DLIT(-2.0) * s.ur * s.uph / s.r - DLIT(2.0) * (cos_t / sin_t) * s.uth * s.uph;
    return d;
}

template <class T> __device__ __forceinline__ SS<T> ss_axpy(const SS<T>& y, const SS<T>& k, T f) {
    return SS<T>{y.r + k.r * f,   y.th + k.th * f,   y.ph + k.ph * f,  y.ut + k.ut * f,
                 y.ur + k.ur * f, y.uth + k.uth * f, y.uph + k.uph * f};
}

template <class T> __device__ __forceinline__ SS<T> schw_rk4(const SS<T>& y, T h, T rs) {
    const T hh = DLIT(0.5) * h;
    const SS<T> k1 = schw_rhs(y, rs);
    const SS<T> k2 = schw_rhs(ss_axpy(y, k1, hh), rs);
    const SS<T> k3 = schw_rhs(ss_axpy(y, k2, hh), rs);
    const SS<T> k4 = schw_rhs(ss_axpy(y, k3, h), rs);
    const T h6 = h / DLIT(6.0);
    auto comb = [&](T y0, T a1, T a2, T a3, T a4) { return y0 + ((a1 + a2 * DLIT(2.0)) + (a3 * DLIT(2.0) + a4)) * h6; };
    return SS<T>{comb(y.r, k1.r, k2.r, k3.r, k4.r),         comb(y.th, k1.th, k2.th, k3.th, k4.th),
                 comb(y.ph, k1.ph, k2.ph, k3.ph, k4.ph),     comb(y.ut, k1.ut, k2.ut, k3.ut, k4.ut),
                 comb(y.ur, k1.ur, k2.ur, k3.ur, k4.ur),     comb(y.uth, k1.uth, k2.uth, k3.uth, k4.uth),
                 comb(y.uph, k1.uph, k2.uph, k3.uph, k4.uph)};
}

template <class T> __device__ __forceinline__ SS<T> schw_init(const View<T>& v, const CamDir<T>& cd) {
    SS<T> s;
    s.r = v.cam_r;
    s.th = v.cam_theta;
    s.ph = v.cam_phi;
    s.ur = cd.ur;
    s.uth = cd.utheta;
    s.uph = cd.uphi;
    const T kin = (cd.ur * cd.ur) / v.f_cam + cd.utheta * cd.utheta * v.cam_r * v.cam_r
                  + cd.uphi * cd.uphi * v.cam_r * v.cam_r * v.sin_th * v.sin_th;
    s.ut = DM<T>::sqrt_(DM<T>::fmax_(kin / v.f_cam, DLIT(0.0)));
    return s;
}

// Equatorial crossing of theta = pi/2 between two samples
// (disc_intersection.h:30-55); frac only meaningful when crossed.
template <class T> __device__ __forceinline__ bool crossed_equator(T th_prev, T th_curr, T& frac) {
    const T mid = DLIT(1.5707963267948966);
    const T dp = th_prev - mid;
    const T dc = th_curr - mid;
    const bool x = (dp * dc) < DLIT(0.0);
    frac = x ? (mid - th_prev) / (th_curr - th_prev) : DLIT(0.0);
    return x;
}

// ---------------------------------------------------------------------------
// Error-controlled Kerr integration (the adaptive extension; the CPU oracle's
// adaptive_oracle.hpp is its specification, operation for operation).  theta
// is carried as (sin theta, cos theta): ds = c dtheta, dc = -s dtheta, so no
// stage evaluates a sine or cosine.
// ---------------------------------------------------------------------------
template <class T> struct KSC {
    T r, s, c, ph, pr, pth;
};

template <class T> __device__ __forceinline__ KSC<T> ksc_axpy(const KSC<T>& y, const KSC<T>& k, T f) {
    if constexpr (std::is_same_v<T, float>) {
        const F2 ff = f2(f, f);
        KSC<T> o;
        unf2(fma2(f2(k.s, k.c), ff, f2(y.s, y.c)), o.s, o.c);
        unf2(fma2(f2(k.r, k.ph), ff, f2(y.r, y.ph)), o.r, o.ph);
        unf2(fma2(f2(k.pr, k.pth), ff, f2(y.pr, y.pth)), o.pr, o.pth);
        return o;
    } else {
        return KSC<T>{y.r + k.r * f, y.s + k.s * f, y.c + k.c * f, y.ph + k.ph * f, y.pr + k.pr * f, y.pth + k.pth * f};
    }
}

template <class T, int FORM>
__device__ __forceinline__ KSC<T> kerr_rhs_scs(const KSC<T>& y, const View<T>& v, const KC<T>& c) {
    const KS<T> k{y.r, DLIT(0.0), y.ph, y.pr, y.pth};
    KS<T> d;
    if constexpr (FORM != RHS_REF) d = kerr_rhs_sep_sc(k, y.s, y.c, v, c);
    else d = kerr_rhs_ref_sc(k, y.s, y.c, v, c);
    if constexpr (std::is_same_v<T, float>) {
        float ds, dc;
        unf2(mul2(f2(y.c, y.s), f2(d.th, -d.th)), ds, dc);
        return KSC<T>{d.r, ds, dc, d.ph, d.pr, d.pth};
    } else {
        return KSC<T>{d.r, y.c * d.th, -(y.s * d.th), d.ph, d.pr, d.pth};
    }
}

// (s, c) back to the unit circle after an accepted step: one Newton step of
// 1/sqrt(x) at x = 1 (s^2 + c^2 stays within ~1e-6 of 1 between steps).
template <class T> __device__ __forceinline__ void renormalise(KSC<T>& y) {
    const T n = DLIT(1.5) - DLIT(0.5) * (y.s * y.s + y.c * y.c);
    if constexpr (std::is_same_v<T, float>) {
        unf2(mul2(f2(y.s, y.c), f2(n, n)), y.s, y.c);
    } else {
        y.s = y.s * n;
        y.c = y.c * n;
    }
}

// Carter constant at the camera (geodesic_kernel.cu:340-344).
template <class T> __device__ __forceinline__ T carter_Q(const View<T>& v, T E, T L, T pth) {
    return pth * pth + v.cos_th * v.cos_th * (L * L / DM<T>::fmax_(v.s2_c, DLIT(1e-6)) - v.a2 * E * E);
}

// The same in FP64 from the mixed form's FP64 constants (the camera's cos and
// sin of theta are the view's T values).
template <class T> __device__ __forceinline__ double carter_Q_fp64(const View<T>& v, double E, double L, double pth) {
    const double ct = double(v.cos_th), st = double(v.sin_th), a = double(v.a);
    const double s2 = st * st;
    return pth * pth + ct * ct * (L * L / (s2 > 1e-6 ? s2 : 1e-6) - a * a * E * E);
}

// p_theta put back onto the ray's Carter constant after an accepted step (a
// projection method; Hairer, Lubich & Wanner, Geometric Numerical
// Integration, IV.4): |p_theta| = sqrt(Theta), Theta = Q - c^2 (L^2 / s^2 -
// a^2 E^2), s^2 guarded at 1e-10 as in the right-hand side, the sign of
// p_theta kept (copysign); +-0 where truncation has carried the state past a
// turning point (Theta < 0).  FP32 takes one approximate reciprocal and square
// root (PTX rcp.approx / sqrt.approx, within 2 ulp of the IEEE results).
template <class T> __device__ __forceinline__ T project_pth(T pth, T s, T c, T Q, const KC<T>& k) {
    const T s2 = DM<T>::fmax_(s * s, DLIT(1e-10));
    const T th = Q - c * c * (k.L * k.L * DM<T>::rcp_fast(s2) - k.aE * k.aE);
    T m;
    if constexpr (std::is_same_v<T, float>) {
        const float x = fmaxf(th, 0.0f);
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(m) : "f"(x));
        return copysignf(m, pth);
    } else {
        m = th > 0.0 ? sqrt(th) : 0.0;
        return copysign(m, pth);
    }
}

// Constants of motion of a final state, in FP64 (diagnostics): the Carter
// constant with theta from (s, c) and 2H in the reference's grouping
// (kerr_hamilton.h:37-60; the CPU oracle's kerr_two_H).
template <class T>
__device__ __forceinline__ void kerr_invariants_fp64(const View<T>& v, double E, double L, double r, double s,
                                                     double c, double pr, double pth, double& Q, double& H2) {
    const double n2 = s * s + c * c;
    const double st2 = s * s / n2, ct2 = c * c / n2;
    const double a = double(v.a), Mm = double(v.M);
    Q = pth * pth + ct2 * (L * L / (st2 > 1e-300 ? st2 : 1e-300) - a * a * E * E);
    const double safe_s2 = st2 < 1e-10 ? 1e-10 : st2;
    const double r2 = r * r, a2 = a * a;
    const double Sigma = r2 + a2 * ct2, Delta = r2 - 2.0 * Mm * r + a2;
    const double A = (r2 + a2) * (r2 + a2) - a2 * Delta * st2;
    const double SD = Sigma * Delta;
    H2 = -A * E * E / SD + 4.0 * Mm * r * a * E * L / SD + (Delta - a2 * safe_s2) * L * L / (SD * safe_s2) +
         Delta * pr * pr / Sigma + pth * pth / Sigma;
}

template <class T> struct KAttempt {
    KSC<T> y4, k4, k5;
    T h6;
};

// RK4 stages from y with k1 = f(y) known, plus the first-same-as-last stage.
template <class T, int FORM>
__device__ __forceinline__ KAttempt<T> kerr_attempt(const KSC<T>& y, const KSC<T>& k1, T h, const View<T>& v,
                                                    const KC<T>& c) {
    KAttempt<T> at;
    const T hh = DLIT(0.5) * h;
    const KSC<T> k2 = kerr_rhs_scs<T, FORM>(ksc_axpy(y, k1, hh), v, c);
    const KSC<T> k3 = kerr_rhs_scs<T, FORM>(ksc_axpy(y, k2, hh), v, c);
    at.k4 = kerr_rhs_scs<T, FORM>(ksc_axpy(y, k3, h), v, c);
    at.h6 = h * DLIT(0.16666666666666666);  // h/6 as a product (the oracle alike)
    if constexpr (std::is_same_v<T, float>) {
        // y0 + (fma(a2, 2, a1) + fma(a3, 2, a4)) h6 on component pairs
        const F2 two = f2(2.0f, 2.0f), h6 = f2(at.h6, at.h6);
        auto comb2 = [&](F2 y0, F2 a1, F2 a2, F2 a3, F2 a4) {
            return fma2(add2(fma2(a2, two, a1), fma2(a3, two, a4)), h6, y0);
        };
        unf2(comb2(f2(y.s, y.c), f2(k1.s, k1.c), f2(k2.s, k2.c), f2(k3.s, k3.c), f2(at.k4.s, at.k4.c)), at.y4.s,
             at.y4.c);
        unf2(comb2(f2(y.r, y.ph), f2(k1.r, k1.ph), f2(k2.r, k2.ph), f2(k3.r, k3.ph), f2(at.k4.r, at.k4.ph)), at.y4.r,
             at.y4.ph);
        unf2(comb2(f2(y.pr, y.pth), f2(k1.pr, k1.pth), f2(k2.pr, k2.pth), f2(k3.pr, k3.pth),
                   f2(at.k4.pr, at.k4.pth)),
             at.y4.pr, at.y4.pth);
    } else {
        auto comb = [&](T y0, T a1, T a2, T a3, T a4) {
            return y0 + ((a1 + a2 * DLIT(2.0)) + (a3 * DLIT(2.0) + a4)) * at.h6;
        };
        at.y4.r = comb(y.r, k1.r, k2.r, k3.r, at.k4.r);
        at.y4.s = comb(y.s, k1.s, k2.s, k3.s, at.k4.s);
        at.y4.c = comb(y.c, k1.c, k2.c, k3.c, at.k4.c);
        at.y4.ph = comb(y.ph, k1.ph, k2.ph, k3.ph, at.k4.ph);
        at.y4.pr = comb(y.pr, k1.pr, k2.pr, k3.pr, at.k4.pr);
        at.y4.pth = comb(y.pth, k1.pth, k2.pth, k3.pth, at.k4.pth);
    }
    at.k5 = kerr_rhs_scs<T, FORM>(at.y4, v, c);
    return at;
}

// |x| as an operand modifier (a compare-and-select would cost two instructions;
// the two differ only in the sign of a zero result).
__device__ __forceinline__ float absv(float x) { return fabsf(x); }
__device__ __forceinline__ double absv(double x) { return fabs(x); }

// max_i |h/6 (k4_i - k5_i)| / (tol (1 + max(|y_i|, |y4_i|))) over r, sin theta,
// cos theta, phi, p_r, p_theta, evaluated in C; NaN/overflow -> 1e30.
template <class C, class T>
__device__ __forceinline__ C error_norm(const KSC<T>& y, const KAttempt<T>& a, float tol_f) {
    const C tol = C(tol_f);
    const C h6 = C(a.h6);
    auto one = [&](T yv, T y4v, T k4v, T k5v) {
        const C ya = absv(C(yv)), yb = absv(C(y4v));
        const C sc = tol * (C(1.0f) + (ya > yb ? ya : yb));
        return absv(h6 * (C(k4v) - C(k5v))) / sc;
    };
    C e = one(y.r, a.y4.r, a.k4.r, a.k5.r);
    C t;
    t = one(y.s, a.y4.s, a.k4.s, a.k5.s);
    e = t > e ? t : e;
    t = one(y.c, a.y4.c, a.k4.c, a.k5.c);
    e = t > e ? t : e;
    t = one(y.ph, a.y4.ph, a.k4.ph, a.k5.ph);
    e = t > e ? t : e;
    t = one(y.pr, a.y4.pr, a.k4.pr, a.k5.pr);
    e = t > e ? t : e;
    t = one(y.pth, a.y4.pth, a.k4.pth, a.k5.pth);
    e = t > e ? t : e;
    if (!(e <= C(1e30f))) e = C(1e30f);
    return e;
}

// The same norm with one approximate reciprocal per component and a single
// scale at the end: max_i |k4_i - k5_i| / (1 + max(|y_i|, |y4_i|)) * |h/6| / tol.
// Equal to error_norm up to rounding (a few ulp), for the FP32 fast path; the
// subtractions, sums and products run on component pairs, k4 - k5 as
// fma(k5, -1, k4) (one rounding, as the subtraction) and |d| / (1 + m) as
// |d / (1 + m)|.
__device__ __forceinline__ float error_norm_fast(const KSC<float>& y, const KAttempt<float>& a, float tol_f) {
    const F2 one2 = f2(1.0f, 1.0f), neg1 = f2(-1.0f, -1.0f);
    float q[6];
    auto pair = [&](float ya, float yb, float y4a, float y4b, float k4a, float k4b, float k5a, float k5b, float& qa,
                    float& qb) {
        const F2 d = fma2(f2(k5a, k5b), neg1, f2(k4a, k4b));
        float da, db;
        unf2(add2(one2, f2(fmaxf(absv(ya), absv(y4a)), fmaxf(absv(yb), absv(y4b)))), da, db);
        unf2(mul2(d, f2(DM<float>::rcp_fast(da), DM<float>::rcp_fast(db))), qa, qb);
    };
    pair(y.r, y.ph, a.y4.r, a.y4.ph, a.k4.r, a.k4.ph, a.k5.r, a.k5.ph, q[0], q[3]);
    pair(y.s, y.c, a.y4.s, a.y4.c, a.k4.s, a.k4.c, a.k5.s, a.k5.c, q[1], q[2]);
    pair(y.pr, y.pth, a.y4.pr, a.y4.pth, a.k4.pr, a.k4.pth, a.k5.pr, a.k5.pth, q[4], q[5]);
    float e = absv(q[0]);
#pragma unroll
    for (int i = 1; i < 6; ++i) e = fmaxf(e, absv(q[i]));
    e = e * (absv(a.h6) * DM<float>::rcp_fast(tol_f));
    if (!(e <= 1e30f)) e = 1e30f;
    return e;
}

// h *= clamp(0.85 / err^(1/4), 0.2, 4) with IEEE sqrt and division only.
template <class C> __device__ __forceinline__ C step_factor(C e) {
    if (e <= C(1e-30f)) return C(4.0f);
    C f = C(0.85f) / sqrt(sqrt(e));
    f = f < C(0.2f) ? C(0.2f) : f;
    f = f > C(4.0f) ? C(4.0f) : f;
    return f;
}

// The same factor as 0.85 * 2^(-log2(e) / 4) from the SFU's base-2
// logarithm and exponential (PTX lg2.approx / ex2.approx, relative error
// ~2^-22 over the range e takes), clamped without branches.
__device__ __forceinline__ float step_factor_fast(float e) {
    float l, p;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(e));
    const float x = -0.25f * l;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(p) : "f"(x));
    const float f = fminf(fmaxf(0.85f * p, 0.2f), 4.0f);
    return e <= 1e-30f ? 4.0f : f;
}

template <class T> __device__ __forceinline__ T hermite(T y0, T y1, T d0, T d1, T h, T s) {
    const T s2 = s * s, s3 = s2 * s;
    const T h00 = DLIT(2.0) * s3 - DLIT(3.0) * s2 + DLIT(1.0);
    const T h10 = s3 - DLIT(2.0) * s2 + s;
    const T h01 = DLIT(3.0) * s2 - DLIT(2.0) * s3;
    const T h11 = s3 - s2;
    return h00 * y0 + h10 * h * d0 + h01 * y1 + h11 * h * d1;
}
template <class T> __device__ __forceinline__ T hermite_d(T y0, T y1, T d0, T d1, T h, T s) {
    const T s2 = s * s;
    const T h00 = DLIT(6.0) * s2 - DLIT(6.0) * s;
    const T h10 = DLIT(3.0) * s2 - DLIT(4.0) * s + DLIT(1.0);
    const T h01 = DLIT(6.0) * s - DLIT(6.0) * s2;
    const T h11 = DLIT(3.0) * s2 - DLIT(2.0) * s;
    return h00 * y0 + h10 * h * d0 + h01 * y1 + h11 * h * d1;
}

// cos(theta) = 0 inside an accepted step: three Newton steps on the Hermite
// interpolant from the linear estimate, clamped to [0, 1].
template <class T> __device__ __forceinline__ T crossing_fraction(T c0, T c1, T d0, T d1, T h) {
    T s = c0 / (c0 - c1);
#pragma unroll 1
    for (int it = 0; it < 3; ++it) {
        const T f = hermite(c0, c1, d0, d1, h, s);
        const T fp = hermite_d(c0, c1, d0, d1, h, s);
        if (!(absv(fp) > DLIT(1e-30))) break;
        T sn = s - f / fp;
        sn = sn < DLIT(0.0) ? DLIT(0.0) : (sn > DLIT(1.0) ? DLIT(1.0) : sn);
        s = sn;
    }
    return s;
}

// Spherical photon orbit with the ray's xi = L/E (Bardeen 1973, Teo 2003):
// 12 bisections inside [r_ph,pro, r_ph,ret]; 3M for a = 0; NaN outside.
template <class T> __device__ __forceinline__ T photon_orbit_radius(const View<T>& v, T xi) {
    const T a = v.a, Mm = v.M;
    if (!(a > DLIT(1e-7)) && !(a < DLIT(-1e-7))) return DLIT(3.0) * Mm;
    // sign of xi(r) - xi without the division by a (r - M) > 0 (a > 0; flipped for a < 0)
    const T sg = a > DLIT(0.0) ? DLIT(1.0) : DLIT(-1.0);
    auto g = [&](T r) { return sg * ((r * r * (DLIT(3.0) * Mm - r) - a * a * (r + Mm)) - xi * a * (r - Mm)); };
    T lo = v.r_ph_pro, hi = v.r_ph_ret;
    const T flo = g(lo), fhi = g(hi);
    if (!(flo * fhi <= DLIT(0.0))) return T(NAN);
    const bool lo_neg = flo <= DLIT(0.0);
#pragma unroll 1
    for (int i = 0; i < 12; ++i) {
        const T mid = DLIT(0.5) * (lo + hi);
        if ((g(mid) <= DLIT(0.0)) == lo_neg) lo = mid;
        else hi = mid;
    }
    return DLIT(0.5) * (lo + hi);
}

// The mixed form's FP64 error norm with a single division: the component of
// largest |h/6 (k4 - k5)| / (tol (1 + max(|y|, |y4|))) is found by
// cross-multiplied comparisons, then divided once (the value equals the max
// of the ratios up to the choice among ratios equal to rounding).
template <class T>
__device__ __forceinline__ double error_norm_fp64_1div(const KSC<T>& y, const KAttempt<T>& a, float tol_f) {
    const double tol = tol_f, h6 = a.h6;
    double num = 0.0, den = 1.0;
    auto one = [&](T yv, T y4v, T k4v, T k5v) {
        const double ya = fabs(double(yv)), yb = fabs(double(y4v));
        const double sc = tol * (1.0 + (ya > yb ? ya : yb));
        const double n = fabs(h6 * (double(k4v) - double(k5v)));
        if (n * den > num * sc) {
            num = n;
            den = sc;
        }
    };
    one(y.r, a.y4.r, a.k4.r, a.k5.r);
    one(y.s, a.y4.s, a.k4.s, a.k5.s);
    one(y.c, a.y4.c, a.k4.c, a.k5.c);
    one(y.ph, a.y4.ph, a.k4.ph, a.k5.ph);
    one(y.pr, a.y4.pr, a.k4.pr, a.k5.pr);
    one(y.pth, a.y4.pth, a.k4.pth, a.k5.pth);
    double e = num / den;
    if (!(e <= 1e30)) e = 1e30;
    return e;
}

// ---------------------------------------------------------------------------
// Bloom extract (render/vulkan/shaders/bloom.hlsl:13-40): one half-resolution
// texel from a 2x2 block of the HDR frame (the values as the half-precision
// frame holds them): the Karis-weighted average (weights 1 / (1 + luma)),
// scaled by the soft knee luma^2 / max(luma + threshold, 1e-4) / luma.  One
// definition for the separate extract kernel and for the extract fused into
// the last accumulation pass, so the two give the same texel.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float bloom_luma(float r, float g, float b) {
    return r * 0.2126f + g * 0.7152f + b * 0.0722f;
}

__device__ __forceinline__ void karis_extract(float4 a, float4 b, float4 c, float4 d, float threshold, float& r,
                                              float& g, float& bl) {
    const float la = 1.0f / (1.0f + bloom_luma(a.x, a.y, a.z));
    const float lb = 1.0f / (1.0f + bloom_luma(b.x, b.y, b.z));
    const float lc = 1.0f / (1.0f + bloom_luma(c.x, c.y, c.z));
    const float ld = 1.0f / (1.0f + bloom_luma(d.x, d.y, d.z));
    const float wden = fmaxf(la + lb + lc + ld, 1e-6f);
    const float ar = (a.x * la + b.x * lb + c.x * lc + d.x * ld) / wden;
    const float ag = (a.y * la + b.y * lb + c.y * lc + d.y * ld) / wden;
    const float ab = (a.z * la + b.z * lb + c.z * lc + d.z * ld) / wden;
    const float l = bloom_luma(ar, ag, ab);
    const float knee = (l * l) / fmaxf(l + threshold, 1e-4f);
    const float k = (l > 1e-4f) ? (knee / l) : 0.0f;
    r = ar * k;
    g = ag * k;
    bl = ab * k;
}

}  // namespace sgxd
