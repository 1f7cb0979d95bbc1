// oracle/diff_oracle.hpp
//
// TEST INFRASTRUCTURE — CPU specification of the differentiable render form
// (the GPU's forward and adjoint kernels in singularity_gb300/csrc/sgx_diff.cu
// implement it).  Only tests/ and bench.py's checks use it.
//
// The reference renders images that are discontinuous in the scene
// parameters (hard annulus edges, a 1000 K colour floor at the inner edge,
// starfield cells, geodesic_kernel.cu:77-171,262-289), so a per-ray derivative
// and a finite difference disagree by boundary terms.  The differentiable form
// changes exactly that, and nothing else:
//   * the camera orbits at azimuth 0 with elevation pi/2 - incl, its frame
//     written in closed form (position (d sin i, 0, d cos i), forward
//     (-sin i, 0, -cos i), right (0, 1, 0), up (cos i, 0, -sin i): the values
//     cuda_cli/main.cpp:68-109 computes, as functions of i);
//   * the starfield is off (escaped and captured rays are black);
//   * the annulus edges are soft: a crossing at radius r emits with weight
//     w(r) = S((r - r_in)/eps) S((r_out - r)/eps), S(x) = 3x^2 - 2x^3 on [0, 1];
//     the ray carries a transmittance tau (1 at launch): each crossing adds
//     tau w c to the colour and multiplies tau by (1 - w); tau = 0 ends the ray.
//     With eps -> 0 this is the reference's first-hit rule;
//   * optionally, the emission of a crossing is multiplied by
//     1 - S((psi - fade_start) / fade_width), psi the angle the ray has swept
//     around the hole when it crosses (accumulated per step as
//     sqrt(dtheta^2 + sin^2(theta) dphi^2) and interpolated to the crossing):
//     images that wind past fade_start fade out, so rays near the critical
//     curve — whose winding grows without bound and whose higher-order
//     images jump in and out as parameters move — contribute nothing;
//   * the blackbody fit (Tanner Helland's, geodesic_kernel.cu:77-104) jumps at
//     6600 K where it switches branch (green by 0.013, blue by 0.01); the form
//     blends the two branches over 6500-6700 K with S, so colour is continuous
//     in temperature (identical outside that band);
//   * the disc temperature scale multiplies the peak temperature.
//   * a ray is captured inside the prograde photon orbit radius less 0.05 M
//     instead of at 1.02 r_+ (see diff_trace), and ends once it moves outward
//     beyond r_out (escaped rays are black here).
// Integration is the reference's fixed-step Kerr RK4 with its pole damping
// (kerr_hamilton.h:165-178), checks and escape as geodesic_kernel.cu:351-401,
// with sin(theta) and cos(theta) carried as two more state components
// (ds = cos(theta) dtheta, dc = -sin(theta) dtheta, put back on the unit
// circle after each step by n = 3/2 - (s^2 + c^2)/2): the right-hand side and
// the pole damping read them instead of evaluating sin and cos, while theta
// itself is still integrated for the crossing test, the swept angle and the
// slab's path length.


#pragma once

#include <cmath>
#include <cstdint>

#include "geodesic_oracle.hpp"

namespace oracle {

struct DiffParams {
    double spin;      // a / M
    double incl;      // inclination, radians
    double r_in;      // disc inner radius, M
    double t_scale;   // multiplies the peak temperature
};

struct DiffOpts {
    float eps;         // soft-edge width, M (0.1)
    float fade_start;  // swept angle (rad) where higher-order images start to fade; <= 0: no fade
    float fade_width;  // fade length in swept angle (rad)
    std::uint32_t model;  // DIFF_MODEL_CROSSING or DIFF_MODEL_SLAB
    float half_thickness;  // slab: half-thickness H of the emitting layer, M
    float tau_perp;        // slab: optical depth of a perpendicular pass through the layer
    float pad0, pad1;
};
enum : std::uint32_t { DIFF_MODEL_CROSSING = 0, DIFF_MODEL_SLAB = 1 };

// Slab profile: (1 - (z/H)^2)^2 on |z| < H (integral 16 H / 15), C1 at |z| = H.
template <class T> inline T slab_profile(T z, T H) {
    const T q = z / H;
    if (!(q * q < OLIT(1.0))) return OLIT(0.0);
    const T b = OLIT(1.0) - q * q;
    return b * b;
}

template <class T> inline T smooth01(T x) {
    if (x <= OLIT(0.0)) return OLIT(0.0);
    if (x >= OLIT(1.0)) return OLIT(1.0);
    return x * x * (OLIT(3.0) - OLIT(2.0) * x);
}

// Blackbody colour continuous at 6600 K: the fit's low (t <= 66) and high
// (t > 66) branches, t = temperature / 100 K, blended by S((t - 65) / 2).
template <class T> inline V3<T> blackbody_c0(T temp) {
    const T t = vclamp(temp, OLIT(1000.0), OLIT(40000.0)) * OLIT(0.01);
    V3<T> lo, hi;
    const bool need_lo = t < OLIT(67.0), need_hi = t > OLIT(65.0);
    if (need_lo) {
        lo.x = OLIT(1.0);
        lo.y = vclamp(OLIT(0.39008157876901960784) * M<T>::log(t) - OLIT(0.63184144378862745098), OLIT(0.0),
                      OLIT(1.0));
        lo.z = (t <= OLIT(19.0)) ? OLIT(0.0)
                                 : vclamp(OLIT(0.54320678911019607843) * M<T>::log(t - OLIT(10.0)) -
                                              OLIT(1.19625408914),
                                          OLIT(0.0), OLIT(1.0));
    }
    if (need_hi) {
        const T t1 = t - OLIT(60.0);
        hi.x = vclamp(OLIT(1.29293618606274509804) * M<T>::pow(t1, OLIT(-0.1332047592)), OLIT(0.0), OLIT(1.0));
        hi.y = vclamp(OLIT(1.12989086089529411765) * M<T>::pow(t1, OLIT(-0.0755148492)), OLIT(0.0), OLIT(1.0));
        hi.z = OLIT(1.0);
    }
    if (!need_hi) return lo;
    if (!need_lo) return hi;
    const T sb = smooth01((t - OLIT(65.0)) * OLIT(0.5));
    return v3(lo.x + sb * (hi.x - lo.x), lo.y + sb * (hi.y - lo.y), lo.z + sb * (hi.z - lo.z));
}

// Kerr disc colour of the form (geodesic_kernel.cu:368-393 with blackbody_c0).
template <class T>
inline V3<T> diff_disc_colour(const Params<T>& u, const KConst<T>& c, T cam_r, T r_cross, T phi_cross, T T_local) {
    const T Mm = u.mass_M;
    const T f_emit = OLIT(1.0) - OLIT(2.0) * Mm / r_cross;
    const T f_obs = OLIT(1.0) - OLIT(2.0) * Mm / cam_r;
    const T g_grav = (u.flags & SGX_FLAG_REDSHIFT_ON)
                         ? M<T>::sqrt(M<T>::fmax(f_emit, OLIT(1e-6)) / M<T>::fmax(f_obs, OLIT(1e-6)))
                         : OLIT(1.0);
    T g_dop = OLIT(1.0);
    if (u.flags & SGX_FLAG_DOPPLER_ON) {
        const T om0 = M<T>::sqrt(Mm / (r_cross * r_cross * r_cross));
        const T omega_K = om0 / (OLIT(1.0) + u.spin_a * om0);
        const T v = r_cross * omega_K / M<T>::sqrt(M<T>::fmax(f_emit, OLIT(1e-6)));
        const T cos_psi = vclamp(c.L / r_cross, OLIT(-1.0), OLIT(1.0));
        g_dop = M<T>::sqrt(M<T>::fmax(OLIT(1.0) - v * v, OLIT(0.0))) / M<T>::fmax(OLIT(1.0) - v * cos_psi, OLIT(1e-4));
    }
    const T g = g_grav * g_dop;
    const V3<T> col = blackbody_c0(g * T_local);
    const T flux = vclamp(M<T>::pow(u.r_in / r_cross, OLIT(3.0)), OLIT(0.05), OLIT(1.5));
    const T bands = disc_band_mask(r_cross, phi_cross, u.r_in, u.turbulence, u.time_sec);
    const T g2 = g * g;
    return vmul(col, flux * bands * g2 * g2);
}

// State of the form: the Kerr state and (sin theta, cos theta).
template <class T> struct DiffState {
    KState<T> k;  // t unused, r, theta, phi, p_r, p_theta
    T s, c;       // sin(theta), cos(theta)
};

// One fixed RK4 step of DiffState with the reference's pole damping
// h clamp(5 |sin theta|, 0.05, 1) (kerr_hamilton.h:165-178).
template <class T> inline DiffState<T> diff_rk4(const DiffState<T>& y, T h, const KConst<T>& cc) {
    T as = y.s < OLIT(0.0) ? -y.s : y.s;
    T ps = as * OLIT(5.0);
    ps = (ps > OLIT(1.0)) ? OLIT(1.0) : ((ps < OLIT(0.05)) ? OLIT(0.05) : ps);
    const T he = h * ps;
    const T hh = OLIT(0.5) * he;
    auto f = [&](const KState<T>& k, T st, T ct, T& ds, T& dc) {
        const KState<T> d = kerr_rhs_sc<T, false>(k, st, ct, cc);
        ds = ct * d.theta;
        dc = -(st * d.theta);
        return d;
    };
    T ds1, dc1, ds2, dc2, ds3, dc3, ds4, dc4;
    const KState<T> k1 = f(y.k, y.s, y.c, ds1, dc1);
    const KState<T> k2 = f(k_add_scaled(y.k, k1, hh), y.s + ds1 * hh, y.c + dc1 * hh, ds2, dc2);
    const KState<T> k3 = f(k_add_scaled(y.k, k2, hh), y.s + ds2 * hh, y.c + dc2 * hh, ds3, dc3);
    const KState<T> k4 = f(k_add_scaled(y.k, k3, he), y.s + ds3 * he, y.c + dc3 * he, ds4, dc4);
    const T h6 = he / OLIT(6.0);
    DiffState<T> o;
    o.k.t = y.k.t;
    o.k.r = rk4_combine(y.k.r, k1.r, k2.r, k3.r, k4.r, h6);
    o.k.theta = rk4_combine(y.k.theta, k1.theta, k2.theta, k3.theta, k4.theta, h6);
    o.k.phi = rk4_combine(y.k.phi, k1.phi, k2.phi, k3.phi, k4.phi, h6);
    o.k.p_r = rk4_combine(y.k.p_r, k1.p_r, k2.p_r, k3.p_r, k4.p_r, h6);
    o.k.p_theta = rk4_combine(y.k.p_theta, k1.p_theta, k2.p_theta, k3.p_theta, k4.p_theta, h6);
    const T s1 = rk4_combine(y.s, ds1, ds2, ds3, ds4, h6);
    const T c1 = rk4_combine(y.c, dc1, dc2, dc3, dc4, h6);
    const T n = OLIT(1.5) - OLIT(0.5) * (s1 * s1 + c1 * c1);
    o.s = s1 * n;
    o.c = c1 * n;
    return o;
}

template <class T> struct DiffOut {
    V3<T> hdr;
    std::uint32_t steps, crossings;
};

// One sample of the differentiable form.  u supplies size, spp, distance
// (|cam_pos|), FOV, aspect, mass, r_out, peak T, h, max_steps, escape radius,
// exposure, turbulence, time and the Doppler/redshift flags.
// The parameters enter as T, so a dual-number T carries their derivatives
// through the whole trace (diff_pixel_grad).
template <class T>
inline DiffOut<T> diff_trace_p(const sgx_uniforms& ub, T spin, T incl, T r_in_M, T t_scale, const DiffOpts& o,
                               std::uint32_t gx, std::uint32_t gy, std::uint32_t s) {
    const Params<T> u = promote<T>(ub);
    const T Mm = u.mass_M;
    const T a = spin * Mm;
    const T r_in = r_in_M * Mm;
    const T peak_T = u.peak_T * t_scale;
    const T eps = T(o.eps) * Mm;
    const T dcam = M<T>::sqrt(T(ub.cam_pos.x) * T(ub.cam_pos.x) + T(ub.cam_pos.y) * T(ub.cam_pos.y) +
                              T(ub.cam_pos.z) * T(ub.cam_pos.z));
    const T si = M<T>::sin(incl), ci = M<T>::cos(incl);
    // camera frame
    const V3<T> fwd = v3(-si, OLIT(0.0), -ci);
    const V3<T> right = v3(OLIT(0.0), OLIT(1.0), OLIT(0.0));
    const V3<T> up = v3(ci, OLIT(0.0), -si);
    T ox, oy;
    if (u.spp == 1u) {
        ox = OLIT(0.5);
        oy = OLIT(0.5);
    } else {
        ox = halton<T>(s + 1u, 2u);
        oy = halton<T>(s + 1u, 3u);
    }
    const T fx = T(float(gx)) + ox, fy = T(float(gy)) + oy;
    const T u_ndc = (OLIT(2.0) * fx / T(float(u.width)) - OLIT(1.0)) * u.aspect * u.tan_half_fov;
    const T v_ndc = -(OLIT(2.0) * fy / T(float(u.height)) - OLIT(1.0)) * u.tan_half_fov;
    const V3<T> dir = vnormalize(vadd(fwd, vadd(vmul(right, u_ndc), vmul(up, v_ndc))));
    // spherical frame at the camera: theta = incl, phi = 0
    const V3<T> rhat = v3(si, OLIT(0.0), ci);
    const V3<T> that = v3(ci, OLIT(0.0), -si);
    const V3<T> phat = v3(OLIT(0.0), OLIT(1.0), OLIT(0.0));
    CamRay<T> cam;
    cam.cart = dir;
    cam.cam_r = dcam;
    cam.cam_theta = incl;
    cam.cam_phi = OLIT(0.0);
    cam.sin_th = si;
    cam.ur = vdot(dir, rhat);
    cam.utheta = vdot(dir, that) / dcam;
    cam.uphi = vdot(dir, phat) / (dcam * M<T>::fmax(si, OLIT(1e-6)));

    Params<T> up_ = u;
    up_.spin_a = a;
    up_.r_in = r_in;
    up_.peak_T = peak_T;
    DiffState<T> ys;
    KState<T>& y = ys.k;
    KConst<T> c;
    DiffOut<T> out{v3(OLIT(0.0), OLIT(0.0), OLIT(0.0)), 0u, 0u};
    // kerr_init reads cos(cam_theta) itself; the closed-form frame above agrees with it.
    if (!kerr_init(cam, up_, y, c)) return out;
    ys.s = si;
    ys.c = ci;
    // Capture radius: the prograde equatorial photon orbit radius (the smallest
    // photon orbit; an ingoing ray from outside that gets inside it falls in)
    // less 0.05 M.  The fixed-step RK4 turns unstable as Delta -> 0, and the
    // reference's cut at 1.02 r_+ lets a blown-up state emit before it stops.
    const T r_pro = OLIT(2.0) * Mm * (OLIT(1.0) + M<T>::cos(OLIT(2.0) / OLIT(3.0) * M<T>::acos(-a / Mm)));
    const T hcut = M<T>::fmax(r_pro - OLIT(0.05) * Mm, kerr_horizon_cut(Mm, a));
    T tau = OLIT(1.0);
    KState<T> prev = y;
    T psi = OLIT(0.0), psi_prev = OLIT(0.0);
    const bool fade = o.fade_start > 0.0f;
    std::uint32_t step = 0;
    const bool slab = o.model == DIFF_MODEL_SLAB;
    const T H = T(o.half_thickness) * Mm;
    const T kappa = T(o.tau_perp) / (OLIT(16.0) / OLIT(15.0) * H);
    for (; step < u.max_steps; ++step) {
        if (!M<T>::isfinite(y.r) || y.r < hcut) break;
        if (y.r > u.escape_r) break;
        if (slab && (u.flags & SGX_FLAG_DISC_ON) && step > 0) {
            // emission and absorption of the step prev -> y, evaluated at y
            const T z = y.r * ys.c;
            const T rho = slab_profile(z, H);
            T w = smooth01((y.r - r_in) / eps) * smooth01((u.r_out - y.r) / eps);
            if (fade) w = w * (OLIT(1.0) - smooth01((psi - T(o.fade_start)) / T(o.fade_width)));
            if (rho > OLIT(0.0) && w > OLIT(0.0)) {
                const T dr = y.r - prev.r, dth = y.theta - prev.theta, dph = y.phi - prev.phi;
                const T st = ys.s;
                const T ds = M<T>::sqrt(dr * dr + y.r * y.r * (dth * dth + st * st * dph * dph));
                const T alpha = w * (OLIT(1.0) - M<T>::exp(-kappa * rho * ds));
                ++out.crossings;
                const T T_local = disc_temperature(y.r, r_in, peak_T);
                V3<T> col = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
                if (T_local > OLIT(0.0)) col = diff_disc_colour(up_, c, dcam, y.r, y.phi, T_local);
                out.hdr = vadd(out.hdr, vmul(col, tau * alpha));
                tau = tau * (OLIT(1.0) - alpha);
            }
        }
        if (!slab && (u.flags & SGX_FLAG_DISC_ON)) {
            const Crossing<T> x = equatorial_crossing(prev.theta, y.theta);
            if (x.crossed) {
                const T r_c = lerp_s(prev.r, y.r, x.frac);
                T w = smooth01((r_c - r_in) / eps) * smooth01((u.r_out - r_c) / eps);
                if (fade) {
                    const T psi_c = lerp_s(psi_prev, psi, x.frac);
                    w = w * (OLIT(1.0) - smooth01((psi_c - T(o.fade_start)) / T(o.fade_width)));
                }
                if (w > OLIT(0.0)) {
                    ++out.crossings;
                    const T T_local = disc_temperature(r_c, r_in, peak_T);
                    V3<T> col = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
                    if (T_local > OLIT(0.0)) col = diff_disc_colour(up_, c, dcam, r_c, y.phi, T_local);
                    const T k = tau * w;
                    out.hdr = vadd(out.hdr, vmul(col, k));
                    tau = tau * (OLIT(1.0) - w);
                    if (!(tau > OLIT(0.0))) break;
                }
            }
        }
        // outgoing beyond the disc (after this step's emission or crossing): no
        // turning point is left (no bound photon orbits outside the photon
        // region) and nothing emits out there
        if (y.p_r > OLIT(0.0) && y.r > u.r_out) break;
        prev = y;
        ys = diff_rk4(ys, u.h_step, c);
        if (fade) {
            const T dth = y.theta - prev.theta, dph = y.phi - prev.phi, st = ys.s;
            psi_prev = psi;
            psi = psi + M<T>::sqrt(dth * dth + st * st * dph * dph);
        }
    }
    out.steps = step;
    return out;
}

template <class T>
inline DiffOut<T> diff_trace(const sgx_uniforms& ub, const DiffParams& dp, const DiffOpts& o, std::uint32_t gx,
                             std::uint32_t gy, std::uint32_t s) {
    return diff_trace_p<T>(ub, T(dp.spin), T(dp.incl), T(dp.r_in), T(dp.t_scale), o, gx, gy, s);
}

// Image of the form: per pixel the mean over samples of ACES(hdr * exposure),
// samples summed in order (geodesic_kernel.cu:482-503).
template <class T>
inline V3<T> diff_pixel(const sgx_uniforms& ub, const DiffParams& dp, const DiffOpts& o, std::uint32_t gx,
                        std::uint32_t gy) {
    const std::uint32_t spp = ub.supersample < 1u ? 1u : (ub.supersample > 1024u ? 1024u : ub.supersample);
    const T exposure = T(ub.exposure);
    V3<T> ldr = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    for (std::uint32_t s = 0; s < spp; ++s) {
        const DiffOut<T> t = diff_trace<T>(ub, dp, o, gx, gy, s);
        ldr = vadd(ldr, aces(vmul(t.hdr, exposure)));
    }
    return vmul(ldr, OLIT(1.0) / T(float(spp)));
}

// ---------------------------------------------------------------------------
// Forward-mode dual numbers (a double and its derivatives with respect to the
// four parameters) and their scalar traits: evaluating the form on Dual4
// yields d(image)/d(spin, incl, r_in, t_scale) of this very code, an FP64
// gradient independent of the GPU's adjoint sweep.
// ---------------------------------------------------------------------------
struct Dual4 {
    double v;
    double d[4];
    Dual4() = default;
    Dual4(double x) : v(x), d{0.0, 0.0, 0.0, 0.0} {}
    static Dual4 var(double x, int k) {
        Dual4 r(x);
        r.d[k] = 1.0;
        return r;
    }
    explicit operator double() const { return v; }
};
inline Dual4 operator+(const Dual4& a, const Dual4& b) {
    Dual4 r(a.v + b.v);
    for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
inline Dual4 operator-(const Dual4& a, const Dual4& b) {
    Dual4 r(a.v - b.v);
    for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
inline Dual4 operator-(const Dual4& a) {
    Dual4 r(-a.v);
    for (int i = 0; i < 4; ++i) r.d[i] = -a.d[i];
    return r;
}
inline Dual4 operator*(const Dual4& a, const Dual4& b) {
    Dual4 r(a.v * b.v);
    for (int i = 0; i < 4; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
inline Dual4 operator/(const Dual4& a, const Dual4& b) {
    Dual4 r(a.v / b.v);
    for (int i = 0; i < 4; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
    return r;
}
inline bool operator<(const Dual4& a, const Dual4& b) { return a.v < b.v; }
inline bool operator>(const Dual4& a, const Dual4& b) { return a.v > b.v; }
inline bool operator<=(const Dual4& a, const Dual4& b) { return a.v <= b.v; }
inline bool operator>=(const Dual4& a, const Dual4& b) { return a.v >= b.v; }
inline Dual4 dchain(const Dual4& x, double f, double df) {
    Dual4 r(f);
    for (int i = 0; i < 4; ++i) r.d[i] = df * x.d[i];
    return r;
}
template <> struct M<Dual4> {
    using D = Dual4;
    static D sqrt(const D& x) {
        const double s = std::sqrt(x.v);
        return dchain(x, s, s > 0.0 ? 0.5 / s : 0.0);
    }
    static D exp(const D& x) {
        const double e = std::exp(x.v);
        return dchain(x, e, e);
    }
    static D sin(const D& x) { return dchain(x, std::sin(x.v), std::cos(x.v)); }
    static D cos(const D& x) { return dchain(x, std::cos(x.v), -std::sin(x.v)); }
    static D acos(const D& x) {
        const double q = 1.0 - x.v * x.v;
        return dchain(x, std::acos(x.v), q > 0.0 ? -1.0 / std::sqrt(q) : 0.0);
    }
    static D log(const D& x) { return dchain(x, std::log(x.v), 1.0 / x.v); }
    // x^y: d = y x^(y-1) dx + x^y log(x) dy
    static D pow(const D& x, const D& y) {
        const double p = std::pow(x.v, y.v);
        D r(p);
        for (int i = 0; i < 4; ++i)
            r.d[i] = (x.v != 0.0 ? y.v * p / x.v : 0.0) * x.d[i] + (x.v > 0.0 ? p * std::log(x.v) : 0.0) * y.d[i];
        return r;
    }
    static D fmin(const D& a, const D& b) { return b.v < a.v ? b : a; }
    static D fmax(const D& a, const D& b) { return b.v > a.v ? b : a; }
    static bool isfinite(const D& x) { return std::isfinite(x.v); }
    static D lit(float, double d) { return D(d); }
};

// Pixel (gx, gy): its LDR mean and d(LDR)/d(spin, incl, r_in, t_scale).
inline void diff_pixel_grad(const sgx_uniforms& ub, const DiffParams& dp, const DiffOpts& o, std::uint32_t gx,
                            std::uint32_t gy, double ldr[3], double dldr[3][4]) {
    const std::uint32_t spp = ub.supersample < 1u ? 1u : (ub.supersample > 1024u ? 1024u : ub.supersample);
    using T = Dual4;
    const T exposure = T(double(ub.exposure));
    V3<T> acc = v3(T(0.0), T(0.0), T(0.0));
    for (std::uint32_t s = 0; s < spp; ++s) {
        const DiffOut<T> t = diff_trace_p<T>(ub, T::var(dp.spin, 0), T::var(dp.incl, 1), T::var(dp.r_in, 2),
                                             T::var(dp.t_scale, 3), o, gx, gy, s);
        acc = vadd(acc, aces(vmul(t.hdr, exposure)));
    }
    const V3<T> mean = vmul(acc, T(1.0) / T(double(float(spp))));
    const T c[3] = {mean.x, mean.y, mean.z};
    for (int k = 0; k < 3; ++k) {
        ldr[k] = c[k].v;
        for (int q = 0; q < 4; ++q) dldr[k][q] = c[k].d[q];
    }
}

}  // namespace oracle
