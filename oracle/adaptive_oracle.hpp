// oracle/adaptive_oracle.hpp
//
// TEST INFRASTRUCTURE — CPU oracle of the error-controlled Kerr integrator.
// Only tests/, the smoke check and bench.py's CPU-baseline leg use it.
//
// The reference integrates every ray with fixed-step RK4
// (shared_shader/kerr_hamilton.h:165-178) and ships no adaptive driver (the
// note at core/include/physics/integrator.hpp:45-46 promises one; the only
// adaptive policy is the radius-proportional adaptive_h of
// shared_shader/geodesic_math.h:91-96).  This file states the adaptive form
// that the GPU kernels implement:
//
//   * the reference's Hamiltonian right-hand side (kerr_rhs in
//     geodesic_oracle.hpp) and the classical RK4 stages;
//   * a fifth, first-same-as-last stage k5 = f(y_{n+1}) giving the embedded
//     third-order solution with weights (1/6, 1/3, 1/3, 0, 1/6); the error
//     estimate is (h/6)(k4 - k5), free on accepted steps because k5 is the
//     next step's k1;
//   * a max-norm over (r, theta, phi, p_r, p_theta) scaled by
//     tol * (1 + max(|y|, |y_new|)), and the step update
//     h *= clamp(0.9 * err^(-1/4), 0.2, 4);
//   * equatorial crossings located on the cubic Hermite interpolant of the
//     step (values and derivatives at both ends), so long steps keep the
//     crossing radius to fourth order;
//   * precision forms: T = float bulk with E, L_z, Q computed in double and
//     rounded, and — for rays within `zone` M of their spherical photon orbit
//     or of the horizon — the step and its error control evaluated in double
//     (the mixed form); T = double throughout (the FP64 form).
//
// Shading (disc colour, starfield, ACES) is the reference's, unchanged; the
// disc band pattern takes phi at the interpolated crossing instead of the
// reference's post-step phi (geodesic_kernel.cu:389), because an adaptive step
// can be long.

#pragma once

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "geodesic_oracle.hpp"

namespace oracle {

// Options block shared (by layout) with the CUDA library's sgx_adaptive_opts.
struct AdaptiveOpts {
    float tol;            // relative/absolute tolerance (1e-6 in the configs)
    float h_init_frac;    // first step = h_init_frac * r_cam
    float h_max_frac;     // step ceiling = h_max_frac * r
    float zone;           // FP64 control zone half-width in M (0.05); <0 disables
    std::uint32_t max_steps;  // attempt budget (accepted + rejected)
    std::uint32_t mixed;      // 1: FP64 constants + FP64 zone control; 0: plain T
    std::uint32_t kahan;      // 1: compensated state update
    std::uint32_t pad;
};

// Per-ray diagnostics for the precision comparison.
struct RayDiag {
    double E, L, Q0;      // constants at launch (double)
    double Q_end;         // Carter constant at the last state (double, from that state)
    double H2_end;        // 2H at the last state (double)
    double norm_Q;        // |Q0| + L^2 + a^2 E^2
    std::uint32_t accepted, rejected, zone_steps, pad;
};

// Spherical photon orbit radius for the ray's xi = L/E (Bardeen 1973 /
// Teo 2003: xi(r) = [r^2 (3M - r) - a^2 (r + M)] / [a (r - M)]), found by
// bisection inside [r_ph,pro, r_ph,retro]; 3M for a = 0.  Returns NaN when
// xi lies outside the photon region's range.
inline double photon_orbit_radius(double a, double Mm, double xi) {
    if (std::fabs(a) < 1e-12) return 3.0 * Mm;
    auto xi_of = [&](double r) { return (r * r * (3.0 * Mm - r) - a * a * (r + Mm)) / (a * (r - Mm)); };
    const double r_pro = 2.0 * Mm * (1.0 + std::cos((2.0 / 3.0) * std::acos(-a / Mm)));
    const double r_ret = 2.0 * Mm * (1.0 + std::cos((2.0 / 3.0) * std::acos(a / Mm)));
    double lo = r_pro, hi = r_ret;
    double flo = xi_of(lo) - xi, fhi = xi_of(hi) - xi;
    if (!(flo * fhi <= 0.0)) return NAN;
    for (int i = 0; i < 60; ++i) {
        const double mid = 0.5 * (lo + hi);
        const double fm = xi_of(mid) - xi;
        if ((fm <= 0.0) == (flo <= 0.0)) {
            lo = mid;
            flo = fm;
        } else {
            hi = mid;
        }
    }
    return 0.5 * (lo + hi);
}

inline double carter_Q(double theta, double p_theta, double E, double L, double a) {
    const double ct = std::cos(theta), st = std::sin(theta);
    const double s2 = std::fmax(st * st, 1e-300);
    return p_theta * p_theta + ct * ct * (L * L / s2 - a * a * E * E);
}

template <class T> struct AState {
    KState<T> y;
    KState<T> comp;  // Kahan compensation (zero when unused)
};

template <class T> inline T abs_(T x) { return x < OLIT(0.0) ? -x : x; }

// One RK4 attempt with FSAL error estimate.  Returns the scaled error norm;
// writes the candidate state and its derivative.
template <class T>
inline T rk4_attempt(const KState<T>& y, const KState<T>& k1, T h, const KConst<T>& c, T tol, KState<T>& y4,
                     KState<T>& k5, const KState<T>* comp, KState<T>* comp_out) {
    const KState<T> k2 = kerr_rhs(k_add_scaled(y, k1, OLIT(0.5) * h), c);
    const KState<T> k3 = kerr_rhs(k_add_scaled(y, k2, OLIT(0.5) * h), c);
    const KState<T> k4 = kerr_rhs(k_add_scaled(y, k3, h), c);
    const T h6 = h / OLIT(6.0);
    auto inc = [&](T a1, T a2, T a3, T a4) { return ((a1 + a2 * OLIT(2.0)) + (a3 * OLIT(2.0) + a4)) * h6; };
    KState<T> d{inc(k1.t, k2.t, k3.t, k4.t), inc(k1.r, k2.r, k3.r, k4.r),
                inc(k1.theta, k2.theta, k3.theta, k4.theta), inc(k1.phi, k2.phi, k3.phi, k4.phi),
                inc(k1.p_r, k2.p_r, k3.p_r, k4.p_r), inc(k1.p_theta, k2.p_theta, k3.p_theta, k4.p_theta)};
    if (comp != nullptr) {
        // Kahan: y4 = y + (d - comp); comp_out = (y4 - y) - (d - comp)
        auto ks = [](T yv, T dv, T cv, T& cout) {
            const T dd = dv - cv;
            const T s = yv + dd;
            cout = (s - yv) - dd;
            return s;
        };
        y4.t = ks(y.t, d.t, comp->t, comp_out->t);
        y4.r = ks(y.r, d.r, comp->r, comp_out->r);
        y4.theta = ks(y.theta, d.theta, comp->theta, comp_out->theta);
        y4.phi = ks(y.phi, d.phi, comp->phi, comp_out->phi);
        y4.p_r = ks(y.p_r, d.p_r, comp->p_r, comp_out->p_r);
        y4.p_theta = ks(y.p_theta, d.p_theta, comp->p_theta, comp_out->p_theta);
    } else {
        y4 = {y.t + d.t, y.r + d.r, y.theta + d.theta, y.phi + d.phi, y.p_r + d.p_r, y.p_theta + d.p_theta};
    }
    k5 = kerr_rhs(y4, c);
    auto comp_err = [&](T yv, T y4v, T k4v, T k5v) {
        const T sc = tol * (OLIT(1.0) + M<T>::fmax(abs_(yv), abs_(y4v)));
        return abs_(h6 * (k4v - k5v)) / sc;
    };
    T e = comp_err(y.r, y4.r, k4.r, k5.r);
    e = M<T>::fmax(e, comp_err(y.theta, y4.theta, k4.theta, k5.theta));
    e = M<T>::fmax(e, comp_err(y.phi, y4.phi, k4.phi, k5.phi));
    e = M<T>::fmax(e, comp_err(y.p_r, y4.p_r, k4.p_r, k5.p_r));
    e = M<T>::fmax(e, comp_err(y.p_theta, y4.p_theta, k4.p_theta, k5.p_theta));
    if (!M<T>::isfinite(e)) e = OLIT(1e30);
    return e;
}

// Step-size factor from an error norm: 0.9 err^(-1/4) clamped to [0.2, 4].
template <class T> inline T step_factor(T e) {
    if (e <= OLIT(1e-30)) return OLIT(4.0);
    T f = OLIT(0.9) * M<T>::pow(e, OLIT(-0.25));
    f = f < OLIT(0.2) ? OLIT(0.2) : f;
    f = f > OLIT(4.0) ? OLIT(4.0) : f;
    return f;
}

// Cubic Hermite interpolant on [0, h] in the unit variable s.
template <class T> inline T hermite(T y0, T y1, T d0, T d1, T h, T s) {
    const T s2 = s * s, s3 = s2 * s;
    const T h00 = OLIT(2.0) * s3 - OLIT(3.0) * s2 + OLIT(1.0);
    const T h10 = s3 - OLIT(2.0) * s2 + s;
    const T h01 = OLIT(-2.0) * s3 + OLIT(3.0) * s2;
    const T h11 = s3 - s2;
    return h00 * y0 + h10 * h * d0 + h01 * y1 + h11 * h * d1;
}
template <class T> inline T hermite_d(T y0, T y1, T d0, T d1, T h, T s) {
    const T s2 = s * s;
    const T h00 = OLIT(6.0) * s2 - OLIT(6.0) * s;
    const T h10 = OLIT(3.0) * s2 - OLIT(4.0) * s + OLIT(1.0);
    const T h01 = OLIT(-6.0) * s2 + OLIT(6.0) * s;
    const T h11 = OLIT(3.0) * s2 - OLIT(2.0) * s;
    return h00 * y0 + h10 * h * d0 + h01 * y1 + h11 * h * d1;
}

// Crossing of theta = pi/2 inside an accepted step: Newton on the Hermite
// interpolant from the linear estimate, kept inside [0, 1].
template <class T>
inline T crossing_fraction(const KState<T>& y0, const KState<T>& y1, const KState<T>& d0, const KState<T>& d1,
                           T h) {
    const T mid = OLIT(1.5707963267948966);
    T s = (mid - y0.theta) / (y1.theta - y0.theta);
    for (int it = 0; it < 3; ++it) {
        const T f = hermite(y0.theta, y1.theta, d0.theta, d1.theta, h, s) - mid;
        const T fp = hermite_d(y0.theta, y1.theta, d0.theta, d1.theta, h, s);
        if (!(abs_(fp) > OLIT(1e-30))) break;
        T sn = s - f / fp;
        sn = sn < OLIT(0.0) ? OLIT(0.0) : (sn > OLIT(1.0) ? OLIT(1.0) : sn);
        s = sn;
    }
    return s;
}

template <class T> inline KState<T> to_T(const KState<double>& s) {
    return {T(float(s.t)), T(float(s.r)), T(float(s.theta)), T(float(s.phi)), T(float(s.p_r)), T(float(s.p_theta))};
}

template <class T> inline KState<double> to_d(const KState<T>& s) {
    auto d = [](T v) { return double(float(v)); };
    return {d(s.t), d(s.r), d(s.theta), d(s.phi), d(s.p_r), d(s.p_theta)};
}
template <> inline KState<double> to_d<double>(const KState<double>& s) { return s; }
template <> inline KState<double> to_T<double>(const KState<double>& s) { return s; }

template <class T>
inline TraceOut<T> trace_kerr_adaptive(const CamRay<T>& cam, const Params<T>& u, const AdaptiveOpts& o,
                                       RayDiag* diag) {
    const V3<T> black = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    KState<T> y;
    KConst<T> c;
    if (!kerr_init(cam, u, y, c)) return {black, 0u, TERM_NO_ROOT};

    // Constants of motion in double from the (T) camera ray when asked.
    KConst<double> cd{double(float(c.E)), double(float(c.L)), double(float(c.Q)), double(float(c.a)),
                      double(float(c.M))};
    const bool mixed = (o.mixed != 0u) || std::is_same<T, double>::value;
    if (mixed) {
        const double Mm = double(float(u.mass_M)), a = double(float(u.spin_a));
        const double r = double(float(cam.cam_r)), th = double(float(cam.cam_theta));
        const double st = double(float(cam.sin_th)), ct = std::cos(th);
        const double Sigma = r * r + a * a * ct * ct, Delta = r * r - 2.0 * Mm * r + a * a, s2 = st * st;
        const double g_tt = -(1.0 - 2.0 * Mm * r / Sigma);
        const double g_tp = -2.0 * Mm * r * a * s2 / Sigma;
        const double g_rr = Sigma / Delta, g_thth = Sigma;
        const double g_pp = s2 * ((r * r + a * a) * (r * r + a * a) - a * a * Delta * s2) / Sigma;
        const double ur = double(float(cam.ur)), uth = double(float(cam.utheta)), uph = double(float(cam.uphi));
        const double B = 2.0 * g_tp * uph, C = g_rr * ur * ur + g_thth * uth * uth + g_pp * uph * uph;
        const double disc = B * B - 4.0 * g_tt * C;
        if (disc < 0.0) return {black, 0u, TERM_NO_ROOT};
        // Stable root of A x^2 + B x + C: the reference's branch (-B - sqrt)/(2A).
        const double ut = (-B - std::sqrt(disc)) / (2.0 * g_tt);
        cd.E = -(g_tt * ut + g_tp * uph);
        cd.L = g_tp * ut + g_pp * uph;
        const double pth = g_thth * uth;
        cd.Q = pth * pth + ct * ct * (cd.L * cd.L / std::fmax(s2, 1e-300) - a * a * cd.E * cd.E);
        cd.a = a;
        cd.M = Mm;
        c.E = T(float(cd.E));
        c.L = T(float(cd.L));
        if (std::is_same<T, double>::value) {
            c.E = T(cd.E);
            c.L = T(cd.L);
        }
        y.p_r = std::is_same<T, double>::value ? T(g_rr * ur) : T(float(g_rr * ur));
        y.p_theta = std::is_same<T, double>::value ? T(pth) : T(float(pth));
    }
    const KConst<double> cstep_d{double(float(c.E)), double(float(c.L)), 0.0, double(float(c.a)),
                                 double(float(c.M))};
    const KConst<double> cd_use = std::is_same<T, double>::value ? cd : cstep_d;

    const double r_plus = double(float(u.mass_M)) + std::sqrt(std::fmax(
        double(float(u.mass_M)) * double(float(u.mass_M)) - double(float(u.spin_a)) * double(float(u.spin_a)), 0.0));
    const double r_c = photon_orbit_radius(cd.a == 0.0 ? double(float(u.spin_a)) : cd.a, double(float(u.mass_M)),
                                           cd.L / cd.E);
    const double zone = double(o.zone);

    const T hcut = kerr_horizon_cut(u.mass_M, u.spin_a);
    const T tol = T(o.tol);
    T h = T(o.h_init_frac) * y.r;
    KState<T> k1 = kerr_rhs(y, c);
    KState<T> comp{OLIT(0.0), OLIT(0.0), OLIT(0.0), OLIT(0.0), OLIT(0.0), OLIT(0.0)};
    std::uint32_t accepted = 0, rejected = 0, zone_steps = 0;
    TraceOut<T> out{black, o.max_steps, TERM_BUDGET};
    bool done = false;
    std::uint32_t attempt = 0;
    for (; attempt < o.max_steps && !done; ++attempt) {
        if (!M<T>::isfinite(y.r) || y.r < hcut) {
            out = {black, attempt, TERM_HORIZON};
            done = true;
            break;
        }
        if (y.r > u.escape_r) {
            out = {(u.flags & SGX_FLAG_STARFIELD_ON) ? sky_color(y.theta, y.phi) : black, attempt, TERM_ESCAPE};
            done = true;
            break;
        }
        const T hmax = T(o.h_max_frac) * y.r;
        if (h > hmax) h = hmax;
        const double rr = double(float(y.r));
        const bool in_zone = mixed && zone >= 0.0 && !std::is_same<T, double>::value
                             && ((std::isfinite(r_c) && std::fabs(rr - r_c) < zone) || (rr - r_plus) < zone);
        KState<T> y4, k5, comp_new = comp;
        T e;
        if (in_zone) {
            ++zone_steps;
            KState<double> yd = to_d(y), y4d, k5d, cn{0, 0, 0, 0, 0, 0};
            const KState<double> k1d = kerr_rhs(yd, cd_use);
            const double ed = rk4_attempt<double>(yd, k1d, double(float(h)), cd_use, double(o.tol), y4d, k5d,
                                                  nullptr, &cn);
            e = T(float(ed));
            y4 = to_T<T>(y4d);
            k5 = to_T<T>(k5d);
            comp_new = {OLIT(0.0), OLIT(0.0), OLIT(0.0), OLIT(0.0), OLIT(0.0), OLIT(0.0)};
        } else {
            e = rk4_attempt(y, k1, h, c, tol, y4, k5, o.kahan ? &comp : nullptr, &comp_new);
        }
        if (e <= OLIT(1.0)) {
            ++accepted;
            // Crossing between y and y4.
            const Crossing<T> x = equatorial_crossing(y.theta, y4.theta);
            if ((u.flags & SGX_FLAG_DISC_ON) && x.crossed) {
                const T sfr = crossing_fraction(y, y4, k1, k5, h);
                const T r_cross = hermite(y.r, y4.r, k1.r, k5.r, h, sfr);
                if (in_annulus(r_cross, u.r_in, u.r_out)) {
                    const T T_local = disc_temperature(r_cross, u.r_in, u.peak_T);
                    if (T_local > OLIT(0.0)) {
                        const T phi_cross = hermite(y.phi, y4.phi, k1.phi, k5.phi, h, sfr);
                        out = {kerr_disc_colour(u, c, cam.cam_r, r_cross, phi_cross, T_local), attempt + 1,
                               TERM_DISC};
                    } else {
                        out = {black, attempt + 1, TERM_DISC_COLD};
                    }
                    y = y4;
                    done = true;
                    break;
                }
            }
            y = y4;
            k1 = k5;
            comp = comp_new;
        } else {
            ++rejected;
        }
        h = h * step_factor(e);
    }
    if (!done) out = {black, attempt, TERM_BUDGET};
    if (diag != nullptr) {
        const KState<double> yd = to_d(y);
        diag->E = cd.E;
        diag->L = cd.L;
        diag->Q0 = cd.Q;
        diag->Q_end = carter_Q(yd.theta, yd.p_theta, cd.E, cd.L, cd.a);
        KConst<double> cq = cd;
        diag->H2_end = kerr_two_H(yd.r, yd.theta, yd.p_r, yd.p_theta, cq);
        diag->norm_Q = std::fabs(cd.Q) + cd.L * cd.L + cd.a * cd.a * cd.E * cd.E;
        diag->accepted = accepted;
        diag->rejected = rejected;
        diag->zone_steps = zone_steps;
    }
    return out;
}

template <class T>
inline TraceOut<T> trace_sample_adaptive(std::uint32_t gx, std::uint32_t gy, std::uint32_t s, const Params<T>& u,
                                         const AdaptiveOpts& o, RayDiag* diag) {
    T ox, oy;
    if (u.spp == 1u) {
        ox = OLIT(0.5);
        oy = OLIT(0.5);
    } else {
        ox = halton<T>(s + 1u, 2u);
        oy = halton<T>(s + 1u, 3u);
    }
    const CamRay<T> cam = camera_ray(gx, gy, ox, oy, u);
    if (u.metric == SGX_METRIC_KERR) return trace_kerr_adaptive(cam, u, o, diag);
    // The error-controlled form is Kerr-only (spin 0 included); the
    // Schwarzschild metric keeps the reference's fixed-step integrator.
    return trace_schwarzschild(cam, u);
}

template <class T>
inline V3<T> shade_pixel_adaptive(std::uint32_t gx, std::uint32_t gy, const Params<T>& u, const AdaptiveOpts& o) {
    V3<T> ldr = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    if (u.spp == 1u) {
        const TraceOut<T> t = trace_sample_adaptive(gx, gy, 0u, u, o, nullptr);
        ldr = aces(vmul(t.hdr, u.exposure));
    } else {
        for (std::uint32_t s = 0; s < u.spp; ++s) {
            const TraceOut<T> t = trace_sample_adaptive(gx, gy, s, u, o, nullptr);
            ldr = vadd(ldr, aces(vmul(t.hdr, u.exposure)));
        }
        ldr = vmul(ldr, OLIT(1.0) / T(float(u.spp)));
    }
    return ldr;
}

}  // namespace oracle
