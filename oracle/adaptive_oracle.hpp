// oracle/adaptive_oracle.hpp
//
// TEST INFRASTRUCTURE — CPU oracle of the error-controlled Kerr integrator.
// Only tests/, the smoke check and bench.py's CPU-baseline leg use it.
//
// The reference integrates every ray with fixed-step RK4
// (shared_shader/kerr_hamilton.h:165-178) and ships no adaptive driver (the
// note at core/include/physics/integrator.hpp:45-46 promises one; the only
// adaptive policy is the radius-proportional adaptive_h of
// shared_shader/geodesic_math.h:91-96).  This file is the specification of the
// adaptive form the GPU kernels implement, operation for operation:
//
//   * the reference's Hamiltonian right-hand side (kerr_rhs_sc in
//     geodesic_oracle.hpp) and the classical RK4 stages, with theta carried
//     as the pair (sin theta, cos theta): the state is (r, s, c, phi, p_r,
//     p_theta) and the theta equation becomes ds = c dtheta, dc = -s dtheta
//     (dtheta = p_theta / Sigma), so no stage evaluates a sine or cosine;
//     after each accepted step the pair is brought back to the unit circle by
//     one Newton step of 1/sqrt(x) at x = 1, n = 3/2 - (s^2 + c^2)/2;
//   * a fifth, first-same-as-last stage k5 = f(y_{n+1}) giving the embedded
//     third-order solution with weights (1/6, 1/3, 1/3, 0, 1/6); the local
//     error estimate is (h/6)(k4 - k5), free on accepted steps because k5 is
//     the next step's k1 (a rejected attempt costs the same four evaluations);
//   * the max-norm over (r, s, c, phi, p_r, p_theta) of that estimate scaled
//     by tol * (1 + max(|y|, |y_new|)); accept when <= 1;
//   * the step update h *= clamp(0.85 / sqrt(sqrt(err)), 0.2, 4) and the ceiling
//     h <= h_max_frac * r, written with IEEE sqrt and division (the GPU's FP32
//     path evaluates the same factor as 0.85 * 2^(-log2(err)/4) on its
//     special-function unit, so its step sizes differ in the last bits);
//   * early capture: a ray with Q >= 0 that is inside both its spherical
//     photon orbit radius r_c(xi) less 0.05 M and the disc's inner edge while
//     moving inward ends as captured.  A photon from outside that reaches
//     r < r_c(xi) has eta > eta_c(xi) (for eta < eta_c the two radial turning
//     points bracket r_c and the outer one stops it; Teo 2003), so no turning
//     point is left outside the horizon, and inside r_in it can no longer
//     reach the disc: the reference's 1.02 r_+ cut would end it with the same
//     (black) result, after the smallest steps of its path;
//   * equatorial crossings: a sign change of cos(theta) with sin(theta) > 0
//     (the reference's theta = pi/2 crossing for theta in (0, pi)), located on
//     the cubic Hermite interpolant of cos(theta) over the accepted step
//     (values and derivatives at both ends, three Newton steps), so long steps
//     keep the crossing radius to fourth order; an escaped ray's sky
//     direction is (s cos phi, s sin phi, c);
//   * precision forms: FP32 (T = float); FP64 (T = double); and the mixed form
//     (T = float with the constants of motion E, L_z, Q and the initial momenta
//     computed in double from the camera ray, and — for a ray within `zone` M
//     of its spherical photon orbit or of the outer horizon — the error norm
//     and step update evaluated in double).
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

// Options block shared (by layout) with tests/ and bench.py.
struct AdaptiveOpts {
    float tol;            // relative/absolute tolerance (1e-6 in the configs)
    float h_init_frac;    // first step = h_init_frac * r_cam
    float h_max_frac;     // step ceiling = h_max_frac * r
    float zone;           // mixed form: FP64 control band half-width in M (0.05)
    std::uint32_t max_steps;  // attempt budget (accepted + rejected); 0 -> the uniforms' max_steps
    std::uint32_t mixed;      // 1: the mixed precision form (T = float only)
    std::uint32_t no_early_capture;  // 1: only the reference's horizon cut ends a captured ray (tests)
    std::uint32_t no_projection;     // 1: leave p_theta as integrated (no projection onto Q)
};

// Per-ray diagnostics for the precision comparison.
struct RayDiag {
    double E, L, Q0;      // constants at launch (double)
    double Q_end;         // Carter constant of the last state (double)
    double H2_end;        // 2H at the last state (double)
    double norm_Q;        // |Q0| + L^2 + a^2 E^2
    std::uint32_t accepted, rejected, zone_steps, pad;
};

// Radius of the unstable spherical photon orbit whose xi = L/E equals the
// ray's (Bardeen 1973; Teo 2003: xi(r) = [r^2 (3M - r) - a^2 (r + M)] / [a (r - M)]),
// by 12 bisections in T inside [r_ph,prograde, r_ph,retrograde]; 3M for a = 0;
// NaN when xi is outside the photon region's range.
template <class T> inline T photon_orbit_radius(T a, T Mm, T xi) {
    if (!(a > OLIT(1e-7)) && !(a < OLIT(-1e-7))) return OLIT(3.0) * Mm;
    // sign of xi(r) - xi, xi(r) = (r^2 (3M - r) - a^2 (r + M)) / (a (r - M)), without
    // the division by a (r - M) (> 0 for a > 0, r > M; the sign flips for a < 0)
    const T sg = a > OLIT(0.0) ? OLIT(1.0) : OLIT(-1.0);
    auto g = [&](T r) { return sg * ((r * r * (OLIT(3.0) * Mm - r) - a * a * (r + Mm)) - xi * a * (r - Mm)); };
    T lo = OLIT(2.0) * Mm * (OLIT(1.0) + M<T>::cos(OLIT(2.0) / OLIT(3.0) * M<T>::acos(-a / Mm)));
    T hi = OLIT(2.0) * Mm * (OLIT(1.0) + M<T>::cos(OLIT(2.0) / OLIT(3.0) * M<T>::acos(a / Mm)));
    const T flo = g(lo), fhi = g(hi);
    if (!(flo * fhi <= OLIT(0.0))) return T(NAN);
    const bool lo_neg = flo <= OLIT(0.0);
    // 12 halvings of [r_pro, r_ret] (< 3M): r_c to 1e-3 M, ample for a 0.05 M band
    for (int i = 0; i < 12; ++i) {
        const T mid = OLIT(0.5) * (lo + hi);
        if ((g(mid) <= OLIT(0.0)) == lo_neg) lo = mid;
        else hi = mid;
    }
    return OLIT(0.5) * (lo + hi);
}

inline double carter_Q(double theta, double p_theta, double E, double L, double a) {
    const double ct = std::cos(theta), st = std::sin(theta);
    const double s2 = std::fmax(st * st, 1e-300);
    return p_theta * p_theta + ct * ct * (L * L / s2 - a * a * E * E);
}

template <class T> inline T abs_(T x) { return x < OLIT(0.0) ? -x : x; }

// p_theta put back onto the ray's Carter constant after an accepted step
// (a projection method, Hairer, Lubich & Wanner, Geometric Numerical
// Integration, IV.4): |p_theta| = sqrt(Theta), Theta = Q - c^2 (L^2 / s^2 -
// a^2 E^2) with s^2 guarded at 1e-10 as in the right-hand side, the sign of
// p_theta kept (copysign); p_theta = +-0 where truncation has carried the
// state past a turning point (Theta < 0).  Q and L are exact constants of
// the flow, so this removes the integrator's drift off the level set Q = Q0
// without touching r, theta, phi or p_r.
template <class T> inline T project_p_theta(T pth, T s, T c, T Q, T L2, T a2E2) {
    const T s2 = s * s;
    const T safe = s2 < OLIT(1e-10) ? OLIT(1e-10) : s2;
    const T th = Q - c * c * (L2 / safe - a2E2);
    const T m = th > OLIT(0.0) ? M<T>::sqrt(th) : OLIT(0.0);
    return M<T>::copysign(m, pth);
}

// State of the error-controlled form: theta carried as (sin theta, cos theta).
template <class T> struct SCState {
    T r, s, c, phi, p_r, p_theta;
};

template <class T> inline SCState<T> sc_add_scaled(const SCState<T>& y, const SCState<T>& k, T f) {
    return {y.r + k.r * f, y.s + k.s * f, y.c + k.c * f, y.phi + k.phi * f, y.p_r + k.p_r * f, y.p_theta + k.p_theta * f};
}

template <class T> inline SCState<T> sc_rhs(const SCState<T>& y, const KConst<T>& c) {
    const KState<T> k{OLIT(0.0), y.r, OLIT(0.0), y.phi, y.p_r, y.p_theta};
    const KState<T> d = kerr_rhs_sc<T, false>(k, y.s, y.c, c);
    return {d.r, y.c * d.theta, -(y.s * d.theta), d.phi, d.p_r, d.p_theta};
}

template <class T> struct Attempt {
    SCState<T> y4, k4, k5;
    T h6;
};

// RK4 stages from y with k1 = f(y) already known, and the FSAL stage.
template <class T> inline Attempt<T> rk4_attempt(const SCState<T>& y, const SCState<T>& k1, T h, const KConst<T>& c) {
    Attempt<T> a;
    const SCState<T> k2 = sc_rhs(sc_add_scaled(y, k1, OLIT(0.5) * h), c);
    const SCState<T> k3 = sc_rhs(sc_add_scaled(y, k2, OLIT(0.5) * h), c);
    a.k4 = sc_rhs(sc_add_scaled(y, k3, h), c);
    a.h6 = h * OLIT(0.16666666666666666);  // h/6 as a product (no division per attempt)
    a.y4.r = rk4_combine(y.r, k1.r, k2.r, k3.r, a.k4.r, a.h6);
    a.y4.s = rk4_combine(y.s, k1.s, k2.s, k3.s, a.k4.s, a.h6);
    a.y4.c = rk4_combine(y.c, k1.c, k2.c, k3.c, a.k4.c, a.h6);
    a.y4.phi = rk4_combine(y.phi, k1.phi, k2.phi, k3.phi, a.k4.phi, a.h6);
    a.y4.p_r = rk4_combine(y.p_r, k1.p_r, k2.p_r, k3.p_r, a.k4.p_r, a.h6);
    a.y4.p_theta = rk4_combine(y.p_theta, k1.p_theta, k2.p_theta, k3.p_theta, a.k4.p_theta, a.h6);
    a.k5 = sc_rhs(a.y4, c);
    return a;
}

// Scaled max-norm of the embedded estimate, evaluated in C (T or double).
template <class C, class T>
inline C error_norm(const SCState<T>& y, const Attempt<T>& a, float tol_f) {
    const C tol = C(tol_f);
    const C h6 = C(a.h6);
    auto one = [&](T yv, T y4v, T k4v, T k5v) {
        const C ya = abs_(C(yv)), yb = abs_(C(y4v));
        const C sc = tol * (C(1.0f) + (ya > yb ? ya : yb));
        return abs_(h6 * (C(k4v) - C(k5v))) / sc;
    };
    C e = one(y.r, a.y4.r, a.k4.r, a.k5.r);
    C t;
    t = one(y.s, a.y4.s, a.k4.s, a.k5.s); e = t > e ? t : e;
    t = one(y.c, a.y4.c, a.k4.c, a.k5.c); e = t > e ? t : e;
    t = one(y.phi, a.y4.phi, a.k4.phi, a.k5.phi); e = t > e ? t : e;
    t = one(y.p_r, a.y4.p_r, a.k4.p_r, a.k5.p_r); e = t > e ? t : e;
    t = one(y.p_theta, a.y4.p_theta, a.k4.p_theta, a.k5.p_theta); e = t > e ? t : e;
    if (!(e <= C(1e30f))) e = C(1e30f);  // NaN or overflow: reject hard
    return e;
}

// h *= clamp(0.85 / err^(1/4), 0.2, 4), computed in C.  Safety factor 0.85:
// on the 4K Kerr a = 0.94 scene 0.9 rejects 14 % of the attempts; 0.85 takes
// 10 % fewer attempts per ray (40.4 against 45.0) for the same error against
// an FP64 solution at tolerance 1e-10 (0.8 and 0.75 take more).
template <class C> inline C step_factor(C e) {
    if (e <= C(1e-30f)) return C(4.0f);
    C f = C(0.85f) / std::sqrt(std::sqrt(e));
    f = f < C(0.2f) ? C(0.2f) : f;
    f = f > C(4.0f) ? C(4.0f) : f;
    return f;
}
template <> inline Counted step_factor<Counted>(Counted e) {
    if (e <= Counted(1e-30f)) return Counted(4.0f);
    Counted f = Counted(0.85f) / M<Counted>::sqrt(M<Counted>::sqrt(e));
    f = f < Counted(0.2f) ? Counted(0.2f) : f;
    f = f > Counted(4.0f) ? Counted(4.0f) : f;
    return f;
}

// Cubic Hermite interpolant on [0, h] in the unit variable s, and its s-derivative.
template <class T> inline T hermite(T y0, T y1, T d0, T d1, T h, T s) {
    const T s2 = s * s, s3 = s2 * s;
    const T h00 = OLIT(2.0) * s3 - OLIT(3.0) * s2 + OLIT(1.0);
    const T h10 = s3 - OLIT(2.0) * s2 + s;
    const T h01 = OLIT(3.0) * s2 - OLIT(2.0) * s3;
    const T h11 = s3 - s2;
    return h00 * y0 + h10 * h * d0 + h01 * y1 + h11 * h * d1;
}
template <class T> inline T hermite_d(T y0, T y1, T d0, T d1, T h, T s) {
    const T s2 = s * s;
    const T h00 = OLIT(6.0) * s2 - OLIT(6.0) * s;
    const T h10 = OLIT(3.0) * s2 - OLIT(4.0) * s + OLIT(1.0);
    const T h01 = OLIT(6.0) * s - OLIT(6.0) * s2;
    const T h11 = OLIT(3.0) * s2 - OLIT(2.0) * s;
    return h00 * y0 + h10 * h * d0 + h01 * y1 + h11 * h * d1;
}

// cos(theta) = 0 inside an accepted step: Newton on the Hermite interpolant
// from the linear estimate, kept inside [0, 1].
template <class T>
inline T crossing_fraction(T c0, T c1, T d0, T d1, T h) {
    T s = c0 / (c0 - c1);
    for (int it = 0; it < 3; ++it) {
        const T f = hermite(c0, c1, d0, d1, h, s);
        const T fp = hermite_d(c0, c1, d0, d1, h, s);
        if (!(abs_(fp) > OLIT(1e-30))) break;
        T sn = s - f / fp;
        sn = sn < OLIT(0.0) ? OLIT(0.0) : (sn > OLIT(1.0) ? OLIT(1.0) : sn);
        s = sn;
    }
    return s;
}

// Constants of motion and initial momenta in double from the camera ray
// (the mixed form's FP64 initialisation; formulas of geodesic_kernel.cu:310-344).
template <class T>
inline bool kerr_init_double(const CamRay<T>& cam, const Params<T>& u, double& E, double& L, double& Q, double& pr,
                             double& pth) {
    const double Mm = double(float(u.mass_M)), a = double(float(u.spin_a));
    const double r = double(float(cam.cam_r));
    const double ct = double(float(M<T>::cos(cam.cam_theta))), st = double(float(cam.sin_th));
    const double Sigma = r * r + a * a * ct * ct, Delta = r * r - 2.0 * Mm * r + a * a, s2 = st * st;
    const double g_tt = -(1.0 - 2.0 * Mm * r / Sigma);
    const double g_tp = -2.0 * Mm * r * a * s2 / Sigma;
    const double g_rr = Sigma / Delta, g_thth = Sigma;
    const double g_pp = s2 * ((r * r + a * a) * (r * r + a * a) - a * a * Delta * s2) / Sigma;
    const double ur = double(float(cam.ur)), uth = double(float(cam.utheta)), uph = double(float(cam.uphi));
    const double B = 2.0 * g_tp * uph;
    const double C = g_rr * ur * ur + g_thth * uth * uth + g_pp * uph * uph;
    const double disc = B * B - 4.0 * g_tt * C;
    if (disc < 0.0) return false;
    const double ut = (-B - std::sqrt(disc)) / (2.0 * g_tt);
    E = -(g_tt * ut + g_tp * uph);
    L = g_tp * ut + g_pp * uph;
    pth = g_thth * uth;
    pr = g_rr * ur;
    Q = pth * pth + ct * ct * (L * L / std::fmax(s2, 1e-6) - a * a * E * E);
    return true;
}

template <class T>
inline TraceOut<T> trace_kerr_adaptive(const CamRay<T>& cam, const Params<T>& u, const AdaptiveOpts& o,
                                       RayDiag* diag) {
    constexpr bool is_double = std::is_same<T, double>::value;
    const V3<T> black = v3(OLIT(0.0), OLIT(0.0), OLIT(0.0));
    const bool mixed = (o.mixed != 0u) && !is_double;
    KState<T> y0;
    KConst<T> c;
    if (!kerr_init(cam, u, y0, c)) return {black, 0u, TERM_NO_ROOT};
    double Ed = double(c.E), Ld = double(c.L), Qd = double(c.Q), prd = 0, pthd = 0;
    if (mixed) {
        if (!kerr_init_double(cam, u, Ed, Ld, Qd, prd, pthd)) return {black, 0u, TERM_NO_ROOT};
        c.E = T(float(Ed));
        c.L = T(float(Ld));
        y0.p_r = T(float(prd));
        y0.p_theta = T(float(pthd));
    }
    SCState<T> y{y0.r, cam.sin_th, M<T>::cos(cam.cam_theta), y0.phi, y0.p_r, y0.p_theta};
    const std::uint32_t max_steps = o.max_steps != 0u ? o.max_steps : u.max_steps;
    const T hcut = kerr_horizon_cut(u.mass_M, u.spin_a);
    const T r_plus = u.mass_M + M<T>::sqrt(M<T>::fmax(u.mass_M * u.mass_M - u.spin_a * u.spin_a, OLIT(0.0)));
    const T r_c = photon_orbit_radius(u.spin_a, u.mass_M, c.L / c.E);
    const T zone = T(o.zone);
    // early capture radius: min(r_c - 0.05 M, r_in) for Q >= 0, else none
    T r_cap = OLIT(0.0);
    if (o.no_early_capture == 0u && c.Q >= OLIT(0.0) && M<T>::isfinite(r_c)) {
        r_cap = r_c - OLIT(0.05) * u.mass_M;
        r_cap = r_cap < u.r_in ? r_cap : u.r_in;
    }

    // the projection's constants: Q in T (the mixed form's from its FP64 value)
    const T Qp = mixed ? T(float(Qd)) : c.Q;
    const T L2 = c.L * c.L, a2E2 = (u.spin_a * c.E) * (u.spin_a * c.E);
    T h = T(o.h_init_frac) * y.r;
    SCState<T> k1 = sc_rhs(y, c);
    std::uint32_t accepted = 0, rejected = 0, zone_steps = 0, steps = 0;
    TraceOut<T> out{black, max_steps, TERM_BUDGET};
    for (;;) {
        if (steps >= max_steps) {
            out = {black, steps, TERM_BUDGET};
            break;
        }
        if (!M<T>::isfinite(y.r) || y.r < hcut || (y.r < r_cap && y.p_r < OLIT(0.0))) {
            out = {black, steps, TERM_HORIZON};
            break;
        }
        if (y.r > u.escape_r) {
            out = {(u.flags & SGX_FLAG_STARFIELD_ON) ? sky_color_sc(y.s, y.c, y.phi) : black, steps, TERM_ESCAPE};
            break;
        }
        const T hmax = T(o.h_max_frac) * y.r;
        h = h > hmax ? hmax : h;
        const Attempt<T> at = rk4_attempt(y, k1, h, c);
        ++steps;
        const bool in_zone = mixed && ((abs_(y.r - r_c) < zone) || (y.r - r_plus < zone));
        bool accept;
        if (in_zone) {
            ++zone_steps;
            // the error measured in FP64, the step factor (a heuristic) in T
            const double e = error_norm<double>(y, at, o.tol);
            accept = e <= 1.0;
            h = h * step_factor<T>(T(float(e)));
        } else {
            const T e = error_norm<T>(y, at, o.tol);
            accept = e <= OLIT(1.0);
            h = h * step_factor<T>(e);
        }
        if (!accept) {
            ++rejected;
            continue;
        }
        ++accepted;
        if ((u.flags & SGX_FLAG_DISC_ON) && (y.c * at.y4.c < OLIT(0.0)) && at.y4.s > OLIT(0.0)) {
            const T hs = at.h6 * OLIT(6.0);
            const T sfr = crossing_fraction(y.c, at.y4.c, k1.c, at.k5.c, hs);
            const T r_cross = hermite(y.r, at.y4.r, k1.r, at.k5.r, hs, sfr);
            if (in_annulus(r_cross, u.r_in, u.r_out)) {
                const T T_local = disc_temperature(r_cross, u.r_in, u.peak_T);
                if (T_local > OLIT(0.0)) {
                    const T phi_cross = hermite(y.phi, at.y4.phi, k1.phi, at.k5.phi, hs, sfr);
                    out = {kerr_disc_colour(u, c, cam.cam_r, r_cross, phi_cross, T_local), steps, TERM_DISC};
                } else {
                    out = {black, steps, TERM_DISC_COLD};
                }
                y = at.y4;
                break;
            }
        }
        y = at.y4;
        const T n = OLIT(1.5) - OLIT(0.5) * (y.s * y.s + y.c * y.c);
        y.s = y.s * n;
        y.c = y.c * n;
        if (o.no_projection == 0u) y.p_theta = project_p_theta(y.p_theta, y.s, y.c, Qp, L2, a2E2);
        k1 = at.k5;
    }
    if (diag != nullptr) {
        const double a = double(float(u.spin_a));
        diag->E = Ed;
        diag->L = Ld;
        diag->Q0 = Qd;
        const double sv = is_double ? double(y.s) : double(float(y.s));
        const double cv = is_double ? double(y.c) : double(float(y.c));
        const double th = std::atan2(sv, cv);
        const double pth = is_double ? double(y.p_theta) : double(float(y.p_theta));
        const double rr = is_double ? double(y.r) : double(float(y.r));
        const double pr = is_double ? double(y.p_r) : double(float(y.p_r));
        diag->Q_end = carter_Q(th, pth, Ed, Ld, a);
        const KConst<double> cq{Ed, Ld, Qd, a, double(float(u.mass_M))};
        diag->H2_end = kerr_two_H(rr, th, pr, pth, cq);
        diag->norm_Q = std::fabs(Qd) + Ld * Ld + a * a * Ed * Ed;
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
