// singularity_gb300/csrc/sgx_diff_impl.cuh
//
// Kernels and launch helpers of the differentiable form and its adjoint,
// shared by sgx_diff.cu (the C ABI and the FP32 instantiations) and
// sgx_diff64.cu (the FP64 instantiations) so the two compile in parallel.
// Everything here has internal linkage; each translation unit instantiates
// only the precision it launches.  The method is described in sgx_diff.cu.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>

#include "sgx.h"
#include "sgx_context.hpp"
#include "sgx_adjoint.cuh"
#include "sgx_dual.cuh"

namespace {

using namespace sgxd;

// Steps between checkpoints.  Sparse (64): the adjoint recomputes each
// segment into thread-local memory (65 states, 2.3 KB a thread, which streams
// through L2 and DRAM).  Dense (10): the 11 states of a segment fit in shared
// memory for 16 resident warps per SM (11 x 9 values x 4 B x 128 threads =
// 50.7 KB a block, four blocks), at 6.4x the checkpoint bytes.  FP32 with the
// hand-derived reverse pass takes the dense form when its records fit the
// form's memory budget, everything else the sparse one.
constexpr int kCkSparse = 64;
constexpr int kCkDense = 10;
constexpr int kBackwardThreads = 128;
constexpr int kMaxCross = 8;  // crossings recorded per ray (crossing model)
constexpr int NS = 8;         // state: r, theta, phi, p_r, p_theta, psi (swept angle), sin(theta), cos(theta)
constexpr int NC = NS + 1;    // checkpoint: state and transmittance

template <class T> struct DiffConst {
    T M, dcam, aspect, tanh_, width_f, height_f;
    T r_out, peak_T, escape_r, h, exposure, turbulence, time_sec;
    T eps, fade_start, fade_width, H, kappa;
    std::uint32_t width, height, spp, max_steps, flags, fade;
};

template <class T> struct DiffParamsT {
    T spin, incl, r_in, t_scale;
};

// SoA views of the per-ray buffers.
template <class T> struct DiffBufs {
    std::uint64_t n;  // rays
    std::uint32_t slots;
    T* ckpt;          // [slots][NC][n]
    T* hdr;           // [3][n]
    std::uint32_t* nsteps;
    std::uint32_t* ncross;  // crossings (crossing model) or emitting steps (slab)
    std::uint32_t* xk;  // [kMaxCross][n]: crossing steps; slab: [0] = last emitting step
    T* xw;              // [kMaxCross][n]
    T* xc;              // [kMaxCross][3][n]
    double* grads;      // [4][n]
    const T* ox;        // [spp] sub-pixel offsets
    const T* oy;
    unsigned long long* overflow;  // [0] dropped crossings, [1] steps of all rays
};

template <class S> __device__ __forceinline__ S selv(bool c, const S& a, const S& b) { return c ? a : b; }

// 1/x of the right-hand side: the SFU reciprocal in FP32 (sgxa::hrcp alike),
// a division in FP64 and for dual numbers.
template <class S> __device__ __forceinline__ S rcp_g(const S& x) {
    if constexpr (std::is_same_v<S, float>) return DM<float>::rcp_fast(x);
    else if constexpr (std::is_same_v<S, double>) return 1.0 / x;
    else {
        using T = decltype(value_of(x));
        return S(T(1)) / x;
    }
}

template <class S> __device__ __forceinline__ S smooth01(const S& x) {
    using T = decltype(value_of(x));
    if (value_of(x) <= T(0)) return S(T(0));
    if (value_of(x) >= T(1)) return S(T(1));
    return x * x * (S(T(3)) - S(T(2)) * x);
}

// Kerr Hamiltonian right-hand side (kerr_hamilton.h:97-155) in Carter's
// separated form, generic in the scalar, with sin(theta), cos(theta) read from
// the state (y[6], y[7]); d[0..6] = dr, dtheta, dphi, dp_r, dp_theta, ds, dc.
// Operation for operation sgxa::rhs7 (sgx_adjoint.cuh), which states the
// equations.
template <class S, class T>
__device__ __forceinline__ void rhs_g7(const S* y, const S& E, const S& L, const S& a, T M, S* d) {
    const S& st = y[6];
    const S& ct = y[7];
    const S r = y[0];
    const S a2 = a * a;
    const S s2 = st * st;
    const S safe_s2 = selv(value_of(s2) < T(1e-10), S(T(1e-10)), s2);
    const S r2 = r * r;
    const S r2a2 = r2 + a2;
    const S Sigma = r2 + a2 * (ct * ct);
    const S Delta = r2a2 - S(T(2) * M) * r;
    const S aE = a * E;
    const S P = r2a2 * E - a * L;
    const S W = L - aE * s2;
    const S iS = rcp_g(Sigma);
    const S iD = rcp_g(Delta);
    const S is2 = rcp_g(safe_s2);
    const S Q = P * iD, U = W * is2;
    d[0] = Delta * y[3] * iS;
    d[1] = y[4] * iS;
    d[2] = (a * Q + U) * iS;
    const S pr2 = y[3] * y[3];
    const S N = ((Delta * pr2 + y[4] * y[4]) - P * Q) + W * U;
    const S NiS = N * iS;
    d[3] = (r * NiS + ((S(M) - r) * (Q * Q + pr2) + (S(T(2)) * E * r) * Q)) * iS;
    d[4] = -(iS * (st * ct)) * (a2 * NiS - U * (S(T(2)) * aE + U));
    d[5] = ct * d[1];
    d[6] = -(st * d[1]);
}

// One fixed RK4 step with the reference's pole damping, plus the swept angle;
// (sin theta, cos theta) integrated with the state and put back on the unit
// circle by n = 3/2 - (s^2 + c^2)/2.  Operation for operation sgxa::step.
template <class S, class T>
__device__ __forceinline__ void step_g(const S* y, const S& E, const S& L, const S& a, T M, T h, bool fade, S* o) {
    const S st0 = y[6];
    S ps = selv(value_of(st0) < T(0), -st0, st0) * S(T(5));
    ps = selv(value_of(ps) > T(1), S(T(1)), selv(value_of(ps) < T(0.05), S(T(0.05)), ps));
    const S he = S(h) * ps;
    const S hh = S(T(0.5)) * he;
    S k1[7], k2[7], k3[7], k4[7], t[NS];
    t[5] = y[5];
    if constexpr (std::is_same_v<S, float>) {
        // FP32: the same fused multiply-adds on pairs of state slots (0, 1),
        // (2, 3), (6, 7) (derivative slots (0, 1), (2, 3), (5, 6)), slot 4 alone
        auto axpy = [&](const float* k, float f) {
            const F2 ff = f2(f, f);
            unf2(fma2(f2(k[0], k[1]), ff, f2(y[0], y[1])), t[0], t[1]);
            unf2(fma2(f2(k[2], k[3]), ff, f2(y[2], y[3])), t[2], t[3]);
            unf2(fma2(f2(k[5], k[6]), ff, f2(y[6], y[7])), t[6], t[7]);
            t[4] = fmaf(k[4], f, y[4]);
        };
        rhs_g7(y, E, L, a, M, k1);
        axpy(k1, hh);
        rhs_g7(t, E, L, a, M, k2);
        axpy(k2, hh);
        rhs_g7(t, E, L, a, M, k3);
        axpy(k3, he);
        rhs_g7(t, E, L, a, M, k4);
        const float h6 = he / 6.0f;
        const F2 two = f2(2.0f, 2.0f), hp = f2(h6, h6);
        auto comb = [&](int i, int j, int si, int sj) {
            const F2 sum = add2(fma2(f2(k2[i], k2[j]), two, f2(k1[i], k1[j])),
                                fma2(f2(k3[i], k3[j]), two, f2(k4[i], k4[j])));
            unf2(fma2(sum, hp, f2(y[si], y[sj])), o[si], o[sj]);
        };
        comb(0, 1, 0, 1);
        comb(2, 3, 2, 3);
        comb(5, 6, 6, 7);
        o[4] = fmaf(fmaf(k2[4], 2.0f, k1[4]) + fmaf(k3[4], 2.0f, k4[4]), h6, y[4]);
    } else {
        rhs_g7(y, E, L, a, M, k1);
#pragma unroll
        for (int i = 0; i < 7; ++i) t[sgxa::sidx(i)] = y[sgxa::sidx(i)] + k1[i] * hh;
        rhs_g7(t, E, L, a, M, k2);
#pragma unroll
        for (int i = 0; i < 7; ++i) t[sgxa::sidx(i)] = y[sgxa::sidx(i)] + k2[i] * hh;
        rhs_g7(t, E, L, a, M, k3);
#pragma unroll
        for (int i = 0; i < 7; ++i) t[sgxa::sidx(i)] = y[sgxa::sidx(i)] + k3[i] * he;
        rhs_g7(t, E, L, a, M, k4);
        const S h6 = he / S(T(6));
#pragma unroll
        for (int i = 0; i < 7; ++i)
            o[sgxa::sidx(i)] = y[sgxa::sidx(i)] + ((k1[i] + k2[i] * S(T(2))) + (k3[i] * S(T(2)) + k4[i])) * h6;
    }
    const S n = S(T(1.5)) - S(T(0.5)) * (o[6] * o[6] + o[7] * o[7]);
    o[6] = o[6] * n;
    o[7] = o[7] * n;
    if (fade) {
        const S dth = o[1] - y[1], dph = o[2] - y[2], st = o[6];
        o[5] = y[5] + DM<S>::sqrt_(dth * dth + st * st * dph * dph);
    } else {
        o[5] = y[5];
    }
}

// Blackbody colour continuous at 6600 K (the fit of geodesic_kernel.cu:77-104
// jumps there when it switches branch): the low (t <= 66) and high branch,
// t = temperature / 100 K, blended by S((t - 65) / 2); identical outside.
template <class S> __device__ __forceinline__ V3<S> blackbody_c0(const S& temp) {
    using T = decltype(value_of(temp));
    const S t = clampv(temp, S(T(1000)), S(T(40000))) * S(DM<T>::lit(0.01f, 0.01));
    const T tv = value_of(t);
    V3<S> lo, hi;
    const bool need_lo = tv < T(67), need_hi = tv > T(65);
    if (need_lo) {
        lo.x = S(T(1));
        lo.y = clampv(S(DM<T>::lit(0.39008157876901960784f, 0.39008157876901960784)) * DM<S>::log_(t) -
                          S(DM<T>::lit(0.63184144378862745098f, 0.63184144378862745098)),
                      S(T(0)), S(T(1)));
        lo.z = tv <= T(19) ? S(T(0))
                           : clampv(S(DM<T>::lit(0.54320678911019607843f, 0.54320678911019607843)) *
                                            DM<S>::log_(t - S(T(10))) -
                                        S(DM<T>::lit(1.19625408914f, 1.19625408914)),
                                    S(T(0)), S(T(1)));
    }
    if (need_hi) {
        const S t1 = t - S(T(60));
        hi.x = clampv(S(DM<T>::lit(1.29293618606274509804f, 1.29293618606274509804)) *
                          DM<S>::pow_(t1, S(DM<T>::lit(-0.1332047592f, -0.1332047592))),
                      S(T(0)), S(T(1)));
        hi.y = clampv(S(DM<T>::lit(1.12989086089529411765f, 1.12989086089529411765)) *
                          DM<S>::pow_(t1, S(DM<T>::lit(-0.0755148492f, -0.0755148492))),
                      S(T(0)), S(T(1)));
        hi.z = S(T(1));
    }
    if (!need_hi) return lo;
    if (!need_lo) return hi;
    const S sb = smooth01((t - S(T(65))) * S(T(0.5)));
    return mk3(lo.x + sb * (hi.x - lo.x), lo.y + sb * (hi.y - lo.y), lo.z + sb * (hi.z - lo.z));
}

// Disc colour at a crossing (geodesic_kernel.cu:368-393 with blackbody_c0),
// generic in the scalar.
template <class S, class T>
__device__ __forceinline__ void disc_colour_g(const S& r_c, const S& ph, const S& L, const S& a, const S& r_in,
                                              const S& T_local, const DiffConst<T>& k, S* col) {
    const T M = k.M;
    const S f_emit = S(T(1)) - S(T(2) * M) / r_c;
    const T f_obs = T(1) - T(2) * M / k.dcam;
    S g_grav = S(T(1));
    if (k.flags & SGX_FLAG_REDSHIFT_ON)
        g_grav = DM<S>::sqrt_(DM<S>::fmax_(f_emit, S(T(1e-6))) / S(f_obs > T(1e-6) ? f_obs : T(1e-6)));
    S g_dop = S(T(1));
    if (k.flags & SGX_FLAG_DOPPLER_ON) {
        const S om0 = DM<S>::sqrt_(S(M) / (r_c * r_c * r_c));
        const S omega_K = om0 / (S(T(1)) + a * om0);
        const S vel = r_c * omega_K / DM<S>::sqrt_(DM<S>::fmax_(f_emit, S(T(1e-6))));
        const S cos_psi = clampv(L / r_c, S(T(-1)), S(T(1)));
        g_dop = DM<S>::sqrt_(DM<S>::fmax_(S(T(1)) - vel * vel, S(T(0)))) /
                DM<S>::fmax_(S(T(1)) - vel * cos_psi, S(T(1e-4)));
    }
    const S g = g_grav * g_dop;
    const V3<S> bb = blackbody_c0(g * T_local);
    const S flux = clampv(DM<S>::pow_(r_in / r_c, S(T(3))), S(T(0.05)), S(T(1.5)));
    const S bands = disc_band_mask(r_c, ph, r_in, S(k.turbulence), S(k.time_sec));
    const S g2 = g * g;
    const S kk = flux * bands * g2 * g2;
    col[0] = bb.x * kk;
    col[1] = bb.y * kk;
    col[2] = bb.z * kk;
}

// Crossing between states y0 (step k-1) and y1 (step k): weight and colour.
template <class S, class T>
__device__ __forceinline__ void crossing_g(const S& r0, const S& th0, const S& psi0, const S& r1, const S& th1,
                                           const S& ph1, const S& psi1, const S& L, const S& a, const S& r_in,
                                           const S& t_scale, const DiffConst<T>& k, S* col, S& w) {
    const S mid = S(T(1.5707963267948966));
    const S frac = (mid - th0) / (th1 - th0);
    const S r_c = r0 + frac * (r1 - r0);
    w = smooth01((r_c - r_in) / S(k.eps)) * smooth01((S(k.r_out) - r_c) / S(k.eps));
    if (k.fade) {
        const S psi_c = psi0 + frac * (psi1 - psi0);
        w = w * (S(T(1)) - smooth01((psi_c - S(k.fade_start)) / S(k.fade_width)));
    }
    const S T_local = disc_temperature(r_c, r_in, S(k.peak_T) * t_scale);
    if (value_of(T_local) > T(0)) {
        disc_colour_g(r_c, ph1, L, a, r_in, T_local, k, col);
    } else {
        col[0] = col[1] = col[2] = S(T(0));
    }
}

// Camera ray and canonical initial state at pixel (gx, gy) with offset (ox, oy).
template <class S, class T>
__device__ __forceinline__ bool init_g(const S& a, const S& incl, const DiffConst<T>& k, std::uint32_t gx,
                                       std::uint32_t gy, T ox, T oy, S* y, S& E, S& L) {
    S si, ci;
    DM<S>::sincos_(incl, &si, &ci);
    const T fx = T(float(gx)) + ox, fy = T(float(gy)) + oy;
    const T u_ndc = (T(2) * fx / k.width_f - T(1)) * k.aspect * k.tanh_;
    const T v_ndc = -(T(2) * fy / k.height_f - T(1)) * k.tanh_;
    // forward (-sin i, 0, -cos i) + right (0, 1, 0) u + up (cos i, 0, -sin i) v
    S dx = -si + ci * S(v_ndc);
    S dy = S(u_ndc);
    S dz = -ci - si * S(v_ndc);
    const S len = DM<S>::fmax_(DM<S>::sqrt_(dx * dx + dy * dy + dz * dz), S(T(1e-20)));
    const S ik = S(T(1)) / len;
    dx = dx * ik;
    dy = dy * ik;
    dz = dz * ik;
    const S ur = dx * si + dz * ci;
    const S uth = (dx * ci - dz * si) / S(k.dcam);
    const S uph = dy / (S(k.dcam) * DM<S>::fmax_(si, S(T(1e-6))));
    const S r = S(k.dcam);
    const S M = S(k.M);
    const S s2 = si * si;
    const S Sigma = r * r + a * a * ci * ci;
    const S Delta = r * r - S(T(2)) * M * r + a * a;
    const S g_tt = -(S(T(1)) - S(T(2)) * M * r / Sigma);
    const S g_tp = S(T(-2)) * M * r * a * s2 / Sigma;
    const S g_rr = Sigma / Delta;
    const S g_pp = s2 * ((r * r + a * a) * (r * r + a * a) - a * a * Delta * s2) / Sigma;
    const S B = S(T(2)) * g_tp * uph;
    const S C = g_rr * ur * ur + Sigma * uth * uth + g_pp * uph * uph;
    const S disc = B * B - S(T(4)) * g_tt * C;
    if (value_of(disc) < T(0)) return false;
    const S ut = (-B - DM<S>::sqrt_(disc)) / (S(T(2)) * g_tt);
    E = -(g_tt * ut + g_tp * uph);
    L = g_tp * ut + g_pp * uph;
    y[0] = r;
    y[1] = incl;
    y[2] = S(T(0));
    y[3] = g_rr * ur;
    y[4] = Sigma * uth;
    y[5] = S(T(0));
    y[6] = si;
    y[7] = ci;
    return true;
}

// Slab emission of the step y0 -> y1, evaluated at y1, in two parts: the
// absorption alpha (false, alpha = 0, outside the layer, the annulus or past
// the fade) and the colour.  The colour depends on (r1, ph1, L, a, r_in,
// t_scale) only, so the adjoint differentiates the parts over their own
// inputs (10 and 6 dual lanes instead of 13).
template <class S, class T>
__device__ __forceinline__ bool slab_alpha_g(const S& r0, const S& th0, const S& ph0, const S& r1, const S& th1,
                                             const S& ph1, const S& psi1, const S& s1, const S& c1, const S& r_in,
                                             const DiffConst<T>& k, S& alpha) {
    const S q = r1 * c1 / S(k.H);
    if (!(value_of(q) * value_of(q) < T(1))) return false;
    S w = smooth01((r1 - r_in) / S(k.eps)) * smooth01((S(k.r_out) - r1) / S(k.eps));
    if (k.fade) w = w * (S(T(1)) - smooth01((psi1 - S(k.fade_start)) / S(k.fade_width)));
    if (!(value_of(w) > T(0))) return false;
    const S b = S(T(1)) - q * q;
    const S rho = b * b;
    const S dr = r1 - r0, dth = th1 - th0, dph = ph1 - ph0;
    const S ds = DM<S>::sqrt_(dr * dr + r1 * r1 * (dth * dth + s1 * s1 * dph * dph));
    alpha = w * (S(T(1)) - DM<S>::exp_(-(S(k.kappa) * rho * ds)));
    return true;
}

template <class S, class T>
__device__ __forceinline__ void slab_colour_g(const S& r1, const S& ph1, const S& L, const S& a, const S& r_in,
                                              const S& t_scale, const DiffConst<T>& k, S* col) {
    const S T_local = disc_temperature(r1, r_in, S(k.peak_T) * t_scale);
    if (value_of(T_local) > T(0)) {
        disc_colour_g(r1, ph1, L, a, r_in, T_local, k, col);
    } else {
        col[0] = col[1] = col[2] = S(T(0));
    }
}

template <class S, class T>
__device__ __forceinline__ bool slab_g(const S& r0, const S& th0, const S& ph0, const S& r1, const S& th1,
                                       const S& ph1, const S& psi1, const S& s1, const S& c1, const S& L,
                                       const S& a, const S& r_in, const S& t_scale, const DiffConst<T>& k, S* col,
                                       S& alpha) {
    if (!slab_alpha_g(r0, th0, ph0, r1, th1, ph1, psi1, s1, c1, r_in, k, alpha)) return false;
    slab_colour_g(r1, ph1, L, a, r_in, t_scale, k, col);
    return true;
}

// Capture radius of the form: the prograde equatorial photon orbit radius
// (the smallest photon orbit: an ingoing ray from outside that gets inside it
// falls in) less 0.05 M, at least the reference's 1.02 r_+.  Closer to the
// horizon the fixed-step RK4 turns unstable (p_r ~ 1/Delta) and a blown-up
// state could emit.
template <class T> __device__ __forceinline__ T capture_radius(T M, T a) {
    const T r_pro = T(2) * M * (T(1) + DM<T>::cos_(T(2) / T(3) * DM<T>::acos_(-a / M)));
    const T hcut = DM<T>::lit(1.02f, 1.02) * (M + DM<T>::sqrt_(DM<T>::fmax_(M * M - a * a, T(0))));
    return DM<T>::fmax_(r_pro - DM<T>::lit(0.05f, 0.05) * M, hcut);
}

template <class T>
__device__ __forceinline__ void ray_pixel(const DiffConst<T>& k, std::uint64_t id, std::uint32_t& gx, std::uint32_t& gy,
                                          std::uint32_t& s) {
    const std::uint64_t pix = id / k.spp;
    s = std::uint32_t(id - pix * k.spp);
    gy = std::uint32_t(pix / k.width);
    gx = std::uint32_t(pix - std::uint64_t(gy) * k.width);
}

template <class T, int CK>
__device__ __forceinline__ void store_ckpt(const DiffBufs<T>& b, std::uint64_t id, std::uint32_t n, const T* y, T tau) {
    const std::uint64_t base = std::uint64_t(n / CK) * NC * b.n + id;
#pragma unroll
    for (int i = 0; i < NS; ++i) b.ckpt[base + std::uint64_t(i) * b.n] = y[i];
    b.ckpt[base + std::uint64_t(NS) * b.n] = tau;
}

// Forward: one thread per ray.  SLAB: emission and absorption every step in
// the layer; otherwise soft crossings of the equatorial plane.
template <class T, bool SLAB, int CK>
__global__ void __launch_bounds__(128) diff_forward_kernel(DiffConst<T> k, DiffParamsT<T> p, DiffBufs<T> b) {
    const std::uint64_t id = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    std::uint32_t n = 0;
    if (id < b.n) {
        std::uint32_t gx, gy, s;
        ray_pixel(k, id, gx, gy, s);
        const T a = p.spin * k.M;
        const T r_in = p.r_in * k.M;
        T y[NS], prev[NS], E, L;
        T hdr[3] = {T(0), T(0), T(0)};
        std::uint32_t nc = 0, last = 0;
        if (init_g<T, T>(a, p.incl, k, gx, gy, b.ox[s], b.oy[s], y, E, L)) {
            const T hcut = capture_radius(k.M, a);
            const bool disc = (k.flags & SGX_FLAG_DISC_ON) != 0u;
            T tau = T(1);
#pragma unroll
            for (int i = 0; i < NS; ++i) prev[i] = y[i];
            for (; n < k.max_steps; ++n) {
                if (!SLAB && n % CK == 0) store_ckpt<T, CK>(b, id, n, y, tau);
                if (!isfinite(y[0]) || y[0] < hcut) break;
                if (y[0] > k.escape_r) break;
                if constexpr (SLAB) {
                    T col[3], alpha;
                    if (disc && n > 0 &&
                        slab_g<T, T>(prev[0], prev[1], prev[2], y[0], y[1], y[2], y[5], y[6], y[7], L, a, r_in,
                                     p.t_scale, k, col, alpha)) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) hdr[c] = hdr[c] + tau * alpha * col[c];
                        tau = tau * (T(1) - alpha);
                        ++nc;
                        last = n;
                    }
                    if (n % CK == 0) store_ckpt<T, CK>(b, id, n, y, tau);
                } else {
                    const T mid = T(1.5707963267948966);
                    if (disc && n > 0 && ((prev[1] - mid) * (y[1] - mid) < T(0))) {
                        T col[3], w;
                        crossing_g<T, T>(prev[0], prev[1], prev[5], y[0], y[1], y[2], y[5], L, a, r_in, p.t_scale,
                                         k, col, w);
                        if (w > T(0)) {
                            if (nc < kMaxCross) {
                                b.xk[std::uint64_t(nc) * b.n + id] = n;
                                b.xw[std::uint64_t(nc) * b.n + id] = w;
#pragma unroll
                                for (int c = 0; c < 3; ++c) b.xc[(std::uint64_t(nc) * 3 + c) * b.n + id] = col[c];
                            } else {
                                atomicAdd(b.overflow, 1ull);
                            }
                            ++nc;
#pragma unroll
                            for (int c = 0; c < 3; ++c) hdr[c] = hdr[c] + tau * w * col[c];
                            tau = tau * (T(1) - w);
                            if (!(tau > T(0))) break;
                        }
                    }
                }
                // outgoing beyond the disc, after this step's emission or crossing: a
                // photon outside the photon region moving out has no turning point
                // left, and nothing emits there (starfield off)
                if (y[3] > T(0) && y[0] > k.r_out) break;
#pragma unroll
                for (int i = 0; i < NS; ++i) prev[i] = y[i];
                step_g<T, T>(prev, E, L, a, k.M, k.h, k.fade != 0u, y);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) b.hdr[std::uint64_t(c) * b.n + id] = hdr[c];
        b.nsteps[id] = n;
        if constexpr (SLAB) {
            b.ncross[id] = nc;
            b.xk[id] = last;
        } else {
            b.ncross[id] = nc < kMaxCross ? nc : kMaxCross;
        }
    }
    // steps of the launch, one atomic per warp
    unsigned long long v = n;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31u) == 0u) atomicAdd(b.overflow + 1, v);
}

// Per pixel: mean over samples of ACES(hdr * exposure) (geodesic_kernel.cu:482-503).
template <class T>
__global__ void diff_image_kernel(DiffConst<T> k, DiffBufs<T> b, float* img) {
    const std::uint64_t pix = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (pix >= std::uint64_t(k.width) * k.height) return;
    T sum[3] = {T(0), T(0), T(0)};
    for (std::uint32_t s = 0; s < k.spp; ++s) {
        const std::uint64_t id = pix * k.spp + s;
#pragma unroll
        for (int c = 0; c < 3; ++c) sum[c] = sum[c] + aces1(b.hdr[std::uint64_t(c) * b.n + id] * k.exposure);
    }
    const T sc = T(1) / T(float(k.spp));
#pragma unroll
    for (int c = 0; c < 3; ++c) img[pix * 3 + c] = float(sum[c] * sc);
}

// d ACES(x) / dx of the Narkowicz fit, 0 where it clamps.
template <class T> __device__ __forceinline__ T aces_d(T x) {
    const T a = T(2.51), bb = T(0.03), c = T(2.43), d = T(0.59), e = T(0.14);
    const T N = x * (a * x + bb), D = x * (c * x + d) + e;
    const T f = N / D;
    if (f <= T(0) || f >= T(1)) return T(0);
    return ((T(2) * a * x + bb) * D - N * (T(2) * c * x + d)) / (D * D);
}

// lam <- J^T lam + pend for the step y_{k-1} -> y_k (J over the 6 state
// components), and the step's terms of dLoss/d(E, L, a).  DUALJ: J built
// column by column with dual numbers (the cross-check); otherwise the
// hand-derived reverse pass of sgx_adjoint.cuh.
template <class T, bool DUALJ>
__device__ __forceinline__ void step_adjoint(const T* yp, T E, T L, T a, const DiffConst<T>& k, bool fade, T* lam,
                                             const T* pend, T& muE, T& muL, T& mua) {
    if constexpr (!DUALJ) {
        T gc[3] = {T(0), T(0), T(0)};
        sgxa::step_vjp<T>(yp, E, L, a, k.M, k.h, fade, lam, gc);
        muE += gc[0];
        muL += gc[1];
        mua += gc[2];
#pragma unroll
        for (int i = 0; i < NS; ++i) lam[i] += pend[i];
        return;
    }
    using DJ = Dual<T, NS + 3>;
    DJ yd[NS], od[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) yd[i] = DJ::var(yp[i], i);
    step_g<DJ, T>(yd, DJ::var(E, NS), DJ::var(L, NS + 1), DJ::var(a, NS + 2), k.M, k.h, fade, od);
    T nl[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        T acc = T(0);
#pragma unroll
        for (int j = 0; j < NS; ++j) acc += lam[j] * od[j].d[i];
        nl[i] = acc;
    }
#pragma unroll
    for (int j = 0; j < NS; ++j) {
        muE += lam[j] * od[j].d[NS];
        muL += lam[j] * od[j].d[NS + 1];
        mua += lam[j] * od[j].d[NS + 2];
    }
#pragma unroll
    for (int i = 0; i < NS; ++i) lam[i] = nl[i] + pend[i];
}

// Adjoint: one thread per ray, a reverse sweep from the ray's last emitting
// step to the camera, one checkpoint segment at a time.  CK = kCkDense keeps
// the recomputed segment in dynamic shared memory, (CK + 1) * NC values a
// thread laid out [slot][value][thread] (consecutive threads, consecutive
// words); CK = kCkSparse in a thread-local array.  Launched with
// kBackwardThreads threads a block.
template <class T, bool SLAB, bool DUALJ, int CK>
__global__ void __launch_bounds__(kBackwardThreads, 4)
    diff_backward_kernel(DiffConst<T> k, DiffParamsT<T> p, DiffBufs<T> b, const float* __restrict__ gimg) {
    constexpr bool SHARED = CK == kCkDense;
    extern __shared__ __align__(16) unsigned char diff_seg_raw[];
    // value v of slot j of this thread's segment (shared form)
    T* const seg = reinterpret_cast<T*>(diff_seg_raw) + threadIdx.x;
    auto at = [](int j, int v) { return (j * NC + v) * kBackwardThreads; };
    const std::uint64_t id = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (id >= b.n) return;
    double* gout = b.grads;
    const std::uint32_t nc = b.ncross[id];
    // the last step whose state the image depends on
    const std::uint32_t klast = nc == 0 ? 0u : (SLAB ? b.xk[id] : b.xk[std::uint64_t(nc - 1) * b.n + id]);
    if (klast == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) gout[std::uint64_t(q) * b.n + id] = 0.0;
        return;
    }
    std::uint32_t gx, gy, s;
    ray_pixel(k, id, gx, gy, s);
    const std::uint64_t pix = id / k.spp;
    T g[3];
    const T inv_spp = T(1) / T(float(k.spp));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T x = b.hdr[std::uint64_t(c) * b.n + id] * k.exposure;
        g[c] = T(gimg[pix * 3 + c]) * inv_spp * aces_d(x) * k.exposure;
    }
    const T a = p.spin * k.M;
    const T r_in = p.r_in * k.M;
    T E, L, y0[NS];
    init_g<T, T>(a, p.incl, k, gx, gy, b.ox[s], b.oy[s], y0, E, L);

    T lam[NS] = {};
    T muE = T(0), muL = T(0), mua = T(0), g_a = T(0), g_rin = T(0), g_ts = T(0);
    const bool fade = k.fade != 0u;
    [[maybe_unused]] T Y[SHARED ? 1 : CK + 1][NS];

    // Crossing model: seeds of the transmittance chain
    //   colour = sum_j tau_j w_j c_j,  tau_{j+1} = tau_j (1 - w_j):
    //   dcolour/dc_j = tau_j w_j,  dcolour/dw_j = tau_j (c_j - R_{j+1}),
    //   R_j = w_j c_j + (1 - w_j) R_{j+1}.
    T xcs[kMaxCross], xgw[kMaxCross];
    std::uint32_t xkk[kMaxCross];
    if constexpr (!SLAB) {
        T w[kMaxCross], c3[kMaxCross][3], tau_j[kMaxCross];
        T tau = T(1);
        for (std::uint32_t j = 0; j < nc; ++j) {
            xkk[j] = b.xk[std::uint64_t(j) * b.n + id];
            w[j] = b.xw[std::uint64_t(j) * b.n + id];
#pragma unroll
            for (int c = 0; c < 3; ++c) c3[j][c] = b.xc[(std::uint64_t(j) * 3 + c) * b.n + id];
            tau_j[j] = tau;
            tau = tau * (T(1) - w[j]);
        }
        T R[3] = {T(0), T(0), T(0)};
        for (int j = int(nc) - 1; j >= 0; --j) {
            xcs[j] = tau_j[j] * w[j];
            xgw[j] = tau_j[j] * (g[0] * (c3[j][0] - R[0]) + g[1] * (c3[j][1] - R[1]) + g[2] * (c3[j][2] - R[2]));
#pragma unroll
            for (int c = 0; c < 3; ++c) R[c] = w[j] * c3[j][c] + (T(1) - w[j]) * R[c];
        }
    }
    // Slab model: the same chain over every emitting step, R carried through the sweep.
    T R[3] = {T(0), T(0), T(0)};
    [[maybe_unused]] T tb[SHARED ? 1 : CK + 1];

    const int mlast = int((klast - 1) / CK);
    for (int m = mlast; m >= 0; --m) {
        const std::uint32_t kbeg = std::uint32_t(m) * CK;
        const std::uint32_t kend = (kbeg + CK < klast) ? kbeg + CK : klast;
        const std::uint64_t cb = std::uint64_t(m) * NC * b.n + id;
        T tau = b.ckpt[cb + std::uint64_t(NS) * b.n];
        if constexpr (SHARED) {
            // the running state in registers, each state stored once
            T yc[NS];
#pragma unroll
            for (int i = 0; i < NS; ++i) {
                yc[i] = b.ckpt[cb + std::uint64_t(i) * b.n];
                seg[at(0, i)] = yc[i];
            }
            for (std::uint32_t kk = kbeg + 1; kk <= kend; ++kk) {
                const int j = int(kk - kbeg);
                T yn[NS];
                step_g<T, T>(yc, E, L, a, k.M, k.h, fade, yn);
                if constexpr (SLAB) {
                    seg[at(j, NS)] = tau;  // transmittance before step kk's emission
                    T col[3], alpha;
                    if (slab_g<T, T>(yc[0], yc[1], yc[2], yn[0], yn[1], yn[2], yn[5], yn[6], yn[7], L, a, r_in,
                                     p.t_scale, k, col, alpha))
                        tau = tau * (T(1) - alpha);
                }
#pragma unroll
                for (int i = 0; i < NS; ++i) {
                    seg[at(j, i)] = yn[i];
                    yc[i] = yn[i];
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < NS; ++i) Y[0][i] = b.ckpt[cb + std::uint64_t(i) * b.n];
            for (std::uint32_t kk = kbeg + 1; kk <= kend; ++kk) {
                const T* yp = Y[kk - 1 - kbeg];
                T* yc = Y[kk - kbeg];
                step_g<T, T>(yp, E, L, a, k.M, k.h, fade, yc);
                if constexpr (SLAB) {
                    tb[kk - kbeg] = tau;  // transmittance before step kk's emission
                    T col[3], alpha;
                    if (slab_g<T, T>(yp[0], yp[1], yp[2], yc[0], yc[1], yc[2], yc[5], yc[6], yc[7], L, a, r_in,
                                     p.t_scale, k, col, alpha))
                        tau = tau * (T(1) - alpha);
                }
            }
        }
        for (std::uint32_t kk = kend; kk > kbeg; --kk) {
            const int j = int(kk - kbeg);
            [[maybe_unused]] T ypr[NS], ycr[NS];
            const T* yp;
            const T* yc;
            if constexpr (SHARED) {
#pragma unroll
                for (int i = 0; i < NS; ++i) {
                    ypr[i] = seg[at(j - 1, i)];
                    ycr[i] = seg[at(j, i)];
                }
                yp = ypr;
                yc = ycr;
            } else {
                yp = Y[j - 1];
                yc = Y[j];
            }
            T pend[NS] = {};
            using D = Dual<T, 11>;
            using DA = Dual<T, 10>;
            using DC = Dual<T, 6>;
            if constexpr (SLAB) {
                T colv[3], alv;
                if ((k.flags & SGX_FLAG_DISC_ON) &&
                    slab_g<T, T>(yp[0], yp[1], yp[2], yc[0], yc[1], yc[2], yc[5], yc[6], yc[7], L, a, r_in,
                                 p.t_scale, k, colv, alv)) {
                    // d alpha / d(r0, th0, ph0, r1, th1, ph1, psi1, s1, c1, r_in)
                    DA ald;
                    slab_alpha_g<DA, T>(DA::var(yp[0], 0), DA::var(yp[1], 1), DA::var(yp[2], 2), DA::var(yc[0], 3),
                                        DA::var(yc[1], 4), DA::var(yc[2], 5), DA::var(yc[5], 6), DA::var(yc[6], 7),
                                        DA::var(yc[7], 8), DA::var(r_in, 9), k, ald);
                    // d colour / d(r1, ph1, L, a, r_in, t_scale)
                    DC col[3];
                    slab_colour_g<DC, T>(DC::var(yc[0], 0), DC::var(yc[2], 1), DC::var(L, 2), DC::var(a, 3),
                                         DC::var(r_in, 4), DC::var(p.t_scale, 5), k, col);
                    T tj;
                    if constexpr (SHARED) tj = seg[at(j, NS)];
                    else tj = tb[j];
                    const T gcs = tj * alv;
                    const T gal = tj * (g[0] * (colv[0] - R[0]) + g[1] * (colv[1] - R[1]) + g[2] * (colv[2] - R[2]));
#pragma unroll
                    for (int c = 0; c < 3; ++c) R[c] = alv * colv[c] + (T(1) - alv) * R[c];
                    T qa[10], qc[6];
#pragma unroll
                    for (int x = 0; x < 10; ++x) qa[x] = gal * ald.d[x];
#pragma unroll
                    for (int x = 0; x < 6; ++x)
                        qc[x] = gcs * (g[0] * col[0].d[x] + g[1] * col[1].d[x] + g[2] * col[2].d[x]);
                    pend[0] += qa[0];
                    pend[1] += qa[1];
                    pend[2] += qa[2];
                    lam[0] += qa[3] + qc[0];
                    lam[1] += qa[4];
                    lam[2] += qa[5] + qc[1];
                    lam[5] += qa[6];
                    lam[6] += qa[7];
                    lam[7] += qa[8];
                    muL += qc[2];
                    g_a += qc[3] * k.M;
                    g_rin += (qa[9] + qc[4]) * k.M;
                    g_ts += qc[5];
                }
            } else {
                for (std::uint32_t j = 0; j < nc; ++j) {
                    if (xkk[j] != kk) continue;
                    // d(colour, weight)/d(r0, th0, psi0, r1, th1, ph1, psi1, L, a, r_in, t_scale)
                    D col[3], wd;
                    crossing_g<D, T>(D::var(yp[0], 0), D::var(yp[1], 1), D::var(yp[5], 2), D::var(yc[0], 3),
                                     D::var(yc[1], 4), D::var(yc[2], 5), D::var(yc[5], 6), D::var(L, 7),
                                     D::var(a, 8), D::var(r_in, 9), D::var(p.t_scale, 10), k, col, wd);
                    T qv[11];
#pragma unroll
                    for (int x = 0; x < 11; ++x)
                        qv[x] = xcs[j] * (g[0] * col[0].d[x] + g[1] * col[1].d[x] + g[2] * col[2].d[x]) +
                                xgw[j] * wd.d[x];
                    pend[0] += qv[0];
                    pend[1] += qv[1];
                    pend[5] += qv[2];
                    lam[0] += qv[3];
                    lam[1] += qv[4];
                    lam[2] += qv[5];
                    lam[5] += qv[6];
                    muL += qv[7];
                    g_a += qv[8] * k.M;
                    g_rin += qv[9] * k.M;
                    g_ts += qv[10];
                }
            }
            step_adjoint<T, DUALJ>(yp, E, L, a, k, fade, lam, pend, muE, muL, mua);
        }
    }
    // Chain through the camera set-up: y0, E, L as functions of (a, incl).
    using D2 = Dual<T, 2>;
    D2 yd0[NS], Ed, Ld;
    init_g<D2, T>(D2::var(a, 0), D2::var(p.incl, 1), k, gx, gy, b.ox[s], b.oy[s], yd0, Ed, Ld);
    T grad_a = g_a + mua * k.M, grad_i = T(0);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        grad_a += lam[i] * yd0[i].d[0] * k.M;
        grad_i += lam[i] * yd0[i].d[1];
    }
    grad_a += (muE * Ed.d[0] + muL * Ld.d[0]) * k.M;
    grad_i += muE * Ed.d[1] + muL * Ld.d[1];
    gout[id] = double(grad_a);
    gout[b.n + id] = double(grad_i);
    gout[2 * b.n + id] = double(g_rin);
    gout[3 * b.n + id] = double(g_ts);
}

// Fixed-order sum of the per-ray gradients: block-level tree over 1024-ray
// chunks, then one block over the chunk sums.
__global__ void reduce_chunks(const double* __restrict__ in, std::uint64_t n, double* __restrict__ part,
                              std::uint32_t nchunks) {
    __shared__ double sh[256];
    const std::uint32_t chunk = blockIdx.x, q = blockIdx.y;
    const std::uint64_t beg = std::uint64_t(chunk) * 1024;
    double acc = 0.0;
    for (int i = 0; i < 4; ++i) {
        const std::uint64_t j = beg + threadIdx.x + i * 256;
        if (j < n) acc += in[std::uint64_t(q) * n + j];
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (int(threadIdx.x) < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[std::uint64_t(q) * nchunks + chunk] = sh[0];
}

__global__ void reduce_final(const double* __restrict__ part, std::uint32_t nchunks, double* __restrict__ out) {
    __shared__ double sh[256];
    const std::uint32_t q = blockIdx.x;
    double acc = 0.0;
    for (std::uint32_t i = threadIdx.x; i < nchunks; i += 256) acc += part[std::uint64_t(q) * nchunks + i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (int(threadIdx.x) < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[q] = sh[0];
}

template <class T> __global__ void offsets_kernel(std::uint32_t spp, T* ox, T* oy) {
    const std::uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < spp) sample_offset<T>(spp, s, ox[s], oy[s]);
}

template <class T>
DiffConst<T> make_const(const sgx_uniforms& u, const sgx_diff_opts& o) {
    DiffConst<T> k{};
    k.M = T(u.mass_M);
    {  // |cam_pos| formed in T from the float components
        const T x = T(u.cam_pos.x), y = T(u.cam_pos.y), z = T(u.cam_pos.z);
        k.dcam = T(std::sqrt(x * x + y * y + z * z));
    }
    k.aspect = T(u.aspect);
    k.tanh_ = T(u.tan_half_fov);
    k.width_f = T(float(u.width));
    k.height_f = T(float(u.height));
    k.r_out = T(u.disc_r_outer);
    k.peak_T = T(u.disc_peak_T);
    k.escape_r = T(u.escape_r);
    k.h = T(u.h_step);
    k.exposure = T(u.exposure);
    k.turbulence = T(u.disc_turbulence);
    k.time_sec = T(u.time_sec);
    k.eps = T(o.edge_width) * T(u.mass_M);
    k.fade_start = T(o.fade_start);
    k.fade_width = T(o.fade_width);
    k.fade = o.fade_start > 0.0f ? 1u : 0u;
    k.H = T(o.half_thickness) * T(u.mass_M);
    k.kappa = T(o.tau_perp) / (T(16) / T(15) * k.H);
    k.width = u.width;
    k.height = u.height;
    k.spp = u.supersample < 1u ? 1u : (u.supersample > 1024u ? 1024u : u.supersample);
    k.max_steps = u.max_steps;
    k.flags = u.flags;
    return k;
}

}  // namespace

// Per-context state of the differentiable form (the forward's records).
struct sgx_diff_state {
    void* mem = nullptr;
    std::size_t cap = 0;
    std::uint64_t n = 0;
    std::uint32_t slots = 0;
    std::uint32_t ck = kCkSparse;  // steps between checkpoints (kCkSparse or kCkDense)
    std::uint32_t precision = SGX_PRECISION_FP32;
    std::uint32_t nx = kMaxCross;  // crossing records per ray (1 for the slab model)
    sgx_uniforms u{};
    sgx_diff_params p{};
    sgx_diff_opts o{};
    bool valid = false;
    float* img = nullptr;  // internal image when the caller passes none
    std::size_t img_cap = 0;
};

namespace {

template <class T>
DiffBufs<T> carve_bufs(sgx_diff_state& st, std::uint32_t spp) {
    DiffBufs<T> b{};
    const std::uint64_t n = st.n;
    unsigned char* p = static_cast<unsigned char*>(st.mem);
    auto take = [&](std::size_t bytes) {
        unsigned char* r = p;
        p += (bytes + 255) / 256 * 256;
        return r;
    };
    b.n = n;
    b.slots = st.slots;
    const std::size_t nx = st.nx;
    b.ckpt = reinterpret_cast<T*>(take(std::size_t(st.slots) * NC * n * sizeof(T)));
    b.hdr = reinterpret_cast<T*>(take(3 * n * sizeof(T)));
    b.nsteps = reinterpret_cast<std::uint32_t*>(take(n * 4));
    b.ncross = reinterpret_cast<std::uint32_t*>(take(n * 4));
    b.xk = reinterpret_cast<std::uint32_t*>(take(nx * n * 4));
    b.xw = nx > 1 ? reinterpret_cast<T*>(take(nx * n * sizeof(T))) : nullptr;
    b.xc = nx > 1 ? reinterpret_cast<T*>(take(nx * 3 * n * sizeof(T))) : nullptr;
    b.grads = reinterpret_cast<double*>(take(4 * n * 8));
    T* off = reinterpret_cast<T*>(take(2 * std::size_t(spp) * sizeof(T)));
    b.ox = off;
    b.oy = off + spp;
    b.overflow = reinterpret_cast<unsigned long long*>(take(64));
    return b;
}

template <class T>
std::size_t state_bytes(std::uint64_t n, std::uint32_t slots, std::uint32_t spp, std::size_t nx) {
    auto r = [](std::size_t x) { return (x + 255) / 256 * 256; };
    return r(std::size_t(slots) * NC * n * sizeof(T)) + r(3 * n * sizeof(T)) + 2 * r(n * 4) + r(nx * n * 4) +
           (nx > 1 ? r(nx * n * sizeof(T)) + r(nx * 3 * n * sizeof(T)) : 0) + r(4 * n * 8) +
           r(2 * std::size_t(spp) * sizeof(T)) + 256 +
           // reduction scratch: 4 x chunk sums + 4 results
           r(4 * ((n + 1023) / 1024) * 8) + 256;
}

template <class T>
cudaError_t run_forward(sgx_diff_state& st, float* img, cudaStream_t s) {
    const DiffConst<T> k = make_const<T>(st.u, st.o);
    const DiffParamsT<T> p{T(st.p.spin), T(st.p.incl), T(st.p.r_in), T(st.p.t_scale)};
    DiffBufs<T> b = carve_bufs<T>(st, k.spp);
    cudaError_t e = cudaMemsetAsync(b.overflow, 0, 16, s);
    if (e != cudaSuccess) return e;
    offsets_kernel<T><<<(k.spp + 127) / 128, 128, 0, s>>>(k.spp, const_cast<T*>(b.ox), const_cast<T*>(b.oy));
    const unsigned grid = unsigned((st.n + 127) / 128);
    const bool slab = st.o.model == SGX_DIFF_MODEL_SLAB;
    bool dense = false;
    if constexpr (sizeof(T) == 4) dense = st.ck == std::uint32_t(kCkDense);
    if constexpr (sizeof(T) == 4) {
        if (dense && slab) diff_forward_kernel<T, true, kCkDense><<<grid, 128, 0, s>>>(k, p, b);
        else if (dense) diff_forward_kernel<T, false, kCkDense><<<grid, 128, 0, s>>>(k, p, b);
    }
    if (!dense && slab) diff_forward_kernel<T, true, kCkSparse><<<grid, 128, 0, s>>>(k, p, b);
    else if (!dense) diff_forward_kernel<T, false, kCkSparse><<<grid, 128, 0, s>>>(k, p, b);
    const std::uint64_t npix = std::uint64_t(k.width) * k.height;
    diff_image_kernel<T><<<unsigned((npix + 255) / 256), 256, 0, s>>>(k, b, img);
    return cudaGetLastError();
}

template <class T>
cudaError_t run_backward(sgx_diff_state& st, const float* gimg, double* d_out4, cudaStream_t s) {
    const DiffConst<T> k = make_const<T>(st.u, st.o);
    const DiffParamsT<T> p{T(st.p.spin), T(st.p.incl), T(st.p.r_in), T(st.p.t_scale)};
    DiffBufs<T> b = carve_bufs<T>(st, k.spp);
    const unsigned grid = unsigned((st.n + kBackwardThreads - 1) / kBackwardThreads);
    const bool slab = st.o.model == SGX_DIFF_MODEL_SLAB, dual = st.o.adjoint_form == SGX_DIFF_ADJOINT_DUAL;
    bool dense = false;
    if constexpr (sizeof(T) == 4) {
        // the dense checkpoints pair with the hand-derived reverse pass only
        dense = st.ck == std::uint32_t(kCkDense);
        if (dense) {
            const int smem = (kCkDense + 1) * NC * kBackwardThreads * int(sizeof(T));
            auto* kern = slab ? diff_backward_kernel<T, true, false, kCkDense>
                              : diff_backward_kernel<T, false, false, kCkDense>;
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            kern<<<grid, kBackwardThreads, smem, s>>>(k, p, b, gimg);
        }
    }
    if (!dense) {
        if (slab && !dual) diff_backward_kernel<T, true, false, kCkSparse><<<grid, kBackwardThreads, 0, s>>>(k, p, b, gimg);
        else if (slab) diff_backward_kernel<T, true, true, kCkSparse><<<grid, kBackwardThreads, 0, s>>>(k, p, b, gimg);
        else if (!dual) diff_backward_kernel<T, false, false, kCkSparse><<<grid, kBackwardThreads, 0, s>>>(k, p, b, gimg);
        else diff_backward_kernel<T, false, true, kCkSparse><<<grid, kBackwardThreads, 0, s>>>(k, p, b, gimg);
    }
    const std::uint32_t nchunks = std::uint32_t((st.n + 1023) / 1024);
    double* part = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(b.overflow) + 256);
    reduce_chunks<<<dim3(nchunks, 4), 256, 0, s>>>(b.grads, st.n, part, nchunks);
    reduce_final<<<4, 256, 0, s>>>(part, nchunks, d_out4);
    return cudaGetLastError();
}

}  // namespace


// Entry points of the two translation units (defined in sgx_diff.cu for
// float and in sgx_diff64.cu for double).
cudaError_t sgx_diff_run_forward_f32(sgx_diff_state& st, float* img, cudaStream_t s);
cudaError_t sgx_diff_run_backward_f32(sgx_diff_state& st, const float* gimg, double* d_out4, cudaStream_t s);
cudaError_t sgx_diff_run_forward_f64(sgx_diff_state& st, float* img, cudaStream_t s);
cudaError_t sgx_diff_run_backward_f64(sgx_diff_state& st, const float* gimg, double* d_out4, cudaStream_t s);
