// singularity_gb300/csrc/sgx_adjoint.cuh
//
// Reverse-mode (vector-Jacobian) products of the Kerr Hamiltonian right-hand
// side and of one fixed RK4 step with the reference's pole damping
// (kerr_hamilton.h:97-178), derived by hand: given the adjoint of a step's
// output, they return the adjoint of its input state and of the constants
// (E, L_z, a).  The adjoint sweep of sgx_diff.cu multiplies by these instead
// of building the step's 8 x 11 Jacobian with dual numbers: four right-hand
// side evaluations and four reverse passes per step instead of eleven-lane
// dual arithmetic.
//
// Host-and-device code (plain arithmetic, sqrt overloads, the SFU reciprocal
// on the device in FP32), so the derivatives can be checked against finite
// differences on the CPU.
#pragma once

#include <cmath>
#include <type_traits>

#if defined(__CUDACC__)
#define SGX_HD __host__ __device__ __forceinline__
#include "sgx_device.cuh"  // packed FP32 pairs (device only)
#else
#define SGX_HD inline
#endif

namespace sgxa {

SGX_HD float hsqrt(float x) { return sqrtf(x); }
SGX_HD double hsqrt(double x) { return sqrt(x); }
// 1/x: PTX rcp.approx.ftz.f32 on the device in FP32 (one SFU instruction, at
// most 1 ulp from 1/x; the forward kernel's rhs_g does the same), exact
// elsewhere.
SGX_HD float hrcp(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}
SGX_HD double hrcp(double x) { return 1.0 / x; }
// State layout: y[0..7] = r, theta, phi, p_r, p_theta, psi (swept angle),
// s = sin(theta), c = cos(theta); derivative layout d[0..6] = dr, dtheta,
// dphi, dp_r, dp_theta, ds, dc.  theta is integrated for the swept angle and
// the emission's path length; the right-hand side reads (s, c).
SGX_HD constexpr int sidx(int i) { return i < 5 ? i : i + 1; }  // state index of derivative i

// o = y + k f over the seven integrated state slots (derivative i -> state
// sidx(i)); on the device in FP32 the same fused multiply-adds run on the
// pairs of state slots (0, 1), (2, 3), (6, 7).
template <class T> SGX_HD void stage7(const T* y, const T* k, T f, T* o) {
#if defined(__CUDA_ARCH__)
    if constexpr (std::is_same_v<T, float>) {
        using namespace sgxd;
        const F2 ff = f2(f, f);
        unf2(fma2(f2(k[0], k[1]), ff, f2(y[0], y[1])), o[0], o[1]);
        unf2(fma2(f2(k[2], k[3]), ff, f2(y[2], y[3])), o[2], o[3]);
        unf2(fma2(f2(k[5], k[6]), ff, f2(y[6], y[7])), o[6], o[7]);
        o[4] = fmaf(k[4], f, y[4]);
        return;
    }
#endif
    for (int i = 0; i < 7; ++i) o[sidx(i)] = y[sidx(i)] + k[i] * f;
}

// The reverse pass's accumulations over the seven integrated slots, on the
// device in FP32 as packed pairs (derivative slots (0, 1), (2, 3), (5, 6),
// state slots (0, 1), (2, 3), (6, 7)); a dot product is then summed as two
// pair lanes, so its last bits can differ from the sequential sum.
// ly[sidx(i)] += g[sidx(i)], lk[i] += f g[sidx(i)], acc += g[sidx(i)] k[i]:
template <class T> SGX_HD void vjp_accum7(const T* g, T f, const T* k, T* ly, T* lk, T& acc) {
#if defined(__CUDA_ARCH__)
    if constexpr (std::is_same_v<T, float>) {
        using namespace sgxd;
        const F2 ff = f2(f, f);
        F2 dot = f2(0.0f, 0.0f);
        for (int p = 0; p < 3; ++p) {
            const int j = p < 2 ? 2 * p : 5, q = p < 2 ? 2 * p : 6;
            const F2 gp = f2(g[q], g[q + 1]);
            unf2(add2(f2(ly[q], ly[q + 1]), gp), ly[q], ly[q + 1]);
            unf2(fma2(gp, ff, f2(lk[j], lk[j + 1])), lk[j], lk[j + 1]);
            dot = fma2(gp, f2(k[j], k[j + 1]), dot);
        }
        float d0, d1;
        unf2(dot, d0, d1);
        ly[4] += g[4];
        lk[4] = fmaf(f, g[4], lk[4]);
        acc = fmaf(g[4], k[4], acc + (d0 + d1));
        return;
    }
#endif
    for (int i = 0; i < 7; ++i) {
        const T gi = g[sidx(i)];
        ly[sidx(i)] += gi;
        lk[i] += f * gi;
        acc += gi * k[i];
    }
}

// From the output adjoint lo: ly[sidx(i)] += l, lk1 = lk4 = l h6,
// lk2 = lk3 = l 2 h6, acc += l ks[i] (l = lo[sidx(i)]).
template <class T>
SGX_HD void vjp_out7(const T* lo, T h6, const T* ks, T* ly, T* lk1, T* lk2, T* lk3, T* lk4, T& acc) {
#if defined(__CUDA_ARCH__)
    if constexpr (std::is_same_v<T, float>) {
        using namespace sgxd;
        const F2 hp = f2(h6, h6), h2p = f2(2.0f * h6, 2.0f * h6);
        F2 dot = f2(0.0f, 0.0f);
        for (int p = 0; p < 3; ++p) {
            const int j = p < 2 ? 2 * p : 5, q = p < 2 ? 2 * p : 6;
            const F2 lp = f2(lo[q], lo[q + 1]);
            unf2(add2(f2(ly[q], ly[q + 1]), lp), ly[q], ly[q + 1]);
            unf2(mul2(lp, hp), lk1[j], lk1[j + 1]);
            unf2(mul2(lp, h2p), lk2[j], lk2[j + 1]);
            lk3[j] = lk2[j];
            lk3[j + 1] = lk2[j + 1];
            lk4[j] = lk1[j];
            lk4[j + 1] = lk1[j + 1];
            dot = fma2(lp, f2(ks[j], ks[j + 1]), dot);
        }
        float d0, d1;
        unf2(dot, d0, d1);
        const float l = lo[4];
        ly[4] += l;
        lk1[4] = lk4[4] = l * h6;
        lk2[4] = lk3[4] = l * (2.0f * h6);
        acc = fmaf(l, ks[4], acc + (d0 + d1));
        return;
    }
#endif
    for (int i = 0; i < 7; ++i) {
        const T l = lo[sidx(i)];
        ly[sidx(i)] += l;
        lk1[i] = l * h6;
        lk2[i] = l * (T(2) * h6);
        lk3[i] = l * (T(2) * h6);
        lk4[i] = l * h6;
        acc += l * ks[i];
    }
}

// ks = (k1 + 2 k2) + (2 k3 + k4), the RK4 weights' sum (pairs on the device in FP32).
template <class T> SGX_HD void ksum7(const T* k1, const T* k2, const T* k3, const T* k4, T* ks) {
#if defined(__CUDA_ARCH__)
    if constexpr (std::is_same_v<T, float>) {
        using namespace sgxd;
        const F2 two = f2(2.0f, 2.0f);
        for (int i = 0; i < 6; i += 2) {
            const int j = i < 4 ? i : 5;  // pairs (0, 1), (2, 3), (5, 6)
            unf2(add2(fma2(f2(k2[j], k2[j + 1]), two, f2(k1[j], k1[j + 1])),
                      fma2(f2(k3[j], k3[j + 1]), two, f2(k4[j], k4[j + 1]))),
                 ks[j], ks[j + 1]);
        }
        ks[4] = fmaf(k2[4], 2.0f, k1[4]) + fmaf(k3[4], 2.0f, k4[4]);
        return;
    }
#endif
    for (int i = 0; i < 7; ++i) ks[i] = (k1[i] + k2[i] * T(2)) + (k3[i] * T(2) + k4[i]);
}

// The right-hand side in Carter's separated form (the same Hamiltonian as
// kerr_hamilton.h:97-155): with P = (r^2 + a^2) E - a L, W = L - a E s2,
// Q = P / Delta, U = W / s2 and N = 2 Sigma H = Delta p_r^2 + p_th^2 - P Q + W U,
//   dr = Delta p_r / Sigma, dth = p_th / Sigma, dphi = (a Q + U) / Sigma,
//   dp_r  = (r N / Sigma + (M - r)(p_r^2 + Q^2) + 2 E r Q) / Sigma,
//   dp_th = -sin(th) cos(th) (a^2 N / Sigma - U (2 a E + U)) / Sigma.
// plus ds = cos(th) dth, dc = -sin(th) dth, with sin(th), cos(th) read from
// the state.  Operation for operation the forward kernel's rhs_g7
// (sgx_diff_impl.cuh).
template <class T>
SGX_HD void rhs7(const T* y, T E, T L, T a, T M, T* d) {
    const T st = y[6], ct = y[7];
    const T r = y[0];
    const T a2 = a * a;
    const T s2 = st * st;
    const T ss = s2 < T(1e-10) ? T(1e-10) : s2;
    const T r2 = r * r;
    const T r2a2 = r2 + a2;
    const T Sig = r2 + a2 * (ct * ct);
    const T Del = r2a2 - (T(2) * M) * r;
    const T aE = a * E;
    const T P = r2a2 * E - a * L;
    const T W = L - aE * s2;
    const T iS = hrcp(Sig), iD = hrcp(Del), is2 = hrcp(ss);
    const T Q = P * iD, U = W * is2;
    d[0] = Del * y[3] * iS;
    d[1] = y[4] * iS;
    d[2] = (a * Q + U) * iS;
    const T pr2 = y[3] * y[3];
    const T N = ((Del * pr2 + y[4] * y[4]) - P * Q) + W * U;
    const T NiS = N * iS;
    d[3] = (r * NiS + ((M - r) * (Q * Q + pr2) + (T(2) * E * r) * Q)) * iS;
    d[4] = -(iS * (st * ct)) * (a2 * NiS - U * (T(2) * aE + U));
    d[5] = ct * d[1];
    d[6] = -(st * d[1]);
}

// w . d(rhs7)/d(r, p_r, p_theta, sin th, cos th, E, L, a), w the adjoint of
// d[0..6].  gy[0..7] receives the state part (zero for theta, phi and psi,
// which the right-hand side does not read); gc[0..2] += the constants' part.
template <class T>
SGX_HD void rhs_vjp7(const T* y, T E, T L, T a, T M, const T* w, T* gy, T* gc) {
    // forward intermediates
    const T st = y[6], ct = y[7];
    const T r = y[0], pr = y[3], pth = y[4];
    const T a2 = a * a;
    const T s2 = st * st;
    const bool s2_free = !(s2 < T(1e-10));
    const T ss = s2_free ? s2 : T(1e-10);
    const T r2 = r * r;
    const T r2a2 = r2 + a2;
    const T c2 = ct * ct;
    const T Sig = r2 + a2 * c2;
    const T Del = r2a2 - (T(2) * M) * r;
    const T aE = a * E;
    const T P = r2a2 * E - a * L;
    const T W = L - aE * s2;
    const T iS = hrcp(Sig), iD = hrcp(Del), is2 = hrcp(ss);
    const T Q = P * iD, U = W * is2;
    const T pr2 = pr * pr;
    const T N = ((Del * pr2 + pth * pth) - P * Q) + W * U;
    const T NiS = N * iS;
    const T X = Q * Q + pr2;
    const T A3 = r * NiS + ((M - r) * X + (T(2) * E * r) * Q);
    const T C2 = a * Q + U;
    const T V1 = T(2) * aE + U;
    const T B4 = a2 * NiS - U * V1;
    const T sc = st * ct;

    // reverse: d5 = ct d1, d6 = -st d1 fold into d1's adjoint;
    // d0 = Del pr iS, d1 = pth iS, d2 = C2 iS, d3 = A3 iS, d4 = -(iS sc) B4
    const T d1v = pth * iS;
    const T w0 = w[0], w1 = w[1] + w[5] * ct - w[6] * st, w2 = w[2], w3 = w[3], w4 = w[4];
    T iS_b = w0 * Del * pr + w1 * pth + w2 * C2 + w3 * A3 - w4 * sc * B4;
    T Del_b = w0 * pr * iS;
    T pr_b = w0 * Del * iS;
    T pth_b = w1 * iS;
    const T C2_b = w2 * iS;
    const T A3_b = w3 * iS;
    const T sc_b = -w4 * iS * B4;
    const T B4_b = -w4 * iS * sc;
    // C2 = a Q + U
    T a_b = C2_b * Q;
    T Q_b = C2_b * a;
    T U_b = C2_b;
    // A3 = r NiS + (M - r) X + 2 E r Q
    T r_b = A3_b * (NiS - X + T(2) * E * Q);
    T NiS_b = A3_b * r;
    const T X_b = A3_b * (M - r);
    T E_b = A3_b * T(2) * r * Q;
    Q_b += A3_b * T(2) * E * r;
    // B4 = a2 NiS - U V1 ; V1 = 2 aE + U
    T a2_b = B4_b * NiS;
    NiS_b += B4_b * a2;
    U_b += -B4_b * V1;
    const T V1_b = -B4_b * U;
    T aE_b = T(2) * V1_b;
    U_b += V1_b;
    // X = Q^2 + pr2
    Q_b += T(2) * Q * X_b;
    T pr2_b = X_b;
    // NiS = N iS
    const T N_b = NiS_b * iS;
    iS_b += NiS_b * N;
    // N = Del pr2 + pth^2 - P Q + W U
    Del_b += N_b * pr2;
    pr2_b += N_b * Del;
    pth_b += T(2) * pth * N_b;
    T P_b = -N_b * Q;
    Q_b += -N_b * P;
    T W_b = N_b * U;
    U_b += N_b * W;
    // Q = P iD ; U = W is2
    P_b += Q_b * iD;
    const T iD_b = Q_b * P;
    W_b += U_b * is2;
    const T is2_b = U_b * W;
    // reciprocals
    const T Sig_b = -iS_b * iS * iS;
    Del_b += -iD_b * iD * iD;
    T s2_b = s2_free ? -is2_b * is2 * is2 : T(0);
    // W = L - aE s2
    T L_b = W_b;
    aE_b += -W_b * s2;
    s2_b += -W_b * aE;
    // P = r2a2 E - a L
    T r2a2_b = P_b * E;
    E_b += P_b * r2a2;
    a_b += -P_b * L;
    L_b += -P_b * a;
    // aE = a E
    a_b += aE_b * E;
    E_b += aE_b * a;
    // Del = r2a2 - 2 M r
    r2a2_b += Del_b;
    r_b += -(T(2) * M) * Del_b;
    // Sig = r2 + a2 c2 ; r2a2 = r2 + a2
    const T r2_b = Sig_b + r2a2_b;
    a2_b += Sig_b * c2 + r2a2_b;
    const T c2_b = Sig_b * a2;
    pr_b += T(2) * pr * pr2_b;
    r_b += T(2) * r * r2_b;
    a_b += T(2) * a * a2_b;
    // sc = st ct ; c2 = ct^2 ; s2 = st^2 ; and d5, d6
    const T st_b = sc_b * ct + T(2) * st * s2_b - w[6] * d1v;
    const T ct_b = sc_b * st + T(2) * ct * c2_b + w[5] * d1v;

    gy[0] = r_b;
    gy[1] = T(0);
    gy[2] = T(0);
    gy[3] = pr_b;
    gy[4] = pth_b;
    gy[5] = T(0);
    gy[6] = st_b;
    gy[7] = ct_b;
    gc[0] += E_b;
    gc[1] += L_b;
    gc[2] += a_b;
}

// Pole-damped step length h * clamp(5 |s|, 0.05, 1) and its derivative in s
// (kerr_hamilton.h:165-178, |sin theta| read from the state).
template <class T> SGX_HD T damped_h_s(T h, T s, T* dh_ds) {
    const T as = s < T(0) ? -s : s;
    T ps = as * T(5);
    T dps = s < T(0) ? T(-5) : T(5);
    if (ps > T(1)) {
        ps = T(1);
        dps = T(0);
    } else if (ps < T(0.05)) {
        ps = T(0.05);
        dps = T(0);
    }
    *dh_ds = h * dps;
    return h * ps;
}

// One RK4 step y -> o: (s, c) back on the unit circle by
// n = 3/2 - (s^2 + c^2)/2, and the swept angle when `fade`.
template <class T> SGX_HD void step(const T* y, T E, T L, T a, T M, T h, bool fade, T* o) {
    T dhd;
    const T he = damped_h_s(h, y[6], &dhd);
    const T hh = T(0.5) * he;
    T k1[7], k2[7], k3[7], k4[7], t[8];
    t[5] = y[5];
    rhs7(y, E, L, a, M, k1);
    for (int i = 0; i < 7; ++i) t[sidx(i)] = y[sidx(i)] + k1[i] * hh;
    rhs7(t, E, L, a, M, k2);
    for (int i = 0; i < 7; ++i) t[sidx(i)] = y[sidx(i)] + k2[i] * hh;
    rhs7(t, E, L, a, M, k3);
    for (int i = 0; i < 7; ++i) t[sidx(i)] = y[sidx(i)] + k3[i] * he;
    rhs7(t, E, L, a, M, k4);
    const T h6 = he / T(6);
    for (int i = 0; i < 7; ++i) o[sidx(i)] = y[sidx(i)] + ((k1[i] + k2[i] * T(2)) + (k3[i] * T(2) + k4[i])) * h6;
    const T n = T(1.5) - T(0.5) * (o[6] * o[6] + o[7] * o[7]);
    o[6] = o[6] * n;
    o[7] = o[7] * n;
    if (fade) {
        const T dth = o[1] - y[1], dph = o[2] - y[2], s = o[6];
        o[5] = y[5] + hsqrt(dth * dth + s * s * dph * dph);
    } else {
        o[5] = y[5];
    }
}

// Adjoint of one step: lam (adjoint of the step's output, 8 components) is
// replaced by the adjoint of its input; gc[0..2] += the step's terms of
// dLoss/d(E, L, a).
template <class T> SGX_HD void step_vjp(const T* y, T E, T L, T a, T M, T h, bool fade, T* lam, T* gc) {
    T dhd;
    const T he = damped_h_s(h, y[6], &dhd);
    const T hh = T(0.5) * he;
    T k1[7], k2[7], k3[7], k4[7], y2[8], y3[8], y4[8];
    y2[5] = y3[5] = y4[5] = y[5];
    rhs7(y, E, L, a, M, k1);
    stage7(y, k1, hh, y2);
    rhs7(y2, E, L, a, M, k2);
    stage7(y, k2, hh, y3);
    rhs7(y3, E, L, a, M, k3);
    stage7(y, k3, he, y4);
    rhs7(y4, E, L, a, M, k4);
    const T h6 = he / T(6);
    T ks[7];
    ksum7(k1, k2, k3, k4, ks);
    // RK4 output before and after the renormalisation of (s, c)
    const T s_hat = y[6] + ks[5] * h6, c_hat = y[7] + ks[6] * h6;
    const T n = T(1.5) - T(0.5) * (s_hat * s_hat + c_hat * c_hat);
    const T os = s_hat * n;
    T lo[8];
    for (int i = 0; i < 8; ++i) lo[i] = lam[i];
    T ly[8];
    for (int i = 0; i < 8; ++i) ly[i] = T(0);
    ly[5] = lam[5];
    // swept angle: o5 = y5 + sqrt(dth^2 + os^2 dph^2)
    T l_y1_psi = T(0), l_y2_psi = T(0);
    if (fade && lam[5] != T(0)) {
        const T dth = ks[1] * h6, dph = ks[2] * h6;
        const T q = hsqrt(dth * dth + os * os * dph * dph);
        if (q > T(0)) {
            const T iq = lam[5] / q;
            lo[1] += iq * dth;
            lo[2] += iq * os * os * dph;
            lo[6] += iq * os * dph * dph;
            l_y1_psi = -iq * dth;
            l_y2_psi = -iq * os * os * dph;
        }
    }
    // (os, oc) = n (s_hat, c_hat)
    {
        const T tt = lo[6] * s_hat + lo[7] * c_hat;
        const T ls = lo[6] * n - s_hat * tt;
        const T lc = lo[7] * n - c_hat * tt;
        lo[6] = ls;
        lo[7] = lc;
    }
    // o = y + ks h6
    T lk1[7], lk2[7], lk3[7], lk4[7];
    T l_he = T(0);
    vjp_out7(lo, h6, ks, ly, lk1, lk2, lk3, lk4, l_he);
    l_he *= T(1) / T(6);
    ly[1] += l_y1_psi;
    ly[2] += l_y2_psi;
    T g[8];
    // k4 = f(y4), y4 = y + he k3
    rhs_vjp7(y4, E, L, a, M, lk4, g, gc);
    vjp_accum7(g, he, k3, ly, lk3, l_he);
    T l_hh = T(0);
    // k3 = f(y3), y3 = y + hh k2
    rhs_vjp7(y3, E, L, a, M, lk3, g, gc);
    vjp_accum7(g, hh, k2, ly, lk2, l_hh);
    // k2 = f(y2), y2 = y + hh k1
    rhs_vjp7(y2, E, L, a, M, lk2, g, gc);
    vjp_accum7(g, hh, k1, ly, lk1, l_hh);
    // k1 = f(y)
    rhs_vjp7(y, E, L, a, M, lk1, g, gc);
    for (int i = 0; i < 7; ++i) ly[sidx(i)] += g[sidx(i)];
    // he = h ps(s), hh = he / 2
    ly[6] += (l_he + T(0.5) * l_hh) * dhd;
    for (int i = 0; i < 8; ++i) lam[i] = ly[i];
}

}  // namespace sgxa
