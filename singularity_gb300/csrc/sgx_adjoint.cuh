// singularity_gb300/csrc/sgx_adjoint.cuh
//
// Reverse-mode (vector-Jacobian) products of the Kerr Hamiltonian right-hand
// side and of one fixed RK4 step with the reference's pole damping
// (kerr_hamilton.h:97-178), derived by hand: given the adjoint of a step's
// output, they return the adjoint of its input state and of the constants
// (E, L_z, a).  The adjoint sweep of sgx_diff.cu multiplies by these instead
// of building the step's 6 x 9 Jacobian with dual numbers: four right-hand
// side evaluations and four reverse passes per step instead of nine-lane
// dual arithmetic.
//
// Host-and-device code (plain arithmetic, sinf/cosf/sqrtf overloads), so the
// derivatives can be checked against finite differences on the CPU.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define SGX_HD __host__ __device__ __forceinline__
// The right-hand side and its reverse pass are called four times per step;
// one out-of-line copy each keeps the adjoint kernel inside the
// instruction cache.
#define SGX_HD_CALL __host__ __device__ __noinline__
#else
#define SGX_HD inline
#define SGX_HD_CALL inline
#endif

namespace sgxa {

SGX_HD float hsin(float x) { return sinf(x); }
SGX_HD float hcos(float x) { return cosf(x); }
SGX_HD float hsqrt(float x) { return sqrtf(x); }
SGX_HD double hsin(double x) { return sin(x); }
SGX_HD double hcos(double x) { return cos(x); }
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
// sine and cosine from one range reduction on the device
SGX_HD void hsincos(float x, float* s, float* c) {
#if defined(__CUDA_ARCH__)
    sincosf(x, s, c);
#else
    *s = sinf(x);
    *c = cosf(x);
#endif
}
SGX_HD void hsincos(double x, double* s, double* c) {
#if defined(__CUDA_ARCH__)
    sincos(x, s, c);
#else
    *s = sin(x);
    *c = cos(x);
#endif
}

// State layout: y[0..5] = r, theta, phi, p_r, p_theta, psi (swept angle);
// derivative layout d[0..4] = dr, dtheta, dphi, dp_r, dp_theta.

// The right-hand side in Carter's separated form (the same Hamiltonian as
// kerr_hamilton.h:97-155): with P = (r^2 + a^2) E - a L, W = L - a E s2,
// Q = P / Delta, U = W / s2 and N = 2 Sigma H = Delta p_r^2 + p_th^2 - P Q + W U,
//   dr = Delta p_r / Sigma, dth = p_th / Sigma, dphi = (a Q + U) / Sigma,
//   dp_r  = (r N / Sigma + (M - r)(p_r^2 + Q^2) + 2 E r Q) / Sigma,
//   dp_th = -sin(th) cos(th) (a^2 N / Sigma - U (2 a E + U)) / Sigma.
// Operation for operation the forward kernel's rhs_g (sgx_diff_impl.cuh).
template <class T>
SGX_HD_CALL void rhs_sc(const T* y, T st, T ct, T E, T L, T a, T M, T* d) {
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
}

template <class T> SGX_HD void rhs(const T* y, T E, T L, T a, T M, T* d) {
    T st, ct;
    hsincos(y[1], &st, &ct);
    rhs_sc(y, st, ct, E, L, a, M, d);
}

// w . d(rhs)/d(r, theta, p_r, p_theta, E, L, a), w the adjoint of d[0..4],
// with st, ct = sin, cos of y[1].  gy[0..4] receives the state part (gy[2] = 0:
// the right-hand side does not depend on phi); gc[0..2] += the constants' part.
template <class T>
SGX_HD_CALL void rhs_vjp_sc(const T* y, T st, T ct, T E, T L, T a, T M, const T* w, T* gy, T* gc) {
    // forward intermediates
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

    // reverse: d0 = Del pr iS, d1 = pth iS, d2 = C2 iS, d3 = A3 iS, d4 = -(iS sc) B4
    const T w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3], w4 = w[4];
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
    // sc = st ct ; c2 = ct^2 ; s2 = st^2 ; st, ct of theta
    const T st_b = sc_b * ct + T(2) * st * s2_b;
    const T ct_b = sc_b * st + T(2) * ct * c2_b;

    gy[0] = r_b;
    gy[1] = st_b * ct - ct_b * st;
    gy[2] = T(0);
    gy[3] = pr_b;
    gy[4] = pth_b;
    gc[0] += E_b;
    gc[1] += L_b;
    gc[2] += a_b;
}

template <class T> SGX_HD void rhs_vjp(const T* y, T E, T L, T a, T M, const T* w, T* gy, T* gc) {
    T st, ct;
    hsincos(y[1], &st, &ct);
    rhs_vjp_sc(y, st, ct, E, L, a, M, w, gy, gc);
}

// Pole-damped step length h * clamp(5 |sin(theta)|, 0.05, 1) and its theta
// derivative (kerr_hamilton.h:165-178).
template <class T> SGX_HD T damped_h_sc(T h, T s, T c, T* dh_dth) {
    const T as = s < T(0) ? -s : s;
    T ps = as * T(5);
    T dps = (s < T(0) ? T(-5) : T(5)) * c;
    if (ps > T(1)) {
        ps = T(1);
        dps = T(0);
    } else if (ps < T(0.05)) {
        ps = T(0.05);
        dps = T(0);
    }
    *dh_dth = h * dps;
    return h * ps;
}
template <class T> SGX_HD T damped_h(T h, T th, T* dh_dth) {
    T s, c;
    hsincos(th, &s, &c);
    return damped_h_sc(h, s, c, dh_dth);
}

// One RK4 step y -> o (with the swept angle when `fade`).
template <class T> SGX_HD void step(const T* y, T E, T L, T a, T M, T h, bool fade, T* o) {
    T dhd;
    const T he = damped_h(h, y[1], &dhd);
    const T hh = T(0.5) * he;
    T k1[5], k2[5], k3[5], k4[5], t[5];
    rhs(y, E, L, a, M, k1);
    for (int i = 0; i < 5; ++i) t[i] = y[i] + k1[i] * hh;
    rhs(t, E, L, a, M, k2);
    for (int i = 0; i < 5; ++i) t[i] = y[i] + k2[i] * hh;
    rhs(t, E, L, a, M, k3);
    for (int i = 0; i < 5; ++i) t[i] = y[i] + k3[i] * he;
    rhs(t, E, L, a, M, k4);
    const T h6 = he / T(6);
    for (int i = 0; i < 5; ++i) o[i] = y[i] + ((k1[i] + k2[i] * T(2)) + (k3[i] * T(2) + k4[i])) * h6;
    if (fade) {
        const T dth = o[1] - y[1], dph = o[2] - y[2], s = hsin(o[1]);
        o[5] = y[5] + hsqrt(dth * dth + s * s * dph * dph);
    } else {
        o[5] = y[5];
    }
}

// Adjoint of one step: lam (adjoint of the step's output, 6 components) is
// replaced by the adjoint of its input; gc[0..2] += the step's terms of
// dLoss/d(E, L, a).
template <class T> SGX_HD void step_vjp(const T* y, T E, T L, T a, T M, T h, bool fade, T* lam, T* gc) {
    // sin, cos of each stage's theta, shared by its right-hand side and reverse pass
    T s1, c1, s2, c2, s3, c3, s4, c4;
    hsincos(y[1], &s1, &c1);
    T dhd;
    const T he = damped_h_sc(h, s1, c1, &dhd);
    const T hh = T(0.5) * he;
    T k1[5], k2[5], k3[5], k4[5], y2[6], y3[6], y4[6];
    rhs_sc(y, s1, c1, E, L, a, M, k1);
    for (int i = 0; i < 5; ++i) y2[i] = y[i] + k1[i] * hh;
    hsincos(y2[1], &s2, &c2);
    rhs_sc(y2, s2, c2, E, L, a, M, k2);
    for (int i = 0; i < 5; ++i) y3[i] = y[i] + k2[i] * hh;
    hsincos(y3[1], &s3, &c3);
    rhs_sc(y3, s3, c3, E, L, a, M, k3);
    for (int i = 0; i < 5; ++i) y4[i] = y[i] + k3[i] * he;
    hsincos(y4[1], &s4, &c4);
    rhs_sc(y4, s4, c4, E, L, a, M, k4);
    const T h6 = he / T(6);
    T lo[5];
    for (int i = 0; i < 5; ++i) lo[i] = lam[i];
    T ly[6];
    ly[5] = lam[5];
    // swept angle: o5 = y5 + sqrt(dth^2 + sin^2(o1) dph^2)
    T l_y1_psi = T(0), l_y2_psi = T(0);
    if (fade && lam[5] != T(0)) {
        T o1 = y[1], o2 = y[2];
        {
            const T s1 = (k1[1] + k2[1] * T(2)) + (k3[1] * T(2) + k4[1]);
            const T s2 = (k1[2] + k2[2] * T(2)) + (k3[2] * T(2) + k4[2]);
            o1 = y[1] + s1 * h6;
            o2 = y[2] + s2 * h6;
        }
        const T dth = o1 - y[1], dph = o2 - y[2];
        T s, c;
        hsincos(o1, &s, &c);
        const T q = hsqrt(dth * dth + s * s * dph * dph);
        if (q > T(0)) {
            const T iq = lam[5] / q;
            lo[1] += iq * (dth + s * c * dph * dph);
            lo[2] += iq * s * s * dph;
            l_y1_psi = -iq * dth;
            l_y2_psi = -iq * s * s * dph;
        }
    }
    // o = y + (k1 + 2 k2 + 2 k3 + k4) h6
    T lk1[5], lk2[5], lk3[5], lk4[5];
    T l_he = T(0);
    for (int i = 0; i < 5; ++i) {
        ly[i] = lo[i];
        lk1[i] = lo[i] * h6;
        lk2[i] = lo[i] * (T(2) * h6);
        lk3[i] = lo[i] * (T(2) * h6);
        lk4[i] = lo[i] * h6;
        l_he += lo[i] * ((k1[i] + k2[i] * T(2)) + (k3[i] * T(2) + k4[i]));
    }
    l_he *= T(1) / T(6);
    ly[1] += l_y1_psi;
    ly[2] += l_y2_psi;
    T g[5];
    // k4 = f(y4), y4 = y + he k3
    rhs_vjp_sc(y4, s4, c4, E, L, a, M, lk4, g, gc);
    for (int i = 0; i < 5; ++i) {
        ly[i] += g[i];
        lk3[i] += he * g[i];
        l_he += g[i] * k3[i];
    }
    T l_hh = T(0);
    // k3 = f(y3), y3 = y + hh k2
    rhs_vjp_sc(y3, s3, c3, E, L, a, M, lk3, g, gc);
    for (int i = 0; i < 5; ++i) {
        ly[i] += g[i];
        lk2[i] += hh * g[i];
        l_hh += g[i] * k2[i];
    }
    // k2 = f(y2), y2 = y + hh k1
    rhs_vjp_sc(y2, s2, c2, E, L, a, M, lk2, g, gc);
    for (int i = 0; i < 5; ++i) {
        ly[i] += g[i];
        lk1[i] += hh * g[i];
        l_hh += g[i] * k1[i];
    }
    // k1 = f(y)
    rhs_vjp_sc(y, s1, c1, E, L, a, M, lk1, g, gc);
    for (int i = 0; i < 5; ++i) ly[i] += g[i];
    // he = h ps(theta), hh = he / 2
    ly[1] += (l_he + T(0.5) * l_hh) * dhd;
    for (int i = 0; i < 6; ++i) lam[i] = ly[i];
}

}  // namespace sgxa
