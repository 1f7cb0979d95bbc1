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

// State layout: y[0..5] = r, theta, phi, p_r, p_theta, psi (swept angle);
// derivative layout d[0..4] = dr, dtheta, dphi, dp_r, dp_theta.

// The right-hand side in the shared-reciprocal algebra.
template <class T>
SGX_HD_CALL void rhs(const T* y, T E, T L, T a, T M, T* d) {
    const T st = hsin(y[1]), ct = hcos(y[1]);
    const T r = y[0], pr = y[3], pth = y[4];
    const T a2 = a * a, s2 = st * st, c2 = ct * ct, r2 = r * r;
    const T ss = s2 < T(1e-10) ? T(1e-10) : s2;
    const T r2a2 = r2 + a2;
    const T Sig = r2 + a2 * c2;
    const T Dr = T(2) * (r - M);
    const T Del = r * (r - T(2) * M) + a2;
    const T a2s2 = a2 * s2;
    const T A = r2a2 * r2a2 - a2s2 * Del;
    const T iS = T(1) / Sig, iD = T(1) / Del, is2 = T(1) / ss;
    const T iSD = iS * iD, iS2 = iS * iS;
    const T E2 = E * E, L2 = L * L;
    const T cEL = T(4) * M * a * E * L;
    const T aL2 = a2 * L2;
    const T tMaE = T(2) * M * a * E;
    d[2] = (tMaE * r * s2 + (Del - a2s2) * L) * iSD * is2;
    d[0] = Del * pr * iS;
    d[1] = pth * iS;
    const T B = (cEL * r - A * E2) - aL2;
    const T Ar = T(4) * r * r2a2 - a2s2 * Dr;
    const T Br = cEL - Ar * E2;
    const T s2t = T(2) * st * ct;
    const T St = -a2 * s2t;
    const T pr2 = pr * pr;
    const T Dp2 = Del * pr2 + pth * pth;
    const T tr = T(2) * r;
    const T Hr = iSD * (Br - B * (tr * Del + Sig * Dr) * iSD) + Dr * pr2 * iS - tr * iS2 * (L2 * is2 + Dp2);
    const T Ht = iSD * (a2 * Del * s2t * E2) - B * St * iS2 * iD - iS2 * (L2 * is2 * (St + Sig * s2t * is2) + Dp2 * St);
    d[3] = T(-0.5) * Hr;
    d[4] = T(-0.5) * Ht;
}

// w . d(rhs)/d(r, theta, p_r, p_theta, E, L, a), w the adjoint of d[0..4].
// gy[0..4] receives the state part (gy[2] = 0: the right-hand side does not
// depend on phi); gc[0..2] += the constants' part.
template <class T>
SGX_HD_CALL void rhs_vjp(const T* y, T E, T L, T a, T M, const T* w, T* gy, T* gc) {
    // forward intermediates
    const T th = y[1];
    const T st = hsin(th), ct = hcos(th);
    const T r = y[0], pr = y[3], pth = y[4];
    const T a2 = a * a, s2 = st * st, c2 = ct * ct, r2 = r * r;
    const bool s2_free = !(s2 < T(1e-10));
    const T ss = s2_free ? s2 : T(1e-10);
    const T r2a2 = r2 + a2;
    const T Sig = r2 + a2 * c2;
    const T Dr = T(2) * (r - M);
    const T Del = r * (r - T(2) * M) + a2;
    const T a2s2 = a2 * s2;
    const T A = r2a2 * r2a2 - a2s2 * Del;
    const T iS = T(1) / Sig, iD = T(1) / Del, is2 = T(1) / ss;
    const T iSD = iS * iD, iS2 = iS * iS;
    const T E2 = E * E, L2 = L * L;
    const T cEL = T(4) * M * a * E * L;
    const T tMaE = T(2) * M * a * E;
    const T P = tMaE * r * s2 + (Del - a2s2) * L;
    const T B = (cEL * r - A * E2) - a2 * L2;
    const T Ar = T(4) * r * r2a2 - a2s2 * Dr;
    const T Br = cEL - Ar * E2;
    const T s2t = T(2) * st * ct;
    const T St = -a2 * s2t;
    const T pr2 = pr * pr;
    const T Dp2 = Del * pr2 + pth * pth;
    const T tr = T(2) * r;
    const T G = tr * Del + Sig * Dr;
    const T X = Br - B * G * iSD;
    const T Y = L2 * is2 + Dp2;
    const T U = a2 * Del * s2t * E2;
    const T W = St + Sig * s2t * is2;
    const T V = L2 * is2 * W + Dp2 * St;

    // reverse
    const T w_r = w[0], w_th = w[1], w_ph = w[2];
    const T Hr_b = T(-0.5) * w[3], Ht_b = T(-0.5) * w[4];
    // Ht = iSD U - B St iS2 iD - iS2 V
    T iSD_b = Ht_b * U;
    const T U_b = Ht_b * iSD;
    T B_b = -Ht_b * St * iS2 * iD;
    T St_b = -Ht_b * B * iS2 * iD;
    T iS2_b = -Ht_b * B * St * iD - Ht_b * V;
    T iD_b = -Ht_b * B * St * iS2;
    const T V_b = -Ht_b * iS2;
    // V = L2 is2 W + Dp2 St
    T L2_b = V_b * is2 * W;
    T is2_b = V_b * L2 * W;
    const T W_b = V_b * L2 * is2;
    T Dp2_b = V_b * St;
    St_b += V_b * Dp2;
    // W = St + Sig s2t is2
    St_b += W_b;
    T Sig_b = W_b * s2t * is2;
    T s2t_b = W_b * Sig * is2;
    is2_b += W_b * Sig * s2t;
    // U = a2 Del s2t E2
    T a2_b = U_b * Del * s2t * E2;
    T Del_b = U_b * a2 * s2t * E2;
    s2t_b += U_b * a2 * Del * E2;
    T E2_b = U_b * a2 * Del * s2t;
    // Hr = iSD X + Dr pr2 iS - tr iS2 Y
    iSD_b += Hr_b * X;
    const T X_b = Hr_b * iSD;
    T Dr_b = Hr_b * pr2 * iS;
    T pr2_b = Hr_b * Dr * iS;
    T iS_b = Hr_b * Dr * pr2;
    T tr_b = -Hr_b * iS2 * Y;
    iS2_b += -Hr_b * tr * Y;
    const T Y_b = -Hr_b * tr * iS2;
    // Y = L2 is2 + Dp2
    L2_b += Y_b * is2;
    is2_b += Y_b * L2;
    Dp2_b += Y_b;
    // X = Br - B G iSD
    const T Br_b = X_b;
    B_b += -X_b * G * iSD;
    const T G_b = -X_b * B * iSD;
    iSD_b += -X_b * B * G;
    // G = tr Del + Sig Dr
    tr_b += G_b * Del;
    Del_b += G_b * tr;
    Sig_b += G_b * Dr;
    Dr_b += G_b * Sig;
    // Dp2 = Del pr2 + pth^2
    Del_b += Dp2_b * pr2;
    pr2_b += Dp2_b * Del;
    T pth_b = T(2) * pth * Dp2_b;
    T pr_b = T(2) * pr * pr2_b;
    // St = -a2 s2t ; s2t = 2 st ct
    a2_b += -St_b * s2t;
    s2t_b += -St_b * a2;
    T st_b = T(2) * ct * s2t_b;
    T ct_b = T(2) * st * s2t_b;
    // Br = cEL - Ar E2 ; Ar = 4 r r2a2 - a2s2 Dr
    T cEL_b = Br_b;
    const T Ar_b = -Br_b * E2;
    E2_b += -Br_b * Ar;
    T r_b = T(4) * r2a2 * Ar_b;
    T r2a2_b = T(4) * r * Ar_b;
    T a2s2_b = -Ar_b * Dr;
    Dr_b += -Ar_b * a2s2;
    // B = cEL r - A E2 - a2 L2
    cEL_b += B_b * r;
    r_b += B_b * cEL;
    const T A_b = -B_b * E2;
    E2_b += -B_b * A;
    a2_b += -B_b * L2;
    L2_b += -B_b * a2;
    // dth = pth iS ; dr = Del pr iS
    pth_b += w_th * iS;
    iS_b += w_th * pth + w_r * Del * pr;
    Del_b += w_r * pr * iS;
    pr_b += w_r * Del * iS;
    // dph = P iSD is2 ; P = tMaE r s2 + (Del - a2s2) L
    const T P_b = w_ph * iSD * is2;
    iSD_b += w_ph * P * is2;
    is2_b += w_ph * P * iSD;
    const T tMaE_b = P_b * r * s2;
    r_b += P_b * tMaE * s2;
    T s2_b = P_b * tMaE * r;
    Del_b += P_b * L;
    a2s2_b += -P_b * L;
    T L_b = P_b * (Del - a2s2);
    // constants: tMaE = 2 M a E ; cEL = 4 M a E L ; E2, L2
    T a_b = tMaE_b * T(2) * M * E + cEL_b * T(4) * M * E * L;
    T E_b = tMaE_b * T(2) * M * a + cEL_b * T(4) * M * a * L + T(2) * E * E2_b;
    L_b += cEL_b * T(4) * M * a * E + T(2) * L * L2_b;
    // iSD = iS iD ; iS2 = iS^2 ; reciprocals
    iS_b += iSD_b * iD + T(2) * iS * iS2_b;
    iD_b += iSD_b * iS;
    Sig_b += -iS_b * iS * iS;
    Del_b += -iD_b * iD * iD;
    if (s2_free) s2_b += -is2_b * is2 * is2;
    // A = r2a2^2 - a2s2 Del ; a2s2 = a2 s2
    r2a2_b += T(2) * r2a2 * A_b;
    a2s2_b += -A_b * Del;
    Del_b += -A_b * a2s2;
    a2_b += a2s2_b * s2;
    s2_b += a2s2_b * a2;
    // Del = r (r - 2M) + a2 ; Dr = 2 (r - M) ; tr = 2 r
    r_b += Del_b * Dr + T(2) * Dr_b + T(2) * tr_b;
    a2_b += Del_b;
    // Sig = r2 + a2 c2 ; r2a2 = r2 + a2 ; r2 = r^2
    T r2_b = Sig_b + r2a2_b;
    a2_b += Sig_b * c2 + r2a2_b;
    const T c2_b = Sig_b * a2;
    r_b += T(2) * r * r2_b;
    // c2 = ct^2 ; s2 = st^2 ; st, ct of theta
    ct_b += T(2) * ct * c2_b;
    st_b += T(2) * st * s2_b;
    a_b += T(2) * a * a2_b;

    gy[0] = r_b;
    gy[1] = st_b * ct - ct_b * st;
    gy[2] = T(0);
    gy[3] = pr_b;
    gy[4] = pth_b;
    gc[0] += E_b;
    gc[1] += L_b;
    gc[2] += a_b;
}

// Pole-damped step length h * clamp(5 |sin(theta)|, 0.05, 1) and its theta
// derivative (kerr_hamilton.h:165-178).
template <class T> SGX_HD T damped_h(T h, T th, T* dh_dth) {
    const T s = hsin(th);
    const T as = s < T(0) ? -s : s;
    T ps = as * T(5);
    T dps = (s < T(0) ? T(-5) : T(5)) * hcos(th);
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
    T dhd;
    const T he = damped_h(h, y[1], &dhd);
    const T hh = T(0.5) * he;
    T k1[5], k2[5], k3[5], k4[5], y2[6], y3[6], y4[6];
    rhs(y, E, L, a, M, k1);
    for (int i = 0; i < 5; ++i) y2[i] = y[i] + k1[i] * hh;
    rhs(y2, E, L, a, M, k2);
    for (int i = 0; i < 5; ++i) y3[i] = y[i] + k2[i] * hh;
    rhs(y3, E, L, a, M, k3);
    for (int i = 0; i < 5; ++i) y4[i] = y[i] + k3[i] * he;
    rhs(y4, E, L, a, M, k4);
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
        const T s = hsin(o1), c = hcos(o1);
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
    rhs_vjp(y4, E, L, a, M, lk4, g, gc);
    for (int i = 0; i < 5; ++i) {
        ly[i] += g[i];
        lk3[i] += he * g[i];
        l_he += g[i] * k3[i];
    }
    T l_hh = T(0);
    // k3 = f(y3), y3 = y + hh k2
    rhs_vjp(y3, E, L, a, M, lk3, g, gc);
    for (int i = 0; i < 5; ++i) {
        ly[i] += g[i];
        lk2[i] += hh * g[i];
        l_hh += g[i] * k2[i];
    }
    // k2 = f(y2), y2 = y + hh k1
    rhs_vjp(y2, E, L, a, M, lk2, g, gc);
    for (int i = 0; i < 5; ++i) {
        ly[i] += g[i];
        lk1[i] += hh * g[i];
        l_hh += g[i] * k1[i];
    }
    // k1 = f(y)
    rhs_vjp(y, E, L, a, M, lk1, g, gc);
    for (int i = 0; i < 5; ++i) ly[i] += g[i];
    // he = h ps(theta), hh = he / 2
    ly[1] += (l_he + T(0.5) * l_hh) * dhd;
    for (int i = 0; i < 6; ++i) lam[i] = ly[i];
}

}  // namespace sgxa
