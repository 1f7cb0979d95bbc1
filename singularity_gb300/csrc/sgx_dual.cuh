// singularity_gb300/csrc/sgx_dual.cuh
//
// Forward-mode dual numbers for the adjoint kernels: a value and N partial
// derivatives, with the arithmetic and the scalar functions the tracer's
// formulas use.  Evaluating a step, a crossing or the camera set-up once on
// Dual<T, N> inputs seeded with unit partials yields its Jacobian; the
// reverse (adjoint) sweep in sgx_diff.cu multiplies those local Jacobians by
// the adjoint vector.  Also specialises the tracer's scalar traits (DM) so the
// shading templates of sgx_device.cuh run unchanged on duals.
#pragma once

#include <cuda_runtime.h>

#include "sgx_device.cuh"

namespace sgxd {

template <class T, int N> struct Dual {
    T v;
    T d[N];
    __device__ __forceinline__ Dual() {}
    __device__ __forceinline__ Dual(T x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = T(0);
    }
    // Independent variable number k (unit partial).
    __device__ __forceinline__ static Dual var(T x, int k) {
        Dual r(x);
        if (k >= 0 && k < N) r.d[k] = T(1);
        return r;
    }
};

#define SGX_DUAL_T template <class T, int N>
SGX_DUAL_T __device__ __forceinline__ Dual<T, N> operator+(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
SGX_DUAL_T __device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
SGX_DUAL_T __device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N>& a) {
    Dual<T, N> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
SGX_DUAL_T __device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
SGX_DUAL_T __device__ __forceinline__ Dual<T, N> operator/(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    const T ib = T(1) / b.v;
    r.v = a.v * ib;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
SGX_DUAL_T __device__ __forceinline__ bool operator<(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v < b.v; }
SGX_DUAL_T __device__ __forceinline__ bool operator>(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v > b.v; }
SGX_DUAL_T __device__ __forceinline__ bool operator<=(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v <= b.v; }
SGX_DUAL_T __device__ __forceinline__ bool operator>=(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v >= b.v; }

// f(a) with f(a.v) = fv and f'(a.v) = dfv
SGX_DUAL_T __device__ __forceinline__ Dual<T, N> chain(const Dual<T, N>& a, T fv, T dfv) {
    Dual<T, N> r;
    r.v = fv;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = dfv * a.d[i];
    return r;
}
#undef SGX_DUAL_T

template <class T, int N> struct DM<Dual<T, N>> {
    using D = Dual<T, N>;
    static __device__ __forceinline__ D lit(float f, double d) { return D(DM<T>::lit(f, d)); }
    static __device__ __forceinline__ D sqrt_(const D& x) {
        const T s = DM<T>::sqrt_(x.v);
        return chain(x, s, s > T(0) ? T(0.5) / s : T(0));
    }
    static __device__ __forceinline__ D sin_(const D& x) { return chain(x, DM<T>::sin_(x.v), DM<T>::cos_(x.v)); }
    static __device__ __forceinline__ D cos_(const D& x) { return chain(x, DM<T>::cos_(x.v), -DM<T>::sin_(x.v)); }
    static __device__ __forceinline__ void sincos_(const D& x, D* s, D* c) {
        T sv, cv;
        DM<T>::sincos_(x.v, &sv, &cv);
        *s = chain(x, sv, cv);
        *c = chain(x, cv, -sv);
    }
    static __device__ __forceinline__ D acos_(const D& x) {
        const T q = T(1) - x.v * x.v;
        return chain(x, DM<T>::acos_(x.v), q > T(0) ? -T(1) / DM<T>::sqrt_(q) : T(0));
    }
    // x^y with a constant exponent (every use in the shading has one).
    static __device__ __forceinline__ D pow_(const D& x, const D& y) {
        const T p = DM<T>::pow_(x.v, y.v);
        return chain(x, p, x.v != T(0) ? y.v * p / x.v : T(0));
    }
    static __device__ __forceinline__ D log_(const D& x) { return chain(x, DM<T>::log_(x.v), T(1) / x.v); }
    static __device__ __forceinline__ D exp_(const D& x) {
        const T e = DM<T>::exp_(x.v);
        return chain(x, e, e);
    }
    static __device__ __forceinline__ D fmin_(const D& a, const D& b) { return (b.v < a.v) ? b : a; }
    static __device__ __forceinline__ D fmax_(const D& a, const D& b) { return (b.v > a.v) ? b : a; }
    static __device__ __forceinline__ D rcp_(const D& x) { return D(T(1)) / x; }
    static __device__ __forceinline__ D rcp_fast(const D& x) { return D(T(1)) / x; }
};

template <class T> __device__ __forceinline__ T value_of(const T& x) { return x; }
template <class T, int N> __device__ __forceinline__ T value_of(const Dual<T, N>& x) { return x.v; }

}  // namespace sgxd
