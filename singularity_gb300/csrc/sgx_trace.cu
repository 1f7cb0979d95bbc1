// singularity_gb300/csrc/sgx_trace.cu
//
// Kernels of the geodesic tracer for sm_103a.
//
// The reference launches one thread per pixel and traces the pixel's samples
// one after another (geodesic_kernel.cu:462-510); a warp then runs as long as
// its slowest ray, and ray lengths span 1 to thousands of steps.  Here the
// unit of work is one (pixel, sample) ray taken from a global queue by a
// persistent kernel:
//   * each warp keeps 32 rays in registers; every `refill` steps the lanes
//     whose ray has ended are found with a ballot, their results are shaded
//     and stored, and one atomic per warp hands them the next ray ids;
//   * ray id = pixel * S + sample, so fresh warps start on neighbouring rays;
//   * a finished ray leaves a 16-byte hit record (where it crossed the disc
//     or which direction it escaped in, and how it ended) in a [S][npix]
//     buffer; the ordered pass then shades each record, tone-maps it and sums
//     a pixel's samples in sample order — the reference's accumulation order —
//     so colour work runs converged, once per sample, outside the step loop,
//     and results do not depend on which warp traced which sample;
//   * view constants and the pass's Halton offsets live in shared memory (a
//     single-view pass takes its view as a kernel parameter instead).
// All loops are bounded: a ray ends after max_steps integrator steps, and the
// queue is a single counter that only grows.

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <type_traits>

#include "sgx_device.cuh"
#include "sgx_kernels.hpp"

namespace sgxk {

using namespace sgxd;

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <class T> __device__ __forceinline__ bool finite_(T x) { return isfinite(x); }

// ---------------------------------------------------------------------------
// Ray policies: the state each lane keeps and one loop iteration of the
// reference (checks on the current state, then one step).
// ---------------------------------------------------------------------------

// Hit record of one finished ray: (t0, t1, t2) and meta = term | steps << 3.
//   disc (Kerr):          r_cross, phi, L_z
//   disc (Schwarzschild): r_cross, phi, u^phi at the crossing
//   escape:               theta, phi
template <class T> struct alignas(4 * sizeof(T)) Rec {
    T t0, t1, t2;
    std::uint32_t meta;
};

__device__ __forceinline__ std::uint32_t pack_meta(std::uint32_t term, std::uint32_t steps) {
    return term | ((steps < 0x1FFFFFFFu ? steps : 0x1FFFFFFFu) << 3);
}

// Policy flags: bit 0 = separated-form Kerr RHS, bit 1 = mixed precision.
constexpr int FL_FAST = 1;    // separated-form Kerr RHS
constexpr int FL_SC = 4;      // fixed step: sin/cos of theta carried in the state
constexpr int FL_MIXED = 2;
// error-controlled form: the Carter projection taken from PassDesc::project at
// run time (the probes) instead of always (the render kernels)
constexpr int FL_RTPROJ = 8;
// error-controlled form: one range test per step, r_slow <= r <= escape_r,
// stands for the capture, horizon, escape and FP64-zone tests, which run only
// outside it (the multi-view kernels: it frees the registers of the early
// capture radius, 78 -> 72 in FP32, +2.4 % on the 64 batched views; the
// single-view kernel, whose view constants are instruction operands, runs
// 1.5 % slower with it, so it keeps the direct tests).  Same decisions, so
// the same frames bit for bit.
constexpr int FL_RANGE = 16;

// Kerr, fixed step (geodesic_kernel.cu:303-403).
template <class T, int FL> struct KerrFixed {
    static constexpr int kMinBlocks = sizeof(T) == 4 ? 4 : 1;
    static constexpr int kMinBlocksMulti = kMinBlocks;
    static constexpr bool FAST = (FL & FL_FAST) != 0;
    static constexpr bool SC = (FL & FL_SC) != 0;
    static constexpr int FORM = FAST ? RHS_SEP : RHS_REF;
    KS<T> y;
    KC<T> c;
    T prev_th, prev_r;
    T s_th, c_th;  // SC: sin, cos of theta
    T t0, t1, t2;  // termination data: (r_cross, phi, T_local) or (theta, phi)
    std::uint32_t steps, term;
    static constexpr std::uint32_t rej = 0, zone = 0;

    __device__ __forceinline__ bool init(const View<T>& v, const CamDir<T>& cd, const PassDesc&) {
        steps = 0;
        T E, L;
        if (!kerr_init(v, cd, y, E, L)) {
            term = TERM_NO_ROOT;
            return false;
        }
        c = make_kc(v, E, L);
        prev_th = y.th;
        prev_r = y.r;
        if constexpr (SC) {
            s_th = v.sin_th;
            c_th = v.cos_th;
        }
        if (v.max_steps == 0u) {
            term = TERM_BUDGET;
            return false;
        }
        return true;
    }

    // Returns true when the ray has ended.
    __device__ __forceinline__ bool step(const View<T>& v, const PassDesc&) {
        if (!finite_(y.r) || y.r < v.hcut) {
            term = TERM_HORIZON;
            return true;
        }
        if (y.r > v.escape_r) {
            term = TERM_ESCAPE;
            if constexpr (SC) {
                t0 = s_th;
                t2 = c_th;
            } else {
                t0 = DM<T>::sin_(y.th);
                t2 = DM<T>::cos_(y.th);
            }
            t1 = y.ph;
            return true;
        }
        T frac;
        if ((v.flags & SGX_FLAG_DISC_ON) && crossed_equator(prev_th, y.th, frac)) {
            const T r_cross = prev_r + frac * (y.r - prev_r);
            if (r_cross >= v.r_in && r_cross <= v.r_out) {
                const T T_local = disc_temperature(r_cross, v.r_in, v.peak_T);
                term = T_local > DLIT(0.0) ? TERM_DISC : TERM_DISC_COLD;
                t0 = r_cross;
                t1 = y.ph;
                t2 = c.L;
                return true;
            }
        }
        prev_th = y.th;
        prev_r = y.r;
        if constexpr (SC) y = kerr_rk4_sc(y, s_th, c_th, fixed_step_h(v, y.r), v, c);
        else y = kerr_rk4<T, FORM>(y, fixed_step_h(v, y.r), v, c);
        if (++steps >= v.max_steps) {
            term = TERM_BUDGET;
            return true;
        }
        return false;
    }

    __device__ __forceinline__ Rec<T> record() const { return Rec<T>{t0, t1, t2, pack_meta(term, steps)}; }
};

// Schwarzschild, fixed step (geodesic_kernel.cu:229-297).
template <class T, int FL> struct SchwFixed {
    static constexpr int kMinBlocks = sizeof(T) == 4 ? 4 : 1;
    static constexpr int kMinBlocksMulti = kMinBlocks;
    SS<T> y;
    T prev_th, prev_r, prev_uph;
    T t0, t1, t2;
    std::uint32_t steps, term;
    static constexpr std::uint32_t rej = 0, zone = 0;

    __device__ __forceinline__ bool init(const View<T>& v, const CamDir<T>& cd, const PassDesc&) {
        steps = 0;
        y = schw_init(v, cd);
        prev_th = y.th;
        prev_r = y.r;
        prev_uph = y.uph;
        if (v.max_steps == 0u) {
            term = TERM_BUDGET;
            return false;
        }
        return true;
    }

    __device__ __forceinline__ bool step(const View<T>& v, const PassDesc&) {
        if (!finite_(y.r) || y.r < v.hcut) {
            term = TERM_HORIZON;
            return true;
        }
        if (y.r > v.escape_r) {
            term = TERM_ESCAPE;
            t0 = DM<T>::sin_(y.th);
            t1 = y.ph;
            t2 = DM<T>::cos_(y.th);
            return true;
        }
        T frac;
        if ((v.flags & SGX_FLAG_DISC_ON) && crossed_equator(prev_th, y.th, frac)) {
            const T r_cross = prev_r + frac * (y.r - prev_r);
            const T uph_cross = prev_uph + frac * (y.uph - prev_uph);
            if (r_cross >= v.r_in && r_cross <= v.r_out) {
                const T T_local = disc_temperature(r_cross, v.r_in, v.peak_T);
                term = T_local > DLIT(0.0) ? TERM_DISC : TERM_DISC_COLD;
                t0 = r_cross;
                // phi_cross = lerp(phi, phi, frac) in the reference (geodesic_kernel.cu:282)
                t1 = y.ph + frac * (y.ph - y.ph);
                t2 = uph_cross;
                return true;
            }
        }
        prev_th = y.th;
        prev_r = y.r;
        prev_uph = y.uph;
        y = schw_rk4(y, fixed_step_h(v, y.r), v.rs);
        if (++steps >= v.max_steps) {
            term = TERM_BUDGET;
            return true;
        }
        return false;
    }

    __device__ __forceinline__ Rec<T> record() const { return Rec<T>{t0, t1, t2, pack_meta(term, steps)}; }
};

// Kerr, error-controlled RK4 with the FSAL third-order estimate (the adaptive
// extension; oracle/adaptive_oracle.hpp is its specification).  One call of
// step() is one attempt; max_steps bounds the attempts.
template <class T, int FL> struct KerrAdaptive {
    static constexpr bool FAST = (FL & FL_FAST) != 0;
    static constexpr int FORM = FAST ? RHS_SEP : RHS_REF;
    static constexpr bool MIXED = (FL & FL_MIXED) != 0;
    static constexpr bool RTPROJ = (FL & FL_RTPROJ) != 0;
    static constexpr bool RANGE = (FL & FL_RANGE) != 0;
    static constexpr int kMinBlocks = sizeof(T) == 4 ? 4 : 1;
    // Multi-view passes hold their view's constants in shared memory and
    // registers rather than the constant bank: 80 registers (3 blocks) beat
    // 64 with spills there (1954 against 1877 Mrays/s on six 4K views).
    static constexpr int kMinBlocksMulti = sizeof(T) == 4 ? 3 : 1;
    KSC<T> y, k1;  // theta carried as (sin theta, cos theta)
    KC<T> c;
    T Q;           // Carter constant the projection holds p_theta to
    T h, r_c;
    // early capture: inside min(r_c - 0.05 M, r_in) moving inward (0: never);
    // RANGE: r_cap holds r_slow, the radius at and above which (inside
    // escape_r) no capture, horizon cut or FP64 zone applies, and r_c is
    // negated when early capture is off for the ray (Q < 0)
    T r_cap;
    T t0, t1, t2;
    std::uint32_t steps, term, rej, zone;

    __device__ __forceinline__ bool init(const View<T>& v, const CamDir<T>& cd, const PassDesc& pass) {
        steps = rej = zone = 0;
        T E, L;
        KS<T> y0;
        if (!kerr_init(v, cd, y0, E, L)) {
            term = TERM_NO_ROOT;
            return false;
        }
        y = KSC<T>{y0.r, v.sin_th, v.cos_th, y0.ph, y0.pr, y0.pth};
        if constexpr (MIXED) {
            double Ed, Ld, prd, pthd;
            if (!kerr_init_fp64_constants(v, cd, Ed, Ld, prd, pthd)) {
                term = TERM_NO_ROOT;
                return false;
            }
            E = float(Ed);
            L = float(Ld);
            y.pr = float(prd);
            y.pth = float(pthd);
            Q = float(carter_Q_fp64(v, Ed, Ld, pthd));
        } else {
            Q = carter_Q(v, E, L, y.pth);
        }
        // a photon from outside inside its spherical photon orbit radius r_c(xi) has no
        // radial turning point left (Teo 2003); inside r_in it cannot reach the disc
        r_c = photon_orbit_radius(v, L / E);
        r_cap = DLIT(0.0);
        const bool cap = finite_(r_c) && carter_Q(v, E, L, y0.pth) >= DLIT(0.0);
        if (cap) r_cap = DM<T>::fmin_(r_c - DLIT(0.05) * v.M, v.r_in);
        if constexpr (RANGE) {
            T rs = DM<T>::fmax_(v.hcut, r_cap);
            if constexpr (MIXED) {
                const T zw = T(pass.zone);
                rs = DM<T>::fmax_(rs, v.r_plus + zw);
                if (finite_(r_c)) rs = DM<T>::fmax_(rs, r_c + zw);
            }
            r_cap = rs * DLIT(1.0001) + DLIT(1e-4);  // a margin for the rounding of the tests it stands for
            if (!cap) r_c = -r_c;
        }
        c = make_kc(v, E, L);
        h = T(pass.h_init_frac) * y.r;
        k1 = kerr_rhs_scs<T, FORM>(y, v, c);
        if (v.max_steps == 0u) {
            term = TERM_BUDGET;
            return false;
        }
        return true;
    }

    __device__ __forceinline__ bool step(const View<T>& v, const PassDesc& pass) {
        bool in_zone = false;
        if constexpr (RANGE) {
            if (!(y.r >= r_cap && y.r <= v.escape_r)) {
                const T rcap = r_c > DLIT(0.0) ? DM<T>::fmin_(r_c - DLIT(0.05) * v.M, v.r_in) : DLIT(0.0);
                if (!(y.r >= v.hcut && y.r <= v.escape_r) || (y.r < rcap && y.pr < DLIT(0.0))) {
                    if (!finite_(y.r) || y.r < v.hcut || y.r < rcap) {
                        term = TERM_HORIZON;
                    } else {
                        term = TERM_ESCAPE;
                        t0 = y.s;
                        t1 = y.ph;
                        t2 = y.c;
                    }
                    return true;
                }
                if constexpr (MIXED) {
                    const T zw = T(pass.zone);
                    in_zone = (absv(y.r - absv(r_c)) < zw) || (y.r - v.r_plus < zw);
                }
            }
        } else {
            // one test for NaN, capture (the reference's cut or the early one) and escape
            if (!(y.r >= v.hcut && y.r <= v.escape_r) || (y.r < r_cap && y.pr < DLIT(0.0))) {
                if (!finite_(y.r) || y.r < v.hcut || y.r < r_cap) {
                    term = TERM_HORIZON;
                } else {
                    term = TERM_ESCAPE;
                    t0 = y.s;
                    t1 = y.ph;
                    t2 = y.c;
                }
                return true;
            }
        }
        h = DM<T>::fmin_(h, T(pass.h_max_frac) * y.r);
        const KAttempt<T> at = kerr_attempt<T, FORM>(y, k1, h, v, c);
        ++steps;
        bool accept;
        if constexpr (MIXED && !RANGE) {
            const T zw = T(pass.zone);
            in_zone = (absv(y.r - r_c) < zw) || (y.r - v.r_plus < zw);
        }
        if (in_zone) {
            ++zone;
            const double e = error_norm_fp64_1div(y, at, pass.tol);
            accept = e <= 1.0;
            h = h * step_factor_fast(float(e));
        } else if constexpr (FAST && std::is_same_v<T, float>) {
            const T e = error_norm_fast(y, at, pass.tol);
            accept = e <= DLIT(1.0);
            h = h * step_factor_fast(e);
        } else {
            const T e = error_norm<T>(y, at, pass.tol);
            accept = e <= DLIT(1.0);
            h = h * step_factor<T>(e);
        }
        if (!accept) {
            ++rej;
        } else {
            // theta = pi/2 for theta in (0, pi): cos(theta) changes sign with sin(theta) > 0
            if ((v.flags & SGX_FLAG_DISC_ON) && (y.c * at.y4.c < DLIT(0.0)) && at.y4.s > DLIT(0.0)) {
                const T hs = at.h6 * DLIT(6.0);
                const T sfr = crossing_fraction(y.c, at.y4.c, k1.c, at.k5.c, hs);
                const T r_cross = hermite(y.r, at.y4.r, k1.r, at.k5.r, hs, sfr);
                if (r_cross >= v.r_in && r_cross <= v.r_out) {
                    const T T_local = disc_temperature(r_cross, v.r_in, v.peak_T);
                    term = T_local > DLIT(0.0) ? TERM_DISC : TERM_DISC_COLD;
                    t0 = r_cross;
                    t1 = hermite(y.ph, at.y4.ph, k1.ph, at.k5.ph, hs, sfr);
                    t2 = c.L;
                    y = at.y4;
                    return true;
                }
            }
            y = at.y4;
            renormalise(y);
            // the render kernels always project (a run-time flag costs 0.6-1.2 %
            // of the 4K pass as a select or a branch); the probes honour
            // PassDesc::project
            const T pp = project_pth(y.pth, y.s, y.c, Q, c);
            if constexpr (RTPROJ) y.pth = pass.project ? pp : y.pth;
            else y.pth = pp;
            k1 = at.k5;
        }
        if (steps >= v.max_steps) {
            term = TERM_BUDGET;
            return true;
        }
        return false;
    }

    __device__ __forceinline__ Rec<T> record() const { return Rec<T>{t0, t1, t2, pack_meta(term, steps)}; }
};

// Colour of a hit record (geodesic_kernel.cu:250-296, 354-402): starfield for
// an escape, disc emission for a hot crossing, black otherwise.
template <class T> __device__ __forceinline__ V3<T> shade_record(const View<T>& v, const Rec<T>& r) {
    const std::uint32_t term = r.meta & 7u;
    if (term == TERM_ESCAPE && (v.flags & SGX_FLAG_STARFIELD_ON)) return sky_color_sc(r.t0, r.t2, r.t1);
    if (term == TERM_DISC) {
        const T T_local = disc_temperature(r.t0, v.r_in, v.peak_T);
        if (v.metric == SGX_METRIC_KERR) return kerr_disc(v, r.t2, r.t0, r.t1, T_local);
        return schw_disc(v, r.t2, r.t0, r.t1, T_local);
    }
    return mk3(DLIT(0.0), DLIT(0.0), DLIT(0.0));
}

template <class T> __device__ __forceinline__ void load_view(View<T>& dst, const View<T>* src) {
    // Cooperative copy of one view's constants into shared memory.
    const int words = int(sizeof(View<T>) / 4);
    const std::uint32_t* s = reinterpret_cast<const std::uint32_t*>(src);
    std::uint32_t* d = reinterpret_cast<std::uint32_t*>(&dst);
    for (int i = threadIdx.x; i < words; i += blockDim.x) d[i] = s[i];
}

// Warp-aggregated add of a per-lane counter.
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0ull) atomicAdd(dst, v);
}

// Shared-memory image of a ViewSet: the views, the offset tables and the
// pass's Halton offsets.  Host and device agree on the layout through
// set_smem_bytes().
template <class T> struct SmemSet {
    View<T>* views;
    std::uint64_t* ray_off;  // n + 1
    std::uint64_t* rec_off;  // n
    std::uint64_t* pix_off;  // n + 1
    std::uint32_t* S;        // n
    T* off_x;                // max_S
    T* off_y;
};

__host__ __device__ constexpr std::size_t align16(std::size_t x) { return (x + 15) & ~std::size_t(15); }

template <class T> __host__ __device__ std::size_t set_smem_bytes(std::uint32_t n, std::uint32_t max_S) {
    return align16(n * sizeof(View<T>)) + align16((n + 1) * 8) + align16(n * 8) + align16((n + 1) * 8) +
           align16(n * 4) + 2 * align16(max_S * sizeof(T));
}

template <class T> __device__ __forceinline__ SmemSet<T> carve(unsigned char* base, std::uint32_t n, std::uint32_t max_S) {
    SmemSet<T> m;
    std::size_t o = 0;
    m.views = reinterpret_cast<View<T>*>(base + o);
    o += align16(n * sizeof(View<T>));
    m.ray_off = reinterpret_cast<std::uint64_t*>(base + o);
    o += align16((n + 1) * 8);
    m.rec_off = reinterpret_cast<std::uint64_t*>(base + o);
    o += align16(n * 8);
    m.pix_off = reinterpret_cast<std::uint64_t*>(base + o);
    o += align16((n + 1) * 8);
    m.S = reinterpret_cast<std::uint32_t*>(base + o);
    o += align16(n * 4);
    m.off_x = reinterpret_cast<T*>(base + o);
    o += align16(max_S * sizeof(T));
    m.off_y = reinterpret_cast<T*>(base + o);
    return m;
}

template <class T> __device__ void load_set(const SmemSet<T>& m, const ViewSet& vs, bool offsets) {
    const int words = int(vs.n * sizeof(View<T>) / 4);
    const std::uint32_t* src = static_cast<const std::uint32_t*>(vs.views);
    std::uint32_t* dst = reinterpret_cast<std::uint32_t*>(m.views);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    for (std::uint32_t i = threadIdx.x; i <= vs.n; i += blockDim.x) {
        m.ray_off[i] = vs.ray_off[i];
        m.pix_off[i] = vs.pix_off[i];
        if (i < vs.n) {
            m.rec_off[i] = vs.rec_off[i];
            m.S[i] = vs.S[i];
        }
    }
    if (offsets) {
        // Halton(s0 + i + 1) in bases 2 and 3 (spp == 1 views use the pixel
        // centre instead, at the point of use).
        for (std::uint32_t i = threadIdx.x; i < vs.max_S; i += blockDim.x)
            sample_offset<T>(2u, vs.s0 + i, m.off_x[i], m.off_y[i]);
    }
}

// Index of the last offset <= x in off[0..n] (off[0] = 0, off[n] = total).
__device__ __forceinline__ std::uint32_t find_view(const std::uint64_t* off, std::uint32_t n, std::uint64_t x) {
    std::uint32_t lo = 0, hi = n;  // invariant: off[lo] <= x < off[hi]
    while (hi - lo > 1u) {
        const std::uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

enum : int { MODE_IDLE = 0, MODE_ACTIVE = 1, MODE_DONE = 2 };

// The persistent tracer over a set of views.  Ray ids enumerate, view by
// view, tiles of tile_w x tile_h pixels (padded to whole tiles), the pixels
// of a tile row-major, and a pixel's samples innermost; ids that land in the
// padding carry no work.  Each policy names its resident blocks of 256 per
// SM (kMinBlocks for a single view, kMinBlocksMulti for a batch), which caps
// its registers: 4 = 64 registers, 3 = 80; FP64 variants keep their
// registers (capped they spill up to 1.4 KB).
// ONE: a single-view pass whose constants arrive as the kernel parameter
// `one`, read from the constant bank as instruction operands instead of
// shared-memory loads held in registers.
template <class T, class Ray, bool ONE>
__global__ void __launch_bounds__(256, ONE ? Ray::kMinBlocks : Ray::kMinBlocksMulti)
    trace_persistent(const __grid_constant__ PassDesc pass, const __grid_constant__ View<T> one) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // Block totals of the ray counters and each lane's record slot live in
    // shared memory, not in registers held across the integration loop.
    __shared__ unsigned long long s_count[5];  // steps, rejected, zone steps, budget hits, rays
    __shared__ std::uint64_t s_rec[256];
    const ViewSet& vs = pass.vs;
    const SmemSet<T> m = carve<T>(smem_raw, vs.n, vs.max_S);
    load_set(m, vs, true);
    if (threadIdx.x < 5u) s_count[threadIdx.x] = 0ull;
    __syncthreads();
    Rec<T>* __restrict__ results = static_cast<Rec<T>*>(pass.results);

    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    Ray ray;
    int mode = MODE_IDLE;
    std::uint32_t vid = 0;
    bool exhausted = false;
    auto view_of = [&](std::uint32_t i) -> const View<T>& {
        if constexpr (ONE) return one;
        else return m.views[i];
    };

    for (;;) {
        // 1. store the hit records of rays that ended.
        if (mode == MODE_DONE) {
            results[s_rec[threadIdx.x]] = ray.record();
            atomicAdd(&s_count[0], (unsigned long long)ray.steps);
            if (ray.rej != 0u) atomicAdd(&s_count[1], (unsigned long long)ray.rej);
            if (ray.zone != 0u) atomicAdd(&s_count[2], (unsigned long long)ray.zone);
            if (ray.term == TERM_BUDGET) atomicAdd(&s_count[3], 1ull);
            atomicAdd(&s_count[4], 1ull);
            mode = MODE_IDLE;
        }
        // 2. refill idle lanes from the queue, one atomic per warp.
        if (!exhausted) {
            const unsigned idle = __ballot_sync(kFull, mode == MODE_IDLE);
            if (idle != 0u) {
                const unsigned n = __popc(idle);
                const int leader = __ffs(idle) - 1;
                unsigned long long base = 0;
                if (int(lane) == leader) base = atomicAdd(&pass.counters->next_ray, (unsigned long long)n);
                base = __shfl_sync(kFull, base, leader);
                if (mode == MODE_IDLE) {
                    const std::uint64_t id = base + __popc(idle & lt_mask);
                    if (id < vs.total_rays) {
                        vid = (ONE || vs.n == 1u) ? 0u : find_view(m.ray_off, vs.n, id);
                        const View<T>& v = view_of(vid);
                        const std::uint32_t Sv = m.S[vid];
                        const std::uint64_t local = id - m.ray_off[vid];
                        const std::uint64_t seq = local / Sv;
                        const std::uint32_t sl = std::uint32_t(local - seq * Sv);
                        // tile_w == 0: whole rows of this view (no padding)
                        const std::uint32_t tw = vs.tile_w == 0u ? v.width : vs.tile_w;
                        const std::uint32_t th = vs.tile_w == 0u ? 1u : vs.tile_h;
                        const std::uint32_t tpix = tw * th;
                        const std::uint32_t tiles_x = (v.width + tw - 1u) / tw;
                        const std::uint32_t tile = std::uint32_t(seq / tpix);
                        const std::uint32_t within = std::uint32_t(seq - std::uint64_t(tile) * tpix);
                        const std::uint32_t ty = tile / tiles_x;
                        const std::uint32_t wy = within / tw;
                        const std::uint32_t gx = (tile - ty * tiles_x) * tw + (within - wy * tw);
                        // a frame slice traces its own rows, numbered locally
                        const bool sliced = vs.slice_count > 1u;
                        const std::uint32_t vh = sliced ? vs.slice_h : v.height;
                        const std::uint32_t gyl = ty * th + wy;
                        if (gx < v.width && gyl < vh) {
                            s_rec[threadIdx.x] = m.rec_off[vid] + std::uint64_t(sl) * (std::uint64_t(v.width) * vh) +
                                                 std::uint64_t(gyl) * v.width + gx;
                            const std::uint32_t gy =
                                sliced ? slice_row(vs.slice_band, vs.slice_count, vs.slice_index, gyl) : gyl;
                            const T ox = v.spp == 1u ? DLIT(0.5) : m.off_x[sl];
                            const T oy = v.spp == 1u ? DLIT(0.5) : m.off_y[sl];
                            const CamDir<T> cd = camera_dir(v, gx, gy, ox, oy);
                            mode = ray.init(v, cd, pass) ? MODE_ACTIVE : MODE_DONE;
                        }
                    }
                }
                if (base + n >= vs.total_rays) exhausted = true;
            }
        }
        if (__ballot_sync(kFull, mode != MODE_IDLE) == 0u) {
            if (exhausted) break;
            continue;  // every id this round fell in tile padding
        }
        // 3. integrate.
        const View<T>& v = view_of(vid);
        for (std::uint32_t j = 0; j < pass.refill; ++j) {
            if (mode == MODE_ACTIVE && ray.step(v, pass)) mode = MODE_DONE;
            if (__all_sync(kFull, mode != MODE_ACTIVE)) break;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0u) {
        if (s_count[0] != 0ull) atomicAdd(&pass.counters->steps, s_count[0]);
        if (s_count[1] != 0ull) atomicAdd(&pass.counters->rejected, s_count[1]);
        if (s_count[2] != 0ull) atomicAdd(&pass.counters->zone_steps, s_count[2]);
        if (s_count[3] != 0ull) atomicAdd(&pass.counters->budget_hits, s_count[3]);
        if (s_count[4] != 0ull) atomicAdd(&pass.counters->rays, s_count[4]);
    }
}

template <class T, class Ray>
__global__ void __launch_bounds__(128) trace_probe(const View<T>* __restrict__ g_view, std::uint64_t n,
                                                   const std::uint32_t* gx, const std::uint32_t* gy,
                                                   const std::uint32_t* s, float* hdr3, std::uint32_t* steps,
                                                   std::uint32_t* term, PassDesc pass) {
    __shared__ View<T> v;
    load_view(v, g_view);
    __syncthreads();
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Ray ray;
    T ox, oy;
    sample_offset<T>(v.spp, s[i], ox, oy);
    const CamDir<T> cd = camera_dir(v, gx[i], gy[i], ox, oy);
    if (ray.init(v, cd, pass)) {
        while (!ray.step(v, pass)) {
        }
    }
    const V3<T> hdr = shade_record(v, ray.record());
    if (hdr3 != nullptr) {
        hdr3[3 * i + 0] = float(hdr.x);
        hdr3[3 * i + 1] = float(hdr.y);
        hdr3[3 * i + 2] = float(hdr.z);
    }
    if (steps != nullptr) steps[i] = ray.steps;
    if (term != nullptr) term[i] = ray.term;
}

// Constants of motion of single samples of the error-controlled form
// (diagnostics): E, L_z and the Carter constant the ray started with, and the
// Carter constant and 2H of its last state, all in FP64.  The starting values
// are recomputed from the camera ray exactly as the policy's init computed
// them (FP32 Q for the FP32 form, FP64 E, L, Q for the mixed form).
template <class T, int FL>
__global__ void __launch_bounds__(128) trace_invariants(const View<T>* __restrict__ g_view, std::uint64_t n,
                                                        const std::uint32_t* gx, const std::uint32_t* gy,
                                                        const std::uint32_t* s, double* inv5, std::uint32_t* term,
                                                        PassDesc pass) {
    using Ray = KerrAdaptive<T, FL>;
    __shared__ View<T> v;
    load_view(v, g_view);
    __syncthreads();
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T ox, oy;
    sample_offset<T>(v.spp, s[i], ox, oy);
    const CamDir<T> cd = camera_dir(v, gx[i], gy[i], ox, oy);
    Ray ray;
    if (ray.init(v, cd, pass)) {
        while (!ray.step(v, pass)) {
        }
    }
    double* o = inv5 + 5 * i;
    if (ray.term == TERM_NO_ROOT) {
        for (int k = 0; k < 5; ++k) o[k] = __longlong_as_double(0x7ff8000000000000ll);  // NaN
    } else {
        KS<T> y0;
        T Ef, Lf;
        kerr_init(v, cd, y0, Ef, Lf);
        double E, L, Q0;
        if constexpr (Ray::MIXED) {
            double prd, pthd;
            kerr_init_fp64_constants(v, cd, E, L, prd, pthd);
            Q0 = carter_Q_fp64(v, E, L, pthd);
        } else {
            E = double(Ef);
            L = double(Lf);
            Q0 = double(carter_Q(v, Ef, Lf, y0.pth));
        }
        double Q, H2;
        kerr_invariants_fp64(v, E, L, double(ray.y.r), double(ray.y.s), double(ray.y.c), double(ray.y.pr),
                             double(ray.y.pth), Q, H2);
        o[0] = E;
        o[1] = L;
        o[2] = Q0;
        o[3] = Q;
        o[4] = H2;
    }
    if (term != nullptr) term[i] = ray.term;
}

template <class T> __global__ void setup_views(const sgx_uniforms* u, std::uint32_t n, View<T>* out) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_view<T>(u[i]);
}

// Final encode of a pixel's mean (geodesic_kernel.cu:502-509).
__device__ __forceinline__ void encode_pixel(float4 sum, float scale, std::uint32_t format, void* out,
                                             std::uint64_t pix) {
    const float r = sum.x * scale, g = sum.y * scale, b = sum.z * scale;
    if (format == SGX_FORMAT_RGBA16F_HDR) {
        // scene-referred HDR mean in half precision, as the realtime backends'
        // rgba16f target holds it
        __half2* o = static_cast<__half2*>(out) + 2 * pix;
        o[0] = __floats2half2_rn(r, g);
        o[1] = __floats2half2_rn(b, 1.0f);
    } else if (format == SGX_FORMAT_RGBA8_SRGB) {
        uchar4 o;
        o.x = to_u8(r);
        o.y = to_u8(g);
        o.z = to_u8(b);
        o.w = 255;
        static_cast<uchar4*>(out)[pix] = o;
    } else {
        static_cast<float4*>(out)[pix] = make_float4(r, g, b, 1.0f);
    }
}

// Shades each hit record of the pass and adds it to the pixel's sum in sample
// order (the reference's `ldr = ldr + aces(hdr * exposure)`,
// geodesic_kernel.cu:492-501); the last pass scales by 1/spp and encodes.
// For the HDR format the sum is of the raw HDR colour (no exposure, no tone
// map), the input of the bloom/blit pipeline.
// The pass's samples of packed pixel p of view vid added to its running sum
// in sample order; the sum is stored back to acc and returned.
template <class T>
__device__ __forceinline__ float4 accum_pixel(const SmemSet<T>& m, const ViewSet& vs, std::uint32_t vid,
                                              std::uint64_t p, const Rec<T>* __restrict__ results,
                                              float4* __restrict__ acc, bool first, bool raw) {
    const View<T>& v = m.views[vid];
    const std::uint64_t pix = p - m.pix_off[vid];
    const std::uint64_t npix = std::uint64_t(v.width) * (vs.slice_count > 1u ? vs.slice_h : v.height);
    const std::uint64_t base = m.rec_off[vid] + pix;
    const std::uint32_t S = m.S[vid];
    float4 sum = first ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : acc[p];
    for (std::uint32_t s = 0; s < S; ++s) {
        const Rec<T> rec = results[base + std::uint64_t(s) * npix];
        const V3<T> hdr = shade_record(v, rec);
        if (raw) {
            sum.x = sum.x + float(hdr.x);
            sum.y = sum.y + float(hdr.y);
            sum.z = sum.z + float(hdr.z);
        } else {
            sum.x = sum.x + float(aces1(hdr.x * v.exposure));
            sum.y = sum.y + float(aces1(hdr.y * v.exposure));
            sum.z = sum.z + float(aces1(hdr.z * v.exposure));
        }
    }
    acc[p] = sum;
    return sum;
}

template <class T>
__global__ void __launch_bounds__(256) accumulate_kernel(ViewSet vs, const Rec<T>* __restrict__ results,
                                                         float4* __restrict__ acc, bool first, bool finalize,
                                                         std::uint32_t format, void* out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const SmemSet<T> m = carve<T>(smem_raw, vs.n, 0);
    load_set(m, vs, false);
    __syncthreads();
    const std::uint64_t p = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= vs.total_pix) return;
    const std::uint32_t vid = vs.n == 1u ? 0u : find_view(m.pix_off, vs.n, p);
    const float4 sum = accum_pixel(m, vs, vid, p, results, acc, first, format == SGX_FORMAT_RGBA16F_HDR);
    if (finalize) encode_pixel(sum, 1.0f / float(m.views[vid].spp), format, out, p);
}

// The last pass of a single-view HDR frame with the bloom extract fused in:
// one lane per pixel as in accumulate_kernel, the four lanes of a 2x2 block of
// the frame (bw x bh = W/2 x H/2 blocks) adjacent in the warp.  Each adds its
// pixel's samples and writes the half-precision HDR mean; the block's first
// lane gathers the four half values by warp shuffles and writes the block's
// half-resolution extract texel (karis_extract, as the separate extract
// kernel computes it from the stored frame).  Lanes past the blocks take the
// pixels outside them (the last column when W is odd, then the last row when
// H is odd).  Every lane of a warp reaches the shuffles.
template <class T>
__global__ void __launch_bounds__(256)
    accumulate_hdr_extract_kernel(ViewSet vs, const Rec<T>* __restrict__ results, float4* __restrict__ acc,
                                  bool first, void* out, __half2* __restrict__ ext, std::uint32_t bw,
                                  std::uint32_t bh, float threshold) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const SmemSet<T> m = carve<T>(smem_raw, vs.n, 0);
    load_set(m, vs, false);
    __syncthreads();
    const View<T>& v = m.views[0];
    const std::uint32_t W = v.width, H = v.height;
    const float scale = 1.0f / float(v.spp);
    const std::uint64_t t = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const std::uint64_t nq = std::uint64_t(bw) * bh;
    const bool in_block = t < 4ull * nq;
    bool valid = true;
    std::uint64_t p = 0;
    if (in_block) {
        const std::uint64_t q = t >> 2;
        const std::uint32_t k = std::uint32_t(t & 3ull);
        const std::uint32_t qy = std::uint32_t(q / bw), qx = std::uint32_t(q - std::uint64_t(qy) * bw);
        p = std::uint64_t(2u * qy + (k >> 1)) * W + 2u * qx + (k & 1u);
    } else {
        std::uint64_t e = t - 4ull * nq;
        if (W > 2u * bw && e < 2ull * bh) {
            p = e * W + (W - 1u);
        } else {
            if (W > 2u * bw) e -= 2ull * bh;
            valid = H > 2u * bh && e < W;
            p = std::uint64_t(H - 1u) * W + e;
        }
    }
    float4 h = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (valid) {
        const float4 sum = accum_pixel(m, vs, 0u, p, results, acc, first, true);
        encode_pixel(sum, scale, SGX_FORMAT_RGBA16F_HDR, out, p);
        // the pixel as the half-precision frame holds it
        const float2 lo = __half22float2(__floats2half2_rn(sum.x * scale, sum.y * scale));
        const float2 hi = __half22float2(__floats2half2_rn(sum.z * scale, 1.0f));
        h = make_float4(lo.x, lo.y, hi.x, hi.y);
    }
    const unsigned lane = threadIdx.x & 31u, lead = lane & ~3u;
    float4 qv[4];
#pragma unroll
    for (unsigned k = 0; k < 4u; ++k) {
        qv[k].x = __shfl_sync(kFull, h.x, lead + k);
        qv[k].y = __shfl_sync(kFull, h.y, lead + k);
        qv[k].z = __shfl_sync(kFull, h.z, lead + k);
        qv[k].w = 1.0f;
    }
    if (in_block && (lane & 3u) == 0u) {
        float r, g, b;
        karis_extract(qv[0], qv[1], qv[2], qv[3], threshold, r, g, b);
        const std::uint64_t q = t >> 2;
        ext[2 * q] = __floats2half2_rn(r, g);
        ext[2 * q + 1] = __floats2half2_rn(b, 1.0f);
    }
}

__global__ void encode_kernel(const float4* __restrict__ acc, std::uint32_t npix, float scale, std::uint32_t format,
                              void* out) {
    const std::uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    encode_pixel(acc[pix], scale, format, out, pix);
}

// ---------------------------------------------------------------------------
// Dispatch
// ---------------------------------------------------------------------------
template <class T, class Ray, bool ONE>
cudaError_t run_kernel(const PassDesc& pass, LaunchShape shape, const void* h_view, cudaStream_t st) {
    auto kern = trace_persistent<T, Ray, ONE>;
    View<T> one{};
    if constexpr (ONE) std::memcpy(&one, h_view, sizeof(View<T>));
    const std::size_t smem = set_smem_bytes<T>(pass.vs.n, pass.vs.max_S);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = shape.block_threads > 0 ? shape.block_threads
                                                : (ONE ? kDefaultBlockThreads : kDefaultBlockThreadsMulti);
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (shape.blocks_per_sm > 0 && shape.blocks_per_sm < per_sm) per_sm = shape.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    std::uint64_t blocks = std::uint64_t(sms) * per_sm;
    const std::uint64_t need = (pass.vs.total_rays + threads - 1) / threads;
    if (need < blocks) blocks = need > 0 ? need : 1;
    kern<<<unsigned(blocks), threads, smem, st>>>(pass, one);
    return cudaGetLastError();
}

template <class T, template <class, int> class Policy, int FL>
cudaError_t run_persistent(const PassDesc& pass, LaunchShape shape, const void* h_view, cudaStream_t st) {
    if (h_view != nullptr && pass.vs.n == 1u) return run_kernel<T, Policy<T, FL>, true>(pass, shape, h_view, st);
    // the multi-view kernels of the error-controlled form take the range test
    constexpr int FLM = std::is_same_v<Policy<T, FL>, KerrAdaptive<T, FL>> ? (FL | FL_RANGE) : FL;
    return run_kernel<T, Policy<T, FLM>, false>(pass, shape, nullptr, st);
}

template <class T, template <class, int> class Policy, int FL>
cudaError_t run_probe(const void* d_view, std::uint64_t n, const std::uint32_t* gx, const std::uint32_t* gy,
                      const std::uint32_t* s, float* hdr3, std::uint32_t* steps, std::uint32_t* term,
                      const PassDesc& pass, cudaStream_t st) {
    const unsigned threads = 128;
    const std::uint64_t blocks = (n + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    trace_probe<T, Policy<T, FL>><<<unsigned(blocks), threads, 0, st>>>(static_cast<const View<T>*>(d_view), n, gx, gy,
                                                                       s, hdr3, steps, term, pass);
    return cudaGetLastError();
}

// One call site per (metric, precision, integrator, RHS form): F is invoked
// with the chosen <T, Policy, FL> as a generic lambda's template arguments.
// rhs_form: 0 the separated form, 1 the reference's divisions, 2 the
// separated form with sin/cos of theta carried in the fixed-step state (FP32;
// FP64 runs form 0; the error-controlled form always carries them).
// XF: extra policy flags of the error-controlled form (FL_RTPROJ for the probes).
template <int XF = 0, class F>
cudaError_t dispatch(int metric, int precision, int integrator, int rhs_form, F&& f) {
    const bool adaptive = integrator == SGX_INTEGRATOR_ADAPTIVE;
    const bool ref = rhs_form == 1, hw = rhs_form == 2;
    if (metric == SGX_METRIC_KERR && adaptive) {
        if (precision == SGX_PRECISION_FP64)
            return ref ? f.template operator()<double, KerrAdaptive, XF>()
                       : f.template operator()<double, KerrAdaptive, FL_FAST | XF>();
        // the error-controlled form evaluates no sine or cosine per stage, so
        // forms 0 and 2 are the same kernel
        if (precision == SGX_PRECISION_MIXED)
            return ref ? f.template operator()<float, KerrAdaptive, FL_MIXED | XF>()
                       : f.template operator()<float, KerrAdaptive, FL_FAST | FL_MIXED | XF>();
        return ref ? f.template operator()<float, KerrAdaptive, XF>()
                   : f.template operator()<float, KerrAdaptive, FL_FAST | XF>();
    }
    if (metric == SGX_METRIC_KERR) {
        if (precision == SGX_PRECISION_FP64)
            return ref ? f.template operator()<double, KerrFixed, 0>()
                       : f.template operator()<double, KerrFixed, FL_FAST>();
        return ref  ? f.template operator()<float, KerrFixed, 0>()
               : hw ? f.template operator()<float, KerrFixed, FL_FAST | FL_SC>()
                    : f.template operator()<float, KerrFixed, FL_FAST>();
    }
    // Schwarzschild: the reference's fixed-step integrator for every form.
    if (precision == SGX_PRECISION_FP64) return f.template operator()<double, SchwFixed, 0>();
    return f.template operator()<float, SchwFixed, 0>();
}

}  // namespace

std::size_t view_bytes() {
    const std::size_t a = sizeof(View<float>), b = sizeof(View<double>);
    return ((a > b ? a : b) + 255) / 256 * 256;
}

std::size_t record_bytes(int precision) {
    return precision == SGX_PRECISION_FP64 ? sizeof(Rec<double>) : sizeof(Rec<float>);
}

std::size_t format_bytes(std::uint32_t format) {
    return format == SGX_FORMAT_RGBA8_SRGB ? 4 : (format == SGX_FORMAT_RGBA16F_HDR ? 8 : 16);
}

bool plan_views(const sgx_uniforms* u, std::uint32_t n, std::uint32_t s0, std::uint32_t S_pass, std::uint32_t tile_w,
                std::uint32_t tile_h, ViewPlan& plan, SliceSpec slice) {
    if (n == 0 || n > kMaxLaunchViews || (tile_w != 0 && tile_h == 0)) return false;
    const bool sliced = slice.count > 1u;
    if (sliced && (n != 1u || slice.index >= slice.count || slice.band == 0u)) return false;
    plan = ViewPlan{};
    plan.n = n;
    plan.s0 = s0;
    plan.tile_w = tile_w;
    plan.tile_h = tile_h;
    if (sliced) {
        plan.slice = slice;
        plan.slice_h = slice_rows(u[0].height, slice.band, slice.count, slice.index);
        if (plan.slice_h == 0u) return false;
    }
    std::uint64_t* ray_off = plan.words;
    std::uint64_t* rec_off = ray_off + (n + 1);
    std::uint64_t* pix_off = rec_off + n;
    std::uint32_t* S = reinterpret_cast<std::uint32_t*>(pix_off + (n + 1));
    std::uint64_t r = 0, q = 0, px = 0;
    for (std::uint32_t i = 0; i < n; ++i) {
        const std::uint32_t spp = u[i].supersample < 1u ? 1u : (u[i].supersample > 1024u ? 1024u : u[i].supersample);
        const std::uint32_t Sv = S_pass == 0 ? spp : S_pass;
        if (Sv == 0 || Sv > kMaxPassSamplesHost) return false;
        const std::uint64_t w = u[i].width, h = sliced ? plan.slice_h : u[i].height;
        // tile_w == 0: whole rows of each view, no padding.
        const std::uint64_t tw = tile_w == 0 ? w : tile_w, th = tile_w == 0 ? 1 : tile_h;
        const std::uint64_t padded = ((w + tw - 1) / tw) * tw * (((h + th - 1) / th) * th);
        ray_off[i] = r;
        rec_off[i] = q;
        pix_off[i] = px;
        S[i] = Sv;
        r += padded * Sv;
        q += w * h * Sv;
        px += w * h;
        if (Sv > plan.max_S) plan.max_S = Sv;
    }
    ray_off[n] = r;
    pix_off[n] = px;
    plan.total_rays = r;
    plan.total_recs = q;
    plan.total_pix = px;
    plan.word_count = (n + 1) + n + (n + 1) + (n + 1) / 2;
    return true;
}

ViewSet make_view_set(const ViewPlan& plan, const void* d_views, const std::uint64_t* d_words) {
    ViewSet vs{};
    const std::uint32_t n = plan.n;
    vs.views = d_views;
    vs.ray_off = d_words;
    vs.rec_off = d_words + (n + 1);
    vs.pix_off = d_words + (n + 1) + n;
    vs.S = reinterpret_cast<const std::uint32_t*>(d_words + (n + 1) + n + (n + 1));
    vs.n = n;
    vs.max_S = plan.max_S;
    vs.s0 = plan.s0;
    vs.tile_w = plan.tile_w;
    vs.tile_h = plan.tile_h;
    if (plan.slice.count > 1u) {
        vs.slice_count = plan.slice.count;
        vs.slice_index = plan.slice.index;
        vs.slice_band = plan.slice.band;
        vs.slice_h = plan.slice_h;
    }
    vs.total_rays = plan.total_rays;
    vs.total_pix = plan.total_pix;
    return vs;
}

cudaError_t launch_setup_views(const sgx_uniforms* d_u, std::uint32_t n, void* d_views, int precision,
                               cudaStream_t st) {
    const unsigned threads = 64;
    const unsigned blocks = (n + threads - 1) / threads;
    if (precision == SGX_PRECISION_FP64) {
        setup_views<double><<<blocks, threads, 0, st>>>(d_u, n, static_cast<View<double>*>(d_views));
    } else {
        setup_views<float><<<blocks, threads, 0, st>>>(d_u, n, static_cast<View<float>*>(d_views));
    }
    return cudaGetLastError();
}

cudaError_t launch_trace(int metric, int precision, int integrator, int rhs_form, const PassDesc& pass,
                         LaunchShape shape, cudaStream_t st, const void* h_view) {
    return dispatch(metric, precision, integrator, rhs_form,
                    [&]<class T, template <class, int> class Policy, int FL>() {
                        return run_persistent<T, Policy, FL>(pass, shape, h_view, st);
                    });
}

cudaError_t launch_probe(const void* d_view, int metric, int precision, int integrator, int rhs_form,
                         std::uint64_t n, const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s,
                         float* hdr3, std::uint32_t* steps, std::uint32_t* term, const PassDesc& opts,
                         cudaStream_t st) {
    PassDesc pass{};
    pass.tol = opts.tol;
    pass.h_init_frac = opts.h_init_frac;
    pass.h_max_frac = opts.h_max_frac;
    pass.zone = opts.zone;
    pass.project = opts.project;
    return dispatch<FL_RTPROJ>(metric, precision, integrator, rhs_form,
                    [&]<class T, template <class, int> class Policy, int FL>() {
                        return run_probe<T, Policy, FL>(d_view, n, gx, gy, s, hdr3, steps, term, pass, st);
                    });
}

cudaError_t launch_invariants(const void* d_view, int precision, int rhs_form, std::uint64_t n,
                              const std::uint32_t* gx, const std::uint32_t* gy, const std::uint32_t* s, double* inv5,
                              std::uint32_t* term, const PassDesc& pass, cudaStream_t st) {
    const unsigned threads = 128;
    const std::uint64_t blocks = (n + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    const bool ref = rhs_form == 1;
    const unsigned b = unsigned(blocks);
    constexpr int R = FL_RTPROJ;
    if (precision == SGX_PRECISION_FP64) {
        const auto* vw = static_cast<const View<double>*>(d_view);
        if (ref) trace_invariants<double, R><<<b, threads, 0, st>>>(vw, n, gx, gy, s, inv5, term, pass);
        else trace_invariants<double, FL_FAST | R><<<b, threads, 0, st>>>(vw, n, gx, gy, s, inv5, term, pass);
    } else {
        const auto* vw = static_cast<const View<float>*>(d_view);
        if (precision == SGX_PRECISION_MIXED) {
            if (ref) trace_invariants<float, FL_MIXED | R><<<b, threads, 0, st>>>(vw, n, gx, gy, s, inv5, term, pass);
            else
                trace_invariants<float, FL_FAST | FL_MIXED | R><<<b, threads, 0, st>>>(vw, n, gx, gy, s, inv5, term,
                                                                                        pass);
        } else {
            if (ref) trace_invariants<float, R><<<b, threads, 0, st>>>(vw, n, gx, gy, s, inv5, term, pass);
            else trace_invariants<float, FL_FAST | R><<<b, threads, 0, st>>>(vw, n, gx, gy, s, inv5, term, pass);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_accumulate(int precision, const ViewSet& vs, const void* results, float4* acc, bool first,
                              bool finalize, std::uint32_t format, void* out, cudaStream_t st) {
    const unsigned threads = 256;
    const std::uint64_t blocks = (vs.total_pix + threads - 1) / threads;
    // a set of many FP64 views needs more than the default 48 KB of shared memory
    if (precision == SGX_PRECISION_FP64) {
        const std::size_t smem = set_smem_bytes<double>(vs.n, 0);
        cudaError_t e = cudaFuncSetAttribute(accumulate_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(smem));
        if (e != cudaSuccess) return e;
        accumulate_kernel<double><<<unsigned(blocks), threads, smem, st>>>(
            vs, static_cast<const Rec<double>*>(results), acc, first, finalize, format, out);
    } else {
        const std::size_t smem = set_smem_bytes<float>(vs.n, 0);
        cudaError_t e = cudaFuncSetAttribute(accumulate_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(smem));
        if (e != cudaSuccess) return e;
        accumulate_kernel<float><<<unsigned(blocks), threads, smem, st>>>(
            vs, static_cast<const Rec<float>*>(results), acc, first, finalize, format, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_accumulate_hdr_extract(int precision, const ViewSet& vs, const void* results, float4* acc,
                                          bool first, void* out, void* ext, std::uint32_t W, std::uint32_t H,
                                          float threshold, cudaStream_t st) {
    if (vs.n != 1u || vs.slice_count > 1u || W < 2u || H < 2u) return cudaErrorInvalidValue;
    const std::uint32_t bw = W / 2u, bh = H / 2u;
    const std::uint64_t n = 4ull * bw * bh + (W > 2u * bw ? 2ull * bh : 0ull) + (H > 2u * bh ? W : 0u);
    const unsigned threads = 256;
    const unsigned blocks = unsigned((n + threads - 1) / threads);
    __half2* e = static_cast<__half2*>(ext);
    if (precision == SGX_PRECISION_FP64) {
        const std::size_t smem = set_smem_bytes<double>(vs.n, 0);
        accumulate_hdr_extract_kernel<double><<<blocks, threads, smem, st>>>(
            vs, static_cast<const Rec<double>*>(results), acc, first, out, e, bw, bh, threshold);
    } else {
        const std::size_t smem = set_smem_bytes<float>(vs.n, 0);
        accumulate_hdr_extract_kernel<float><<<blocks, threads, smem, st>>>(
            vs, static_cast<const Rec<float>*>(results), acc, first, out, e, bw, bh, threshold);
    }
    return cudaGetLastError();
}

cudaError_t launch_encode(const float4* acc, std::uint32_t npix, float scale, std::uint32_t format, void* out,
                          cudaStream_t st) {
    const unsigned threads = 256;
    const unsigned blocks = (npix + threads - 1) / threads;
    encode_kernel<<<blocks, threads, 0, st>>>(acc, npix, scale, format, out);
    return cudaGetLastError();
}

static_assert(sizeof(Rec<float>) == 16 && sizeof(Rec<double>) == 32, "hit record sizes");

}  // namespace sgxk
