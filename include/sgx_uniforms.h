/*
 * sgx_uniforms.h — the per-launch parameter block of the geodesic tracer.
 *
 * Byte-for-byte the same layout as the reference's `Uniforms`
 * (shared_shader/uniforms.h:54-95): 160 bytes, 16-byte aligned, every
 * 3-vector stored as four floats (w unused).  A caller that already packs the
 * reference struct can hand its bytes to this library unchanged; the static
 * asserts below pin every offset.
 *
 * Flag bits and metric selectors keep the reference values
 * (shared_shader/uniforms.h:41-52).
 */
#ifndef SGX_UNIFORMS_H
#define SGX_UNIFORMS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGX_FLAG_DOPPLER_ON (1u << 0)
#define SGX_FLAG_REDSHIFT_ON (1u << 1)
#define SGX_FLAG_DISC_ON (1u << 2)
#define SGX_FLAG_STARFIELD_ON (1u << 3)
#define SGX_FLAG_ADAPTIVE_STEP (1u << 4)

#define SGX_METRIC_SCHWARZSCHILD 0u
#define SGX_METRIC_KERR 1u

typedef struct sgx_vec4 {
    float x, y, z, w;
} sgx_vec4;

typedef struct sgx_uniforms {
    sgx_vec4 cam_pos;   /*   0: camera position, Cartesian, units of M            */
    sgx_vec4 cam_fwd;   /*  16: unit forward                                     */
    sgx_vec4 cam_right; /*  32: unit right                                       */
    sgx_vec4 cam_up;    /*  48: unit up                                          */
    float mass_M;       /*  64: mass in geometrized units                        */
    float spin_a;       /*  68: spin a (not a/M), 0 <= a <= M                     */
    float rs;           /*  72: 2M                                               */
    float tan_half_fov; /*  76: tan(fov_y / 2)                                   */
    float disc_r_inner; /*  80 */
    float disc_r_outer; /*  84 */
    float disc_peak_T;  /*  88: K                                                */
    float aspect;       /*  92: width / height                                   */
    float h_step;       /*  96: RK4 step in affine parameter                     */
    float escape_r;     /* 100 */
    float horizon_cut;  /* 104: Schwarzschild capture radius (1.02 rs)           */
    float time_sec;     /* 108: disc band animation phase                        */
    uint32_t width;     /* 112 */
    uint32_t height;    /* 116 */
    uint32_t metric_type; /* 120: SGX_METRIC_*                                   */
    uint32_t flags;       /* 124: SGX_FLAG_*                                     */
    uint32_t max_steps;   /* 128: integrator step budget per ray                 */
    uint32_t frame_index; /* 132 */
    uint32_t supersample; /* 136: samples per pixel (1..1024), Halton(2,3)       */
    uint32_t pad_b;       /* 140 */
    float exposure;        /* 144 */
    float bloom_threshold; /* 148 */
    float bloom_strength;  /* 152 */
    float disc_turbulence; /* 156 */
} sgx_uniforms;

#ifdef __cplusplus
#define SGX_STATIC_ASSERT static_assert
#else
#define SGX_STATIC_ASSERT _Static_assert
#endif

SGX_STATIC_ASSERT(sizeof(sgx_uniforms) == 160, "sgx_uniforms must be 160 bytes");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, cam_fwd) == 16, "cam_fwd offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, mass_M) == 64, "mass_M offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, disc_r_inner) == 80, "disc_r_inner offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, h_step) == 96, "h_step offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, width) == 112, "width offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, max_steps) == 128, "max_steps offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, exposure) == 144, "exposure offset");
SGX_STATIC_ASSERT(offsetof(sgx_uniforms, disc_turbulence) == 156, "disc_turbulence offset");

#ifdef __cplusplus
}
#endif

#endif /* SGX_UNIFORMS_H */
