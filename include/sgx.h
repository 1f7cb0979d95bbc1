/*
 * sgx.h — C ABI of the GB300 geodesic tracer (the drop-in boundary).
 *
 * Plain C: pointers, sizes, status codes; no CUDA or torch types.  Every entry
 * point below names the reference interface it replaces.  The reference's
 * boundary is the C++ class CudaBackend
 * (render/cuda/cuda_backend.hpp:17-46, render/include/render_backend.hpp:107-132)
 * and below it the kernel `singularity_geodesic_kernel(uint8_t*, Uniforms)`
 * (render/cuda/kernels/geodesic_kernel.cu:462).  The C++ shim
 * singularity_gb300/csrc/cuda_backend.hpp re-creates that class on top of
 * these functions, so the reference's cuda_cli relinks unchanged.
 *
 * Error behaviour: the reference prints CUDA errors and carries on
 * (cuda_backend.cu:38-43); here every call returns an sgx_status and the
 * context keeps the last message for sgx_last_error().
 *
 * Threading: a context is used by one host thread at a time; all its GPU
 * work runs on the context's own stream.
 */
#ifndef SGX_H
#define SGX_H

#include <stddef.h>
#include <stdint.h>

#include "sgx_uniforms.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SGX_ABI_VERSION 1

typedef enum sgx_status {
    SGX_OK = 0,
    SGX_ERR_INVALID_ARGUMENT = 1,
    SGX_ERR_CUDA = 2,
    SGX_ERR_OUT_OF_MEMORY = 3,
    SGX_ERR_NOT_RENDERED = 4,
    SGX_ERR_UNSUPPORTED = 5
} sgx_status;

/* Output encodings of a rendered frame. */
typedef enum sgx_format {
    SGX_FORMAT_RGBA8_SRGB = 0, /* reference output: ACES per sample, mean, sRGB, u8 */
    SGX_FORMAT_RGBA32F = 1,    /* the same mean before sRGB/quantisation, float, alpha 1 */
    SGX_FORMAT_RGBA16F_HDR = 2 /* mean scene-referred HDR (before exposure), half, alpha 1 */
} sgx_format;

/* Arithmetic of the integration. */
typedef enum sgx_precision {
    SGX_PRECISION_FP32 = 0,  /* bulk FP32 */
    SGX_PRECISION_MIXED = 1, /* FP32 bulk, FP64 constants of motion and FP64 step control
                                near the photon orbit and the horizon */
    SGX_PRECISION_FP64 = 2   /* FP64 throughout */
} sgx_precision;

typedef enum sgx_integrator {
    SGX_INTEGRATOR_FIXED = 0,   /* the reference: fixed-step RK4, h = u.h_step */
    SGX_INTEGRATOR_ADAPTIVE = 1 /* error-controlled RK4 with FSAL third-order estimate (Kerr) */
} sgx_integrator;

/* Per-render options.  sgx_render_opts_default() gives the reference's
 * behaviour: FP32, fixed step, every sample, RGBA8 sRGB. */
typedef struct sgx_render_opts {
    uint32_t struct_size;    /* sizeof(sgx_render_opts) */
    uint32_t precision;      /* sgx_precision */
    uint32_t integrator;     /* sgx_integrator */
    uint32_t format;         /* sgx_format kept by sgx_capture's default */
    float tolerance;         /* adaptive: error tolerance (default 1e-6) */
    float h_init_frac;       /* adaptive: first step = h_init_frac * r_camera (default 0.1) */
    float h_max_frac;        /* adaptive: step ceiling = h_max_frac * r (default 0.1) */
    float fp64_zone;         /* mixed: FP64 control band half-width in M (default 0.05) */
    uint32_t sample_begin;   /* first Halton sample of this pass (default 0) */
    uint32_t sample_count;   /* samples in this pass; 0 = all remaining (default 0) */
    uint32_t block_threads;  /* launch shape: threads per block, a multiple of 32 up to 256;
                                0 = tuned default (64 for one view, 128 for a batch) */
    uint32_t blocks_per_sm;  /* launch shape: resident blocks per SM; 0 = occupancy limit */
    uint32_t refill_interval;/* steps between warp refills of finished rays; 0 = 128 */
    uint32_t rhs_form;       /* Kerr right-hand side: 0 = the same Hamiltonian in Carter's
                                    separated form, three reciprocals (default),
                                1 = the reference's division-for-division form,
                                2 = form 0 with sin/cos of theta carried in the fixed-step
                                    state instead of evaluated per stage (FP32; the adaptive
                                    integrator always carries them, so there 2 equals 0) */
    uint32_t tile_w;         /* ray order: tiles of tile_w x tile_h pixels, samples innermost;  */
    uint32_t tile_h;         /*   0 = whole rows (tile_w = width, tile_h = 1)                  */
    uint32_t projection;     /* adaptive: after every accepted step p_theta is projected back
                                onto the ray's Carter constant; renders always do (1, the
                                default); 0 turns it off in sgx_trace_samples and
                                sgx_trace_invariants only (a diagnostic of the plain
                                integrator's drift); a render given 0 returns
                                SGX_ERR_UNSUPPORTED */
    uint32_t slice_count;    /* frame split (one frame over several GPUs): the rows are dealt in  */
    uint32_t slice_index;    /*   bands of slice_band rows, band b to slice b % slice_count; the  */
    uint32_t slice_band;     /*   render traces slice slice_index only and writes its rows packed
                                  top to bottom: width x sgx_slice_rows(...) pixels, each equal to
                                  the whole frame's pixel.  slice_count 0 or 1 = the whole frame;
                                  slice_band 0 = SGX_SLICE_BAND_DEFAULT.  sgx_render_device only. */
} sgx_render_opts;

#define SGX_SLICE_BAND_DEFAULT 8u

/* Counters of the last render (summed over its passes). */
typedef struct sgx_render_stats {
    uint64_t rays;        /* camera samples traced */
    uint64_t steps;       /* integrator steps taken (accepted + rejected) */
    uint64_t rejected;    /* adaptive: rejected attempts */
    uint64_t zone_steps;  /* mixed: steps taken with FP64 control */
    uint64_t budget_hits; /* rays that exhausted max_steps */
    float trace_ms;       /* device time of the trace kernel(s) of the last pass */
    float total_ms;       /* device time of the last pass, all kernels */
} sgx_render_stats;

/* The reference's Scene (render_backend.hpp:46-82), as C. */
typedef struct sgx_scene {
    uint32_t metric; /* SGX_METRIC_* */
    float mass_solar;
    float spin_a_over_M;
    float disc_inner_M;
    float disc_outer_M;
    uint32_t disc_doppler_on;
    uint32_t disc_redshift_on;
    uint32_t disc_texture_on;
    uint32_t show_overlay;
    uint32_t render_supersample;
    float exposure;
    float bloom_threshold;
    float bloom_strength;
    float disc_turbulence;
    float disc_peak_T_K;
    uint32_t max_steps;
    float h_step;
    uint32_t adaptive_step_on;
} sgx_scene;

/* The reference's CameraState (render_backend.hpp:84-99). */
typedef struct sgx_camera {
    float position[3];
    float basis[9]; /* row-major rows: right, up, -forward */
    float fov_y_radians;
} sgx_camera;

/* The reference's SceneConfig (core/include/scene/scene_config.hpp:39-58). */
typedef struct sgx_scene_config {
    float mass;
    float spin;
    float disc_r_inner;
    float disc_r_outer;
    uint32_t disc_doppler_on;
    uint32_t disc_redshift_on;
    float camera_fov_deg;
    float camera_distance;
    float camera_elevation;
    float h_step;
    int32_t max_steps;
} sgx_scene_config;

/* SceneLoadStatus (scene_config.hpp:60-65). */
typedef enum sgx_scene_status {
    SGX_SCENE_OK = 0,
    SGX_SCENE_FILE_NOT_FOUND = 1,
    SGX_SCENE_PARSE_ERROR = 2,
    SGX_SCENE_UNKNOWN_KEY = 3
} sgx_scene_status;

typedef struct sgx_context sgx_context;

/* ---- library ---------------------------------------------------------- */
int sgx_abi_version(void);
const char* sgx_status_string(sgx_status s);
void sgx_render_opts_default(sgx_render_opts* opts);

/* ---- host helpers (no GPU needed) ------------------------------------- */
/* Scene{} defaults (render_backend.hpp:46-82). */
void sgx_scene_default(sgx_scene* out);
/* build_orbital_camera (cuda_cli/main.cpp:68-109). */
void sgx_build_orbital_camera(sgx_camera* cam, float distance_M, float elevation_rad, float azimuth_rad,
                              float fov_y_deg);
/* pack_uniforms_cuda (render/cuda/cuda_backend.cu:45-101). */
void sgx_pack_uniforms(const sgx_scene* scene, const sgx_camera* cam, uint32_t width, uint32_t height,
                       float time_sec, sgx_uniforms* out);
/* SceneConfig defaults and load_scene_config_from_file / _from_stream
 * (scene_config.hpp:134-199).  On failure *line gets the 1-based line and
 * errbuf the offending line (or key, or path), as SceneLoadResult does. */
void sgx_scene_config_default(sgx_scene_config* out);
sgx_scene_status sgx_scene_config_load_file(const char* path, sgx_scene_config* out, int* line, char* errbuf,
                                            size_t errbuf_len);
sgx_scene_status sgx_scene_config_load_string(const char* text, sgx_scene_config* out, int* line,
                                              char* errbuf, size_t errbuf_len);
/* kerr_isco_prograde (core/include/physics/kerr.hpp:85-104). */
float sgx_kerr_isco_prograde(float mass, float spin);
/* Frame split (no counterpart in the reference, which renders a frame on one
 * GPU, render/cuda/cuda_backend.cu:140-152): the rows of slice `index` of
 * `count` (bands of `band` rows dealt round-robin; band 0 =
 * SGX_SLICE_BAND_DEFAULT): how many, and the frame row of its local row
 * `local` (UINT32_MAX when out of range). */
uint32_t sgx_slice_rows(uint32_t height, uint32_t band, uint32_t count, uint32_t index);
uint32_t sgx_slice_row(uint32_t height, uint32_t band, uint32_t count, uint32_t index, uint32_t local);

/* ---- context: CudaBackend lifecycle ----------------------------------- */
/* CudaBackend() + the device it runs on.  device < 0 -> the current device. */
sgx_status sgx_create(int device, sgx_context** out);
/* ~CudaBackend / shutdown() (cuda_backend.cu:107-127). */
void sgx_destroy(sgx_context* ctx);
/* initialize(RenderConfig) / resize() (cuda_backend.cu:111-138): sizes the
 * context's device image.  Rendering at another size resizes implicitly. */
sgx_status sgx_resize(sgx_context* ctx, uint32_t width, uint32_t height);
/* render_frame (cuda_backend.cu:140-152): traces u into the context's image.
 * opts may be NULL (reference behaviour).  With opts->sample_count set, one
 * call renders one progressive pass [sample_begin, sample_begin+count); the
 * image is final after the pass that reaches u->supersample. */
sgx_status sgx_render(sgx_context* ctx, const sgx_uniforms* u, const sgx_render_opts* opts);
/* capture_frame (cuda_backend.cu:154-166): copies the last image sgx_render
 * made to host memory in `format`; bytes must be width*height*(4 | 16 | 8).
 * Renders into a caller's buffer (sgx_render_device) leave the context's
 * image, and what sgx_capture and sgx_bloom see, unchanged. */
sgx_status sgx_capture(sgx_context* ctx, void* host_out, size_t bytes, uint32_t format);
/* Counters of the last sgx_render. */
sgx_status sgx_get_stats(const sgx_context* ctx, sgx_render_stats* out);
/* Message of the last failed call on ctx (never NULL). */
const char* sgx_last_error(const sgx_context* ctx);

/* Kernel-level entry: the work of singularity_geodesic_kernel<<<>>>
 * (geodesic_kernel.cu:462) into a caller-owned device buffer d_out (format as
 * given), on the caller's cudaStream_t (passed as void*; NULL = the context's
 * stream).  Scratch memory comes from the context. */
sgx_status sgx_render_device(sgx_context* ctx, const sgx_uniforms* u, const sgx_render_opts* opts, void* d_out,
                             uint32_t format, void* stream);

/* Parity probe: trace n individual samples (pixel gx, gy, Halton index s) and
 * return their HDR colour (before exposure and tone map), integrator steps and
 * termination kind (0 horizon, 1 escape, 2 disc, 3 budget, 4 cold disc,
 * 5 no root) — the per-sample values of geodesic_kernel.cu:483-501.  Host
 * arrays; any output may be NULL. */
sgx_status sgx_trace_samples(sgx_context* ctx, const sgx_uniforms* u, const sgx_render_opts* opts, uint64_t n,
                             const uint32_t* gx, const uint32_t* gy, const uint32_t* s, float* hdr3,
                             uint32_t* steps, uint32_t* term);

/* Constants of motion of n samples traced as sgx_trace_samples traces them,
 * for the error-controlled Kerr integrator (opts->integrator ADAPTIVE, Kerr
 * uniforms; anything else is SGX_ERR_UNSUPPORTED).  No counterpart in the
 * reference, whose Carter-constant claim (README.md:97) no code measures.
 * inv5 (host, n x 5 doubles) gets per sample, evaluated in FP64: E, L_z, the
 * Carter constant Q0 the ray started with (the FP32 form's FP32 value, the
 * mixed and FP64 forms' FP64 value), the Carter constant of the ray's last
 * state and 2H of that state (kerr_hamilton.h:37-60); a sample whose camera
 * ray has no root gets NaNs.  term (may be NULL) as in sgx_trace_samples. */
sgx_status sgx_trace_invariants(sgx_context* ctx, const sgx_uniforms* u, const sgx_render_opts* opts, uint64_t n,
                                const uint32_t* gx, const uint32_t* gy, const uint32_t* s, double* inv5,
                                uint32_t* term);

/* ---- HDR bloom and display transform ------------------------------------------ */
/* The realtime backends' post-process (render/vulkan/shaders/bloom.hlsl:8-77,
 * blit.hlsl:43-57), which the reference's CUDA path lacks: on the last frame,
 * rendered in SGX_FORMAT_RGBA16F_HDR (the per-pixel mean HDR colour), a
 * half-resolution Karis-weighted extract with a soft-knee threshold, a
 * separable blur, and the compose hdr + bloom * strength, times exposure,
 * ACES, then sRGB (RGBA8) or linear (RGBA32F).  Capture the result with
 * sgx_capture in that format.  The extract at the uniforms' threshold is made
 * by the render itself (sgx_render in SGX_FORMAT_RGBA16F_HDR fuses it into
 * its last accumulation pass), so with threshold < 0 the first call after a
 * render blurs and composes only; a threshold of the caller's own, or a
 * later call on the same frame, extracts again from the HDR frame. */
typedef struct sgx_bloom_opts {
    uint32_t struct_size;
    float sigma_px;  /* blur sigma in full-resolution pixels; <= 0: the reference's 7-tap kernel */
    float threshold; /* < 0: the uniforms' bloom_threshold */
    float strength;  /* < 0: the uniforms' bloom_strength */
    uint32_t format; /* SGX_FORMAT_RGBA8_SRGB or SGX_FORMAT_RGBA32F */
} sgx_bloom_opts;
sgx_status sgx_bloom(sgx_context* ctx, const sgx_bloom_opts* opts);

/* ---- batched views ----------------------------------------------------------- */
/* No counterpart in the reference (one view per launch there,
 * render/cuda/cuda_backend.cu:140-152).  A batch is 1..SGX_BATCH_MAX_VIEWS
 * views of one metric, each with its own size, scene, camera and samples per
 * pixel, traced by ONE persistent launch over a shared ray queue; creation
 * captures the whole frame set (counters, per-view constants, trace,
 * accumulation, encode) into a CUDA graph that sgx_batch_launch replays.
 * Frames are packed view after view in one device buffer (pixel offsets from
 * sgx_batch_output), in `format` (RGBA8 sRGB or RGBA32F).  opts may be NULL;
 * sample_begin/sample_count must be 0 (every sample of every view). */
#define SGX_BATCH_MAX_VIEWS 128u
typedef struct sgx_batch sgx_batch;
sgx_status sgx_batch_create(sgx_context* ctx, const sgx_uniforms* views, uint32_t n, const sgx_render_opts* opts,
                            uint32_t format, sgx_batch** out);
/* New uniforms for the same views (each view keeps its size, samples and
 * metric); the next launch renders them. */
sgx_status sgx_batch_update(sgx_batch* b, const sgx_uniforms* views);
/* Replays the graph on `stream` (NULL: the context's stream); asynchronous. */
sgx_status sgx_batch_launch(sgx_batch* b, void* stream);
/* Waits for the last launch; stats (may be NULL) get its counters and time. */
sgx_status sgx_batch_wait(sgx_batch* b, sgx_render_stats* stats);
/* Device pointer of the packed frames and the n + 1 pixel offsets of the views. */
sgx_status sgx_batch_output(const sgx_batch* b, const void** d_frames, uint64_t* pixel_offsets);
/* Copies view `view`'s frame to host memory (waits for the last launch). */
sgx_status sgx_batch_capture(sgx_batch* b, uint32_t view, void* host_out, size_t bytes);
void sgx_batch_destroy(sgx_batch* b);
/* Launch-shape autotuner: times every combination of threads per block
 * {64, 128, 256}, refill interval {16, 32, 64, 128} and ray-order tile {rows, 8x4,
 * 16x8, 32x2} on the views with samples capped at sample_cap (0: 4) and writes
 * the fastest into *best (other fields from base); *best_ms gets its time. */
sgx_status sgx_autotune(sgx_context* ctx, const sgx_uniforms* views, uint32_t n, const sgx_render_opts* base,
                        uint32_t sample_cap, sgx_render_opts* best, float* best_ms);

/* ---- allocation-free render ------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory — host applications (game engines, plug-in renderers) that reserve
 * the GPU's memory for their own pool at start-up and forbid allocations by
 * libraries, and frame-paced callers that cannot take the device-wide
 * synchronisation of cudaFree mid-frame — this renders one whole frame (all
 * samples, fixed-step integrator, FP32 or FP64) into the caller's device
 * buffer d_out on the caller's stream without allocating anything: its
 * scratch is a fixed SGX_NOALLOC_SCRATCH_BYTES array inside the library, held
 * by every GPU that loads the library until exit.  A frame needs
 * 4096 + align256(16 * width * height) + R * width * height * spp bytes of it
 * (R = 16 for FP32, 32 for FP64; align256 rounds up to a multiple of 256);
 * larger frames return SGX_ERR_INVALID_ARGUMENT with the reason in err (a
 * caller buffer, may be NULL).  The first call on a device does a one-time
 * set-up (looks up the array's device address) and should come before any
 * stream capture.  Calls share the array: calls whose GPU work overlaps race,
 * so issue them on one stream. */
#define SGX_NOALLOC_SCRATCH_BYTES (64ull << 20)
sgx_status sgx_render_noalloc(const sgx_uniforms* u, const sgx_render_opts* opts, void* d_out, uint32_t format,
                              void* stream, char* err, size_t err_len);

/* ---- differentiable render and its adjoint ---------------------------------- */
/* No counterpart in the reference.  A Kerr render form that is differentiable
 * in four scene parameters, and the gradient of an image loss with respect to
 * them by a reverse (adjoint) sweep of the fixed-step RK4 with a state
 * checkpoint every 64 steps.  The form keeps the reference's integrator
 * (kerr_hamilton.h:97-178), escape test and disc shading
 * (geodesic_kernel.cu:300-401) and changes what makes the image discontinuous
 * in the parameters:
 *   - the camera orbits at azimuth 0, its frame a closed-form function of the
 *     inclination; the starfield is off;
 *   - the disc (SGX_DIFF_MODEL_SLAB, the default) is an emitting, absorbing
 *     layer of half-thickness H = half_thickness * M with the vertical profile
 *     (1 - (z/H)^2)^2: every RK4 step inside it absorbs
 *     alpha = w (1 - exp(-kappa rho ds)) (ds the step's length, kappa set so
 *     that a perpendicular pass has optical depth tau_perp) and adds
 *     tau alpha c to the colour, tau the ray's transmittance;
 *     SGX_DIFF_MODEL_CROSSING keeps the reference's equatorial crossings,
 *     each emitting with weight w through the transmittance (its image jumps
 *     where a ray grazes the plane, so only r_in and t_scale are smooth);
 *   - w = S((r - r_in)/e) S((r_out - r)/e) softens the annulus edges (S the
 *     cubic smoothstep, e = edge_width * M); with fade_start > 0, w is also
 *     multiplied by 1 - S((psi - fade_start)/fade_width), psi the angle the ray
 *     has swept around the hole.  Rays that pass close to the photon orbit
 *     before reaching the disc move on parameter scales below 1e-3 (their
 *     bending grows like -log(b - b_c)), which no finite difference and no
 *     FP32 trace resolves; they all sweep more than ~3 pi / 4, so the default
 *     fade (5 pi / 8, pi / 8) keeps the direct image of the disc out to that
 *     angle and drops them;
 *   - the blackbody fit is blended across its 6600 K branch switch;
 *   - rays are captured inside the prograde photon orbit radius less 0.05 M
 *     (the reference's 1.02 r_+ lets the fixed-step RK4 blow up first).
 * The image is W x H x 3 floats, per pixel the mean over samples of
 * ACES(hdr * exposure) (the reference's tone map, before sRGB encoding). */
typedef struct sgx_diff_params {
    double spin;     /* a / M, in [0, 1) */
    double incl;     /* inclination of the camera from the spin axis, radians, in (0, pi) */
    double r_in;     /* disc inner radius, units of M */
    double t_scale;  /* multiplies the disc's peak temperature */
} sgx_diff_params;
#define SGX_DIFF_MODEL_CROSSING 0u
#define SGX_DIFF_MODEL_SLAB 1u
/* How the backward pass multiplies by a step's Jacobian: the hand-derived
 * reverse pass (default), or the Jacobian built with 9-lane dual numbers
 * (slower; kept as the cross-check of the first). */
#define SGX_DIFF_ADJOINT_REVERSE 0u
#define SGX_DIFF_ADJOINT_DUAL 1u
typedef struct sgx_diff_opts {
    uint32_t struct_size;
    uint32_t precision;    /* SGX_PRECISION_FP32 or SGX_PRECISION_FP64 */
    float edge_width;      /* soft annulus edge, units of M (0.1) */
    float fade_start;      /* swept angle where images fade, rad (5 pi / 8); <= 0: no fade */
    float fade_width;      /* fade length, rad (pi / 8) */
    uint32_t model;        /* SGX_DIFF_MODEL_SLAB (default) or SGX_DIFF_MODEL_CROSSING */
    float half_thickness;  /* slab half-thickness, units of M (0.3) */
    float tau_perp;        /* slab optical depth across (4) */
    uint32_t adjoint_form; /* SGX_DIFF_ADJOINT_REVERSE (default) or SGX_DIFF_ADJOINT_DUAL */
    uint32_t checkpoint_interval; /* steps between the forward's checkpoints: 0 (default) = 10 for FP32
                                     with the reverse-pass adjoint when its records fit the form's 16 GiB
                                     budget (the adjoint keeps its recomputed segment in shared
                                     memory), else 64 (segment in thread-local memory); or 10 or 64 */
} sgx_diff_opts;
void sgx_diff_opts_default(sgx_diff_opts* opts);
/* Forward pass: renders the form for `params` with size, samples, distance
 * (|cam_pos|), field of view, mass, r_out, peak temperature, step, max_steps,
 * escape radius, exposure, turbulence, time and the Doppler/redshift flags
 * from `base` (a Kerr uniform block), into d_image (device, W*H*3 floats; NULL:
 * an internal buffer) and keeps what the backward pass needs (a state and
 * transmittance checkpoint every C = opts->checkpoint_interval steps,
 * (max_steps/C + 1) * 9 values per ray).  Synchronous. */
sgx_status sgx_diff_forward(sgx_context* ctx, const sgx_uniforms* base, const sgx_diff_params* params,
                            const sgx_diff_opts* opts, float* d_image, void* stream);
/* Backward pass of the last forward: d_grad_image (device, W*H*3 floats) is
 * dLoss/dImage; grad[4] (host) receives dLoss/d(spin, incl, r_in, t_scale).
 * The per-ray terms are summed in a fixed order (deterministic). */
sgx_status sgx_diff_backward(sgx_context* ctx, const float* d_grad_image, double* grad, void* stream);
/* Rays and RK4 steps of the last forward, and (crossing model) how many
 * crossings beyond the 8 recorded per ray were left out of the backward pass. */
sgx_status sgx_diff_stats(sgx_context* ctx, uint64_t* rays, uint64_t* steps, uint64_t* crossing_overflow);
/* Steps between the checkpoints of the last forward (10 or 64; 0 before one). */
uint32_t sgx_diff_checkpoint_steps(const sgx_context* ctx);

/* ---- measurement --------------------------------------------------------- */
/* No counterpart in the reference: the device's FP32 FMA issue ceiling in
 * TFLOP/s (2 flops per FMA), measured with a register-resident FMA kernel of
 * `iters` iterations on `device` (< 0: current).  The roofline denominator of
 * the tracer, whose work is FP32 SIMT arithmetic. */
sgx_status sgx_measure_fp32_peak(int device, int iters, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* SGX_H */
