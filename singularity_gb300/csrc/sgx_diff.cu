// singularity_gb300/csrc/sgx_diff.cu
//
// Differentiable render form and its adjoint (no counterpart in the
// reference): the C ABI (sgx_diff_*) and the FP32 instantiations; kernels in
// sgx_diff_impl.cuh, FP64 instantiations in sgx_diff64.cu.  The form is
// specified operation for operation by the CPU oracle oracle/diff_oracle.hpp:
// the reference's fixed-step Kerr RK4 with pole damping
// (kerr_hamilton.h:165-178), the camera at azimuth 0 with the inclination as
// a parameter, starfield off, an emitting and absorbing slab disc (or the
// reference's equatorial crossings) with soft annulus edges and a
// transmittance, and a fade of images that wind past a swept angle.
// Parameters: spin a/M, inclination, disc inner radius, temperature scale.
//
// Forward: one thread per (pixel, sample) ray.  Each ray stores its state and
// transmittance every 10 or 64 steps (structure-of-arrays checkpoints in HBM,
// component-major so neighbouring rays write neighbouring words), its last
// emitting step (slab) or its crossings (crossing model), and its HDR colour;
// an image kernel averages ACES(hdr * exposure) per pixel.
//
// Adjoint: given dLoss/dImage, each ray seeds dLoss/dhdr and sweeps the steps
// backwards from its last emitting step, one checkpoint segment at a time
// (the segment's states recomputed from its checkpoint into shared memory
// for 10-step segments, thread-local memory for 64-step ones).  Emission terms go through the transmittance chain with their
// local derivatives from dual numbers (sgx_dual.cuh); the adjoint vector is
// carried through each RK4 step by the hand-derived reverse pass of
// sgx_adjoint.cuh (or, as a cross-check, by the step's Jacobian built with
// dual numbers); the camera set-up is differentiated with dual numbers.
// Per-ray gradients are summed in a fixed order, so the result is
// deterministic.

#include "sgx_diff_impl.cuh"

using sgx_internal::cuda_fail;
using sgx_internal::fail;

cudaError_t sgx_diff_run_forward_f32(sgx_diff_state& st, float* img, cudaStream_t s) {
    return run_forward<float>(st, img, s);
}
cudaError_t sgx_diff_run_backward_f32(sgx_diff_state& st, const float* gimg, double* d_out4, cudaStream_t s) {
    return run_backward<float>(st, gimg, d_out4, s);
}

extern "C" {

void sgx_diff_opts_default(sgx_diff_opts* o) {
    if (o == nullptr) return;
    std::memset(o, 0, sizeof(*o));
    o->struct_size = sizeof(*o);
    o->precision = SGX_PRECISION_FP32;
    o->edge_width = 0.1f;
    o->fade_start = 1.96349540849362f;  // 5 pi / 8
    o->fade_width = 0.39269908169872f;  // pi / 8
    o->model = SGX_DIFF_MODEL_SLAB;
    o->half_thickness = 0.3f;
    o->tau_perp = 4.0f;
}

sgx_status sgx_diff_forward(sgx_context* c, const sgx_uniforms* base, const sgx_diff_params* params,
                            const sgx_diff_opts* opts, float* d_image, void* stream) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (base == nullptr || params == nullptr) return fail(c, SGX_ERR_INVALID_ARGUMENT, "NULL uniforms or params");
    if (base->metric_type != SGX_METRIC_KERR) return fail(c, SGX_ERR_INVALID_ARGUMENT, "the differentiable form is Kerr");
    if (base->width == 0 || base->height == 0) return fail(c, SGX_ERR_INVALID_ARGUMENT, "empty image");
    if (base->max_steps == 0 || base->max_steps > 200000)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "max_steps must be in [1, 200000]");
    sgx_diff_opts o;
    sgx_diff_opts_default(&o);
    if (opts != nullptr) {
        if (opts->struct_size != sizeof(sgx_diff_opts))
            return fail(c, SGX_ERR_INVALID_ARGUMENT, "sgx_diff_opts.struct_size mismatch");
        o = *opts;
    }
    if (o.precision != SGX_PRECISION_FP32 && o.precision != SGX_PRECISION_FP64)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "the differentiable form runs in FP32 or FP64");
    if (o.model != SGX_DIFF_MODEL_SLAB && o.model != SGX_DIFF_MODEL_CROSSING)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown disc model");
    if (!(o.edge_width > 0.0f) || (o.fade_start > 0.0f && !(o.fade_width > 0.0f)))
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "edge_width and fade_width must be positive");
    if (o.adjoint_form != SGX_DIFF_ADJOINT_REVERSE && o.adjoint_form != SGX_DIFF_ADJOINT_DUAL)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "unknown adjoint_form");
    if (o.checkpoint_interval != 0u && o.checkpoint_interval != std::uint32_t(kCkDense) &&
        o.checkpoint_interval != std::uint32_t(kCkSparse))
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "checkpoint_interval must be 0 (automatic), 10 or 64");
    const bool dense_ok = o.precision == SGX_PRECISION_FP32 && o.adjoint_form == SGX_DIFF_ADJOINT_REVERSE;
    if (o.checkpoint_interval == std::uint32_t(kCkDense) && !dense_ok)
        return fail(c, SGX_ERR_UNSUPPORTED, "10-step checkpoints apply to FP32 with the reverse-pass adjoint");
    if (o.model == SGX_DIFF_MODEL_SLAB && !(o.half_thickness > 0.0f && o.tau_perp > 0.0f))
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "half_thickness and tau_perp must be positive");
    if (!(params->spin >= 0.0 && params->spin < 1.0) || !(params->incl > 0.0 && params->incl < 3.14159265) ||
        !(params->r_in > 0.0) || !(params->t_scale > 0.0))
        return fail(c, SGX_ERR_INVALID_ARGUMENT,
                    "parameters out of range (0 <= spin < 1, 0 < incl < pi, r_in > 0, t_scale > 0)");
    cudaSetDevice(c->device);
    if (c->diff == nullptr) c->diff = new sgx_diff_state();
    sgx_diff_state& st = *c->diff;
    st.valid = false;
    const std::uint32_t spp = base->supersample < 1u ? 1u : (base->supersample > 1024u ? 1024u : base->supersample);
    st.n = std::uint64_t(base->width) * base->height * spp;
    st.precision = o.precision;
    st.nx = o.model == SGX_DIFF_MODEL_SLAB ? 1u : std::uint32_t(kMaxCross);
    auto bytes_for = [&](std::uint32_t ck) {
        const std::uint32_t slots = base->max_steps / ck + 1;
        return o.precision == SGX_PRECISION_FP64 ? state_bytes<double>(st.n, slots, spp, st.nx)
                                                 : state_bytes<float>(st.n, slots, spp, st.nx);
    };
    const std::size_t limit = c->workspace_budget * 4;
    std::uint32_t ck = o.checkpoint_interval;
    if (ck == 0u)
        ck = dense_ok && bytes_for(std::uint32_t(kCkDense)) <= limit ? std::uint32_t(kCkDense)
                                                                      : std::uint32_t(kCkSparse);
    st.ck = ck;
    st.slots = base->max_steps / ck + 1;
    const std::size_t need = bytes_for(ck);
    if (need > limit)
        return fail(c, SGX_ERR_INVALID_ARGUMENT, "differentiable render needs " + std::to_string(need >> 20) +
                                                     " MiB of records: fewer rays or max_steps");
    if (st.cap < need) {
        if (st.mem) cudaFree(st.mem);
        st.mem = nullptr;
        st.cap = 0;
        cudaError_t e = cudaMalloc(&st.mem, need);
        if (e != cudaSuccess) return cuda_fail(c, e, "sgx_diff_forward: cudaMalloc");
        st.cap = need;
    }
    const std::size_t img_bytes = std::size_t(base->width) * base->height * 3 * sizeof(float);
    if (d_image == nullptr) {
        if (st.img_cap < img_bytes) {
            if (st.img) cudaFree(st.img);
            st.img = nullptr;
            st.img_cap = 0;
            cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&st.img), img_bytes);
            if (e != cudaSuccess) return cuda_fail(c, e, "sgx_diff_forward: cudaMalloc");
            st.img_cap = img_bytes;
        }
        d_image = st.img;
    }
    st.u = *base;
    st.p = *params;
    st.o = o;
    cudaStream_t s = stream != nullptr ? static_cast<cudaStream_t>(stream) : c->stream;
    cudaError_t e = o.precision == SGX_PRECISION_FP64 ? sgx_diff_run_forward_f64(st, d_image, s)
                                                      : sgx_diff_run_forward_f32(st, d_image, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_diff_forward");
    st.valid = true;
    return SGX_OK;
}

sgx_status sgx_diff_backward(sgx_context* c, const float* d_grad_image, double* grad4, void* stream) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (d_grad_image == nullptr || grad4 == nullptr) return fail(c, SGX_ERR_INVALID_ARGUMENT, "NULL argument");
    if (c->diff == nullptr || !c->diff->valid)
        return fail(c, SGX_ERR_NOT_RENDERED, "sgx_diff_backward needs a preceding sgx_diff_forward");
    cudaSetDevice(c->device);
    sgx_diff_state& st = *c->diff;
    cudaStream_t s = stream != nullptr ? static_cast<cudaStream_t>(stream) : c->stream;
    // results land after the reduction scratch
    const std::uint32_t spp = st.u.supersample < 1u ? 1u : (st.u.supersample > 1024u ? 1024u : st.u.supersample);
    const std::size_t used = st.precision == SGX_PRECISION_FP64 ? state_bytes<double>(st.n, st.slots, spp, st.nx)
                                                                : state_bytes<float>(st.n, st.slots, spp, st.nx);
    double* d_out4 = reinterpret_cast<double*>(static_cast<unsigned char*>(st.mem) + used - 256);
    cudaError_t e = st.precision == SGX_PRECISION_FP64 ? sgx_diff_run_backward_f64(st, d_grad_image, d_out4, s)
                                                       : sgx_diff_run_backward_f32(st, d_grad_image, d_out4, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad4, d_out4, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_diff_backward");
    return SGX_OK;
}

sgx_status sgx_diff_stats(sgx_context* c, uint64_t* rays, uint64_t* steps, uint64_t* crossing_overflow) {
    if (c == nullptr) return SGX_ERR_INVALID_ARGUMENT;
    if (c->diff == nullptr || !c->diff->valid) return fail(c, SGX_ERR_NOT_RENDERED, "no differentiable render");
    sgx_diff_state& st = *c->diff;
    if (rays != nullptr) *rays = st.n;
    const std::uint32_t spp = st.u.supersample < 1u ? 1u : (st.u.supersample > 1024u ? 1024u : st.u.supersample);
    unsigned long long h[2] = {0, 0};
    void* ov = st.precision == SGX_PRECISION_FP64 ? static_cast<void*>(carve_bufs<double>(st, spp).overflow)
                                                  : static_cast<void*>(carve_bufs<float>(st, spp).overflow);
    cudaError_t e = cudaMemcpy(h, ov, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "sgx_diff_stats");
    if (steps != nullptr) *steps = h[1];
    if (crossing_overflow != nullptr) *crossing_overflow = h[0];
    return SGX_OK;
}

uint32_t sgx_diff_checkpoint_steps(const sgx_context* c) {
    return c != nullptr && c->diff != nullptr && c->diff->valid ? c->diff->ck : 0u;
}

}  // extern "C"

void sgx_internal_free_diff(sgx_context* c) {
    if (c == nullptr || c->diff == nullptr) return;
    if (c->diff->mem) cudaFree(c->diff->mem);
    if (c->diff->img) cudaFree(c->diff->img);
    delete c->diff;
    c->diff = nullptr;
}
