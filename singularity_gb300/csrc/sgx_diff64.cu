// singularity_gb300/csrc/sgx_diff64.cu
//
// FP64 instantiations of the differentiable form's kernels (the kernels and
// the method are in sgx_diff_impl.cuh and sgx_diff.cu); a separate
// translation unit so it compiles in parallel with the FP32 one.
#include "sgx_diff_impl.cuh"

cudaError_t sgx_diff_run_forward_f64(sgx_diff_state& st, float* img, cudaStream_t s) {
    return run_forward<double>(st, img, s);
}
cudaError_t sgx_diff_run_backward_f64(sgx_diff_state& st, const float* gimg, double* d_out4, cudaStream_t s) {
    return run_backward<double>(st, gimg, d_out4, s);
}
