// FP32 issue-rate probe: the roofline denominator for the narrow phase, which is FP32-pipe bound
// and compiled without FMA contraction (one FMUL or FADD per lane per instruction).  Eight
// independent multiply/add chains per thread keep the pipe busy; the result is written so the work
// cannot be removed.
#include "common.cuh"

namespace mwd {
namespace {

__global__ void __launch_bounds__(256) fp32_probe_kernel(int iters, float* out)
{
    float a[8], b = 1.0000001f + threadIdx.x * 1e-9f, c = 1e-7f;
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = a[k] * b + c;  // FMUL + FADD (no contraction)
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678f) out[blockIdx.x] = s;
}

}  // namespace
}  // namespace mwd

extern "C" int mwd_probe_fp32(int32_t iters, float* scratch, double* tflops_out, mwd_stream_t stream)
{
    using namespace mwd;
    if (iters < 1 || !scratch || !tflops_out) {
        set_error("mwd_probe_fp32: bad arguments");
        return MWD_ERR_INVALID;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int blocks = num_sms() * 8;
    cudaEvent_t e0, e1;
    MWD_CUDA(cudaEventCreate(&e0));
    MWD_CUDA(cudaEventCreate(&e1));
    fp32_probe_kernel<<<blocks, 256, 0, s>>>(iters, scratch);  // warm-up
    MWD_CUDA(cudaEventRecord(e0, s));
    fp32_probe_kernel<<<blocks, 256, 0, s>>>(iters, scratch);
    MWD_CUDA(cudaEventRecord(e1, s));
    MWD_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    MWD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double ops = (double)blocks * 256.0 * (double)iters * 8.0 * 2.0;
    *tflops_out = ops / (ms * 1e-3) / 1e12;
    return MWD_OK;
}
