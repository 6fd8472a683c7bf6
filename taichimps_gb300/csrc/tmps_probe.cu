// FP64 pipe probe: the denominator of the FP64 form's roofline.
//
// This part's FP64 pipe is far narrower than its FP32 pipe, so the plain
// FP64 form of the step is bound by FP64 instruction issue rather than by
// HBM.  tmps_probe_fp64 runs eight independent DFMA chains per thread over a
// grid of the caller's choosing (a multiple of the SM count fills the part);
// the caller times it and counts 8 * iters * blocks * threads DFMA (two
// flops each).  Each thread writes one double to d_out (blocks * threads
// slots, caller memory).  No reference counterpart.
#include "tmps_common.cuh"

using namespace tmps;

namespace {

__global__ void __launch_bounds__(256) k_probe_dfma(double* __restrict__ out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1e-6 * (double)threadIdx.x + 1e-3 * (double)k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int tmps_probe_fp64(int32_t blocks, int32_t threads, int32_t iters, double* d_out, void* stream) {
    if (blocks < 1 || threads < 32 || threads > 256 || threads % 32 || iters < 1 || !d_out) return TMPS_ERR_BAD_ARG;
    k_probe_dfma<<<blocks, threads, 0, (cudaStream_t)stream>>>(d_out, iters, 0.999999, 1e-7);
    note_launches(1);
    return cudaPeekAtLastError() == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}
