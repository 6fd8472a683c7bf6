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

// Self-check of the integer-operation conversions (tmps_common.cuh) against
// the hardware's rounding, on the caller's operands: mine[i] and hw[i] must
// agree bit for bit.  No reference counterpart.
//   which 0: (float)a[i]             f32_rn    vs the hardware conversion (float bits)
//   which 1: (double)(float)a[i]     f64_of    vs the hardware widening
//   which 2: hi, lo split of a[i]    split_dw  vs the hardware's (float bits, two outputs per operand)
namespace {

__global__ void k_selftest(int which, const double* __restrict__ a, int n, double* __restrict__ mine,
                           double* __restrict__ hw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i];
    switch (which) {
        case 0:
            mine[i] = (double)__float_as_uint(f32_rn(x));
            hw[i] = (double)__float_as_uint(__double2float_rn(x));
            break;
        case 1: {
            const float f = __double2float_rn(x);
            mine[i] = f64_of(f);
            hw[i] = (double)f;
            break;
        }
        default: {
            float h, l;
            split_dw(x, h, l);
            const float hh = __double2float_rn(x);
            const float ll = __double2float_rn(x - (double)hh);
            mine[2 * i] = (double)__float_as_uint(h);
            mine[2 * i + 1] = (double)__float_as_uint(l);
            hw[2 * i] = (double)__float_as_uint(hh);
            hw[2 * i + 1] = (double)__float_as_uint(ll);
            break;
        }
    }
}

}  // namespace

extern "C" int tmps_selftest_arith(int32_t which, const double* d_a, int32_t n, double* d_mine, double* d_hw,
                                   void* stream) {
    if (which < 0 || which > 2 || n < 0 || !d_a || !d_mine || !d_hw) return TMPS_ERR_BAD_ARG;
    if (n == 0) return TMPS_OK;
    k_selftest<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(which, d_a, n, d_mine, d_hw);
    note_launches(1);
    return cudaPeekAtLastError() == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}
