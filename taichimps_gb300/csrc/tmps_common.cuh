// Shared device helpers for the GB300 DEM contact path (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/taichimps_gb300.h"

#define TMPS_DEV __device__ __forceinline__

// Bits 27..31 of a neighbor entry carry the stencil offset of the partner's
// cell relative to the row atom's cell, (ox+1) + 3 (oy+1) + 9 (oz+1); the low
// 27 bits are the partner's internal index (n < 2^27 atoms).
constexpr int kNbrIndexBits = 27;
constexpr int32_t kNbrIndexMask = (1 << kNbrIndexBits) - 1;
constexpr int kMaxSlots = 64;  // one bit per slot in the touch mask

namespace tmps {

// Number of kernels this library has launched (all entry points, all
// threads); read through tmps_launch_count().
void note_launches(int k);

inline int grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    return (int)(g < 1 ? 1 : g);
}

// A double as an FP32 value from its bits alone: the sign, the exponent
// rebiased and the top 20 bits of the significand (the rest truncated), so
// the relative error is below 2^-20; zero below the FP32 normal range,
// infinity above it, NaN kept.  Integer operations only: on this part a
// double -> float conversion issues on the narrow FP64 pipe, and screens that
// reject far pairs before an exact FP64 test do not need a rounded value.
TMPS_DEV float approx_f32(double x) {
    const uint32_t hi = (uint32_t)__double2hiint(x);
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const uint32_t m = hi & 0xfffffu;
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
    const int ef = e - 1023 + 127;
    if (ef <= 0) return __uint_as_float(sign);
    if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((uint32_t)ef << 23) | (m << 3));
}

// |a| + |b| + |c|
TMPS_DEV float l1f(float a, float b, float c) { return (fabsf(a) + fabsf(b)) + fabsf(c); }

// Conversions between double and float done with integer operations, which
// issue on the wide integer pipes instead of this part's narrow FP64 pipe.
// Both give the same bits as the hardware conversion; the rare operands
// outside the plain case (results below the FP32 normal range, infinities,
// NaNs) go to the hardware conversion.

// isfinite(x) from the exponent bits
TMPS_DEV bool finite_bits(double x) { return ((__double2hiint(x) >> 20) & 0x7ff) != 0x7ff; }

// (float)x, round to nearest even
TMPS_DEV float f32_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    if ((b << 1) == 0ull) return __uint_as_float(sign);  // +-0
    const int e = (int)((b >> 52) & 0x7ff);
    const int ef = e - 1023 + 127;
    if (e == 0x7ff || ef <= 0 || ef >= 255) return (float)x;
    const unsigned long long m = b & 0xfffffffffffffull;
    uint32_t keep = (uint32_t)(m >> 29);
    const uint32_t rest = (uint32_t)(m & 0x1fffffffull);
    if (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) ++keep;
    // a carry out of the significand steps the exponent (to infinity past the top)
    return __uint_as_float(sign | (((uint32_t)ef << 23) + keep));
}

// (double)f, exact
TMPS_DEV double f64_of(float f) {
    const uint32_t u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const uint32_t e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) {
        if ((u << 1) == 0u) return __longlong_as_double((long long)sign);  // +-0
        return (double)f;
    }
    const unsigned long long m = (unsigned long long)(u & 0x7fffffu) << 29;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e - 127 + 1023) << 52) | m));
}

// hi + lo of a double as two floats: hi = (float)v, lo = (float)(v - hi)
// (v - hi is exact in FP64)
TMPS_DEV void split_dw(double v, float& hi, float& lo) {
    hi = f32_rn(v);
    lo = f32_rn(__dsub_rn(v, f64_of(hi)));
}

TMPS_DEV double4 ld4(const double* p, int i) { return reinterpret_cast<const double4*>(p)[i]; }
TMPS_DEV void st4(double* p, int i, double4 v) { reinterpret_cast<double4*>(p)[i] = v; }
TMPS_DEV float4 ld4f(const float* p, int i) { return reinterpret_cast<const float4*>(p)[i]; }
TMPS_DEV void st4f(float* p, int i, float4 v) { reinterpret_cast<float4*>(p)[i] = v; }

// Block-wide sum of `nv` doubles held per thread; the result lands in
// out[0..nv) of thread 0.  Fixed tree order: deterministic for a given
// block size.
template <int NV, int BLOCK>
TMPS_DEV void block_sum(double (&v)[NV], double* smem /* [NV][BLOCK/32] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double s = v[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) smem[c * (BLOCK / 32) + warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            double s = lane < BLOCK / 32 ? smem[c * (BLOCK / 32) + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            v[c] = s;
        }
    }
}

}  // namespace tmps
