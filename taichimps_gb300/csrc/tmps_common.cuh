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
