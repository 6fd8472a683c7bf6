// The fused step: Simulation._sub_step_inner (simulation.py:205-247) for
// fix nve/sphere + optional damping/cundall + optional deform/pressure, as
// three launches per step with no host round trip (see tmps_engine in the
// header).
//
//   A  final half-kick of the previous step, pending remap x, first
//      half-kick, drift, skin check          (nve_sphere.py:44-96,
//                                             deform_pressure.py:512-530,
//                                             neighbor.py:242-245)
//   C  contact law + Cundall damping + pair and kinetic virial
//                                            (GRANULAR/*, damping_cundall.py:36-53,
//                                             thermo.py:89-102)
//   S  rebuild decision, virial total, servo (neighbor.py:371-403,
//                                             deform_pressure.py:598-702)
//
// Two arithmetic forms share the launch structure:
//   FP64:  absolute FP64 positions, every operation FP64 (divisions by m and
//          I become products with 1/m, 1/I computed at each rebuild).
//   mixed: split positions (FP64 offset from the atom's cell origin at the
//          last build), FP32 contact arithmetic and FP32 per-atom force
//          accumulation; FP64 kept for the velocity and position updates, the
//          per-contact shear history and the virial reduction.
#include "tmps_contact.cuh"
#include "tmps_servo.cuh"

using namespace tmps;

namespace {

constexpr int kBlockA = 256;
constexpr int kBlockC = 128;

// Error-free transformations in FP32 (Knuth's two-sum; FMA for products):
// s + e == a + b exactly.  Used to form the separation and the overlap of a
// near-contact pair to ~2^-48 relative precision out of FP32 words.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// hi + lo of a double as two floats (integer-op conversions: off the FP64 pipe)
__device__ __forceinline__ void split(double v, float& hi, float& lo) { split_dw(v, hi, lo); }

// |a| >= |b| (or a == 0): s + e == a + b exactly
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// (hi, lo) += b for a double-word value hi + lo
__device__ __forceinline__ void dw_add(float& hi, float& lo, float b) {
    float s, e;
    two_sum(hi, b, s, e);
    fast_two_sum(s, __fadd_rn(e, lo), hi, lo);
}

// (hi, lo) += (bh, bl)
__device__ __forceinline__ void dw_add2(float& hi, float& lo, float bh, float bl) {
    float s, e;
    two_sum(hi, bh, s, e);
    fast_two_sum(s, __fadd_rn(e, __fadd_rn(lo, bl)), hi, lo);
}

// (hi, lo) += (ah + al) * (bh + bl), dropping al * bl
__device__ __forceinline__ void dw_add_prod(float& hi, float& lo, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    const float pe = __fmaf_rn(ah, bh, -p);  // exact error of the product
    const float t = __fadd_rn(pe, __fadd_rn(__fmul_rn(ah, bl), __fmul_rn(al, bh)));
    dw_add2(hi, lo, p, t);
}

// Block-wide double-word sum of NV values per thread, fixed tree order; the
// result lands in (h, l) of thread 0.  The mixed form reduces its virial
// partials this way: an FP64 warp shuffle tree costs more issue slots on this
// part's narrow FP64 pipe than the rest of the pass.
template <int NV, int BLOCK>
__device__ __forceinline__ void block_sum_dw(float (&h)[NV], float (&l)[NV], float2* smem /* [NV][BLOCK/32] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float bh = __shfl_down_sync(0xffffffffu, h[c], o), bl = __shfl_down_sync(0xffffffffu, l[c], o);
            dw_add2(h[c], l[c], bh, bl);
        }
        if (lane == 0) smem[c * (BLOCK / 32) + warp] = make_float2(h[c], l[c]);
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const float2 q = lane < BLOCK / 32 ? smem[c * (BLOCK / 32) + lane] : make_float2(0.0f, 0.0f);
            h[c] = q.x;
            l[c] = q.y;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float bh = __shfl_down_sync(0xffffffffu, h[c], o), bl = __shfl_down_sync(0xffffffffu, l[c], o);
                dw_add2(h[c], l[c], bh, bl);
            }
        }
    }
}

// Programmatic dependent launch.  The four kernels of a step are launched
// with programmatic stream serialization, so each may be scheduled while its
// predecessor drains.  Each one first waits for its predecessor grid to
// complete and its writes to be visible (griddepcontrol.wait: a hardware
// wait, no spin), and only then touches memory and lets its own successor be
// scheduled.  Waits chain, so every earlier kernel has completed too.
// A history component in the row atom's own sense: the two copies of a
// contact are exact negatives (for a double word, both words negated).
__device__ __forceinline__ double hsign(double h, bool keep) { return keep ? h : -h; }
__device__ __forceinline__ DW hsign(DW h, bool keep) { return keep ? h : DW{-h.hi, -h.lo}; }

__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Scratch layout of one instance: [flag words, one per 32-atom group + 1]
// [per-group gaps][per-atom gaps][groups in ascending gap order][their gaps]
// [sort keys, a power of two of them][virial partials, component-major
// [6][blocks of A and C]], each region on a 256-byte boundary.
__host__ __device__ inline size_t lay_round256(size_t b) { return (b + 255) & ~size_t(255); }
__host__ __device__ inline int lay_groups(int n) { return (n + 31) / 32; }
__host__ __device__ inline int lay_npad(int n) {
    int p = 2;
    while (p < lay_groups(n)) p <<= 1;
    return p;
}
__host__ __device__ inline size_t lay_gap(int n) { return lay_round256((size_t)(lay_groups(n) + 1) * sizeof(uint32_t)); }
__host__ __device__ inline size_t lay_agap(int n) { return lay_gap(n) + lay_round256((size_t)lay_groups(n) * sizeof(float)); }
__host__ __device__ inline size_t lay_order(int n) { return lay_agap(n) + lay_round256((size_t)n * sizeof(float)); }
__host__ __device__ inline size_t lay_sgap(int n) { return lay_order(n) + lay_round256((size_t)lay_groups(n) * sizeof(int32_t)); }
__host__ __device__ inline size_t lay_keys(int n) { return lay_sgap(n) + lay_round256((size_t)lay_groups(n) * sizeof(float)); }
__host__ __device__ inline size_t lay_part(int n) { return lay_keys(n) + lay_round256((size_t)lay_npad(n) * sizeof(uint64_t)); }

__device__ __forceinline__ bool rebuild_due(const tmps_engine* __restrict__ e, int64_t s) {
    const int64_t since = s - e->last_build_step;
    if (since <= 0) return false;  // built in this very step already
    if (since < e->delay) return false;
    if (e->every > 0 && since % e->every != 0) return false;
    if (!e->check) return true;
    return e->disp_stamp == (int32_t)s;
}

// ------------------------------------------------------------------- A, FP64

// Running maximum of |x - x0|^2 since the reference of the contact bounds
// (non-negative FP32 values order as their bit patterns; NaN above all).
__device__ __forceinline__ void note_displacement(tmps_engine* __restrict__ e, float dd) {
    const uint32_t m = __reduce_max_sync(0xffffffffu, __float_as_uint(dd));
    if ((threadIdx.x & 31) == 0 && m > *(volatile uint32_t*)&e->maxd2_bits) atomicMax(&e->maxd2_bits, m);
}

// Bit of atom i in the flag words: its force and torque may be nonzero (the
// words of C's first pass; all ones before the first pass after a build).
__device__ __forceinline__ bool force_live(const uint32_t* __restrict__ flags, int i) {
    return flags == nullptr || ((flags[i >> 5] >> (i & 31)) & 1u);
}

// A negative zero becomes a positive zero, every other value (NaN included)
// is kept: the result of adding +0 to it, by integer operations.
__device__ __forceinline__ double plus_zero(double x) {
    const long long b = __double_as_longlong(x);
    return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}

// Block sum of the FP64 update's six kinetic components by halving
// exchanges: the FP64 pipe charges an instruction per warp however few lanes
// use it, so a shuffle tree per component (30 additions per warp) costs as
// much as several atoms' updates.  Padded to eight components, each exchange
// keeps half of what a lane holds (4 + 2 + 1 + 1 + 1 = 9 additions per
// warp), after which lane l holds component 4 b4 + 2 b3 + b2 (its lane bits
// 4, 3, 2) of the warp's total.  Lanes 0..5 of warp 0 then add the warp
// totals of their component in warp order and return the block's total; the
// other threads return 0.  Fixed order: deterministic for a block size.
__device__ __forceinline__ double block_sum6_halving(const double (&v)[6], double* smem /* [6][kBlockA / 32] */) {
    constexpr int kW = kBlockA / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double a[8] = {v[0], v[1], v[2], v[3], v[4], v[5], 0.0, 0.0};
    const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0, b2 = (lane & 4) != 0;
    double r4[4], r2[2];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double send = b4 ? a[k] : a[4 + k], keep = b4 ? a[4 + k] : a[k];
        r4[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const double send = b3 ? r4[k] : r4[2 + k], keep = b3 ? r4[2 + k] : r4[k];
        r2[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    double r = (b2 ? r2[1] : r2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? r2[0] : r2[1], 4);
    r += __shfl_xor_sync(0xffffffffu, r, 2);  // both lanes of a pair add the same two values
    r += __shfl_xor_sync(0xffffffffu, r, 1);
    const int c = (b4 ? 4 : 0) + (b3 ? 2 : 0) + (b2 ? 1 : 0);
    if ((lane & 3) == 0 && c < 6) smem[c * kW + warp] = r;
    __syncthreads();
    double t = 0.0;
    if (warp == 0 && lane < 6) {
        t = smem[lane * kW];
#pragma unroll
        for (int w = 1; w < kW; ++w) t += smem[lane * kW + w];
    }
    return t;
}

// A runs as one resident wave striding over the atoms; besides the update
// it sums the kinetic part of the virial, sum m v(t+dt/2) v(t+dt/2), over
// every atom into per-block partials: an atom C finds contact-free ends the
// step with that velocity, and C adds m (v(t+dt) v(t+dt) - v(t+dt/2)
// v(t+dt/2)) for the rest (thermo.py:94-101).
//
// An atom whose flag bit is clear holds a force and torque of exact zeros:
// with 1/m and 1/I positive and finite and dt > 0 (tmps_fused_prepare
// records any exception in kick_all) its half-kicks v += (dt/2) (f/m) add +0
// to each component, which changes a negative zero alone, so such an atom
// takes plus_zero instead of the FP64 kick arithmetic (half of this kernel's
// FP64 instructions) and its 1/m, 1/I are not read.  The results are the
// kick's, bit for bit.
__device__ __forceinline__ void a64_body(const tmps_atoms& a, const tmps_box* __restrict__ b,
                                         tmps_engine* __restrict__ e, const uint32_t* __restrict__ flags,
                                         double* __restrict__ part, const int bid, const int nblk) {
    __shared__ double smem[6 * (kBlockA / 32)];
    pdl_enter();
    if (e->aborted || e->step >= e->stop_step) return;
    const int n = a.n;
    const int nb = e->nblocks;  // partials are component-major, [6][nb]
    const int lane = threadIdx.x & 31;
    const int32_t s = (int32_t)(e->step + 1);
    const double dt = e->dt, dtf = 0.5 * dt;
    const bool fin = e->final_pending != 0, remap = b->remap_pending != 0;
    const bool kick_all = e->kick_all != 0 || !(dtf > 0.0);
    const float trig32 = approx_f32(e->trigger_sq);
    bool hit = false;
    float dd = 0.0f;
    double K[6] = {0, 0, 0, 0, 0, 0};
    const int stride = nblk * blockDim.x;
    for (int b0 = bid * blockDim.x + (threadIdx.x & ~31); b0 < n; b0 += stride) {
        const int i = b0 + lane;
        if (i >= n) continue;
        double4 x = ld4(a.xr, i), v = ld4(a.vm, i), w = ld4(a.om, i);
        // the skin check's reference with the state (not after the stores, which might alias it)
        const double x0x = __ldcs(a.x0 + i), x0y = __ldcs(a.x0 + n + i), x0z = __ldcs(a.x0 + 2 * n + i);
        const bool live = force_live(flags, i);
        if (live || kick_all) {
            const double im = __ldcs(a.rinv + i), iI = __ldcs(a.rinv + n + i);
            double f[3] = {0.0, 0.0, 0.0}, t[3] = {0.0, 0.0, 0.0};
            if (live) {
                f[0] = __ldcs(a.f + i); f[1] = __ldcs(a.f + n + i); f[2] = __ldcs(a.f + 2 * n + i);
                t[0] = __ldcs(a.torque + i); t[1] = __ldcs(a.torque + n + i); t[2] = __ldcs(a.torque + 2 * n + i);
            }
            if (fin) {  // second half-kick of the previous step
                v.x += dtf * (f[0] * im); v.y += dtf * (f[1] * im); v.z += dtf * (f[2] * im);
                w.x += dtf * (t[0] * iI); w.y += dtf * (t[1] * iI); w.z += dtf * (t[2] * iI);
            }
            v.x += dtf * (f[0] * im); v.y += dtf * (f[1] * im); v.z += dtf * (f[2] * im);
            w.x += dtf * (t[0] * iI); w.y += dtf * (t[1] * iI); w.z += dtf * (t[2] * iI);
        } else {
            v.x = plus_zero(v.x); v.y = plus_zero(v.y); v.z = plus_zero(v.z);
            w.x = plus_zero(w.x); w.y = plus_zero(w.y); w.z = plus_zero(w.z);
        }
        if (remap) {  // remap x of the previous step's servo update
            x.x = b->lo[0] + (x.x - b->old_lo[0]) * e->remap_scale[0];
            x.y = b->lo[1] + (x.y - b->old_lo[1]) * e->remap_scale[1];
            x.z = b->lo[2] + (x.z - b->old_lo[2]) * e->remap_scale[2];
        }
        x.x = x.x + dt * v.x; x.y = x.y + dt * v.y; x.z = x.z + dt * v.z;
        st4(a.xr, i, x);
        st4(a.vm, i, v);
        st4(a.om, i, w);
        const double d0 = __dsub_rn(x.x, x0x), d1 = __dsub_rn(x.y, x0y), d2 = __dsub_rn(x.z, x0z);
        // |d|^2 first in FP32 from the truncated differences (integer operations;
        // relative error under 1e-5): the exact FP64 test decides only within
        // that margin of the trigger, or for a non-finite displacement
        const float f0 = approx_f32(d0), f1 = approx_f32(d1), f2 = approx_f32(d2);
        const float q32 = (f0 * f0 + f1 * f1) + f2 * f2;
        bool far;
        if (q32 < trig32 * 0.99998f) {
            far = false;
        } else if (q32 > trig32 * 1.00002f && q32 <= 3e38f) {
            far = true;
        } else {
            const double q = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
            // a non-finite displacement forces the rebuild, whose binning reports the position
            far = !(q <= e->trigger_sq);
        }
        hit = hit || far;
        // the running maximum only has to bound |d|^2 from above (C's cull threshold)
        dd = q32 == q32 ? fmaxf(dd, q32 * 1.00002f + 1e-30f) : __int_as_float(0x7fffffff);
        const double kin[6] = {(v.w * v.x) * v.x, (v.w * v.y) * v.y, (v.w * v.z) * v.z,
                               (v.w * v.x) * v.y, (v.w * v.x) * v.z, (v.w * v.y) * v.z};
#pragma unroll
        for (int c = 0; c < 6; ++c) K[c] += kin[c];
    }
    if (__any_sync(0xffffffffu, hit) && lane == 0) e->disp_stamp = s;
    note_displacement(e, dd);
    const double tot = block_sum6_halving(K, smem);
    if (threadIdx.x < 6) part[(size_t)threadIdx.x * nb + bid] = tot;
}

__global__ void __launch_bounds__(kBlockA) k_a64(tmps_atoms a, const tmps_box* __restrict__ b,
                                                  tmps_engine* __restrict__ e, const uint32_t* __restrict__ flags,
                                                  double* __restrict__ part) {
    a64_body(a, b, e, flags, part, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ A, mixed

__device__ __forceinline__ int cell_x(int32_t c) { return c & 1023; }
__device__ __forceinline__ int cell_y(int32_t c) { return (c >> 10) & 1023; }
__device__ __forceinline__ int cell_z(int32_t c) { return (c >> 20) & 1023; }

// The mixed form's velocity and angular velocity words of atom i as four
// float4: v = (v hi, m), vl = (v lo, 1/m), w = (omega hi, -), wl = (omega lo,
// 1/I).  In memory the low words are packed so that no per-build constant is
// rewritten with them: om32 = (omega hi, v lo x), lo32 = (v lo y, v lo z,
// omega lo x, omega lo y), wlz32 = omega lo z, inv32 = (1/m, 1/I) (read only).
// CS: the low words with streaming (evict-first) hints; INV: also 1/m and 1/I
// (else vl.w and wl.w are left 0).
template <bool CS, bool INV = true>
__device__ __forceinline__ void load_vw(const tmps_atoms& a, int i, float4& v, float4& vl, float4& w, float4& wl) {
    v = ld4f(a.vel32, i);
    const float4 o = ld4f(a.om32, i);
    float4 q;
    float wz;
    float2 inv = make_float2(0.0f, 0.0f);
    if constexpr (CS) {
        q = __ldcs(reinterpret_cast<const float4*>(a.lo32) + i);
        wz = __ldcs(a.wlz32 + i);
        if constexpr (INV) inv = __ldcs(reinterpret_cast<const float2*>(a.inv32) + i);
    } else {
        q = ld4f(a.lo32, i);
        wz = a.wlz32[i];
        if constexpr (INV) inv = reinterpret_cast<const float2*>(a.inv32)[i];
    }
    w = make_float4(o.x, o.y, o.z, 0.0f);
    vl = make_float4(o.w, q.x, q.y, inv.x);
    wl = make_float4(q.z, q.w, wz, inv.y);
}

template <bool CS>
__device__ __forceinline__ void store_vw(const tmps_atoms& a, int i, float4 v, float4 vl, float4 w, float4 wl) {
    st4f(a.vel32, i, v);
    st4f(a.om32, i, make_float4(w.x, w.y, w.z, vl.x));
    const float4 q = make_float4(vl.y, vl.z, wl.x, wl.y);
    if constexpr (CS) {
        __stcs(reinterpret_cast<float4*>(a.lo32) + i, q);
        __stcs(a.wlz32 + i, wl.z);
    } else {
        reinterpret_cast<float4*>(a.lo32)[i] = q;
        a.wlz32[i] = wl.z;
    }
}

// Streaming (evict-first) loads and stores for the per-atom words only A
// touches each step: A moves ~150 MB through the 129 MB L2 every step, and
// marking that traffic evict-first keeps C's working set (flag words, gap
// bounds, row lengths and heads, high position words) resident.
__device__ __forceinline__ float4 ld4f_cs(const float* p, int i) { return __ldcs(reinterpret_cast<const float4*>(p) + i); }
__device__ __forceinline__ void st4f_cs(float* p, int i, float4 v) { __stcs(reinterpret_cast<float4*>(p) + i, v); }

__device__ __forceinline__ void a32_body(const tmps_atoms& a, const tmps_box* __restrict__ b,
                                         tmps_engine* __restrict__ e, const uint32_t* __restrict__ flags,
                                         double* __restrict__ part, const int bid, const int nblk) {
    // Double-word state (hi + lo, both FP32) updated with error-free FP32
    // transforms: the FP64 pipe of this part is ~70x narrower than FP32, and
    // a double<->float conversion costs as much as a DFMA, so this kernel
    // issues no FP64 instruction at all.
    __shared__ float2 smem[6 * (kBlockA / 32)];
    pdl_enter();
    if (e->aborted || e->step >= e->stop_step) return;
    const int n = a.n;
    const int nb = e->nblocks;  // partials are component-major, [6][nb]
    const int lane = threadIdx.x & 31;
    const int32_t s = (int32_t)(e->step + 1);
    const float dth = e->dt_hi, dtl = e->dt_lo;
    // merged half-kicks: the previous step's second and this step's first
    const float kick = e->final_pending ? dth : 0.5f * dth;
    const bool remap = b->remap_pending != 0;
    bool hit = false;
    float dd = 0.0f;
    float Kh[6] = {0, 0, 0, 0, 0, 0}, Kl[6] = {0, 0, 0, 0, 0, 0};
    const int stride = nblk * blockDim.x;
    for (int b0 = bid * blockDim.x + (threadIdx.x & ~31); b0 < n; b0 += stride) {
        const int i = b0 + lane;
        if (i >= n) continue;
        float4 p = ld4f(a.pos32, i), pl = ld4f_cs(a.pos32lo, i);
        float4 v, vl, w, wl;
        load_vw<true, false>(a, i, v, vl, w, wl);
        // the skin check's words with the state's, in the same round trip (the stores below could
        // alias them as far as the compiler knows, so it would not hoist these loads above them)
        const int32_t c = __ldcs(a.cell32 + i);
        const float o0x = __ldcs(a.o0_32 + i), o0y = __ldcs(a.o0_32 + n + i), o0z = __ldcs(a.o0_32 + 2 * n + i);
        if (force_live(flags, i)) {  // an unflagged atom's force is an exact zero: nothing to add
            const float2 inv = __ldcs(reinterpret_cast<const float2*>(a.inv32) + i);  // 1/m, 1/I
            const float km = kick * inv.x, kI = kick * inv.y;
            dw_add(v.x, vl.x, km * __ldcs(a.f32 + i));
            dw_add(v.y, vl.y, km * __ldcs(a.f32 + n + i));
            dw_add(v.z, vl.z, km * __ldcs(a.f32 + 2 * n + i));
            dw_add(w.x, wl.x, kI * __ldcs(a.torque32 + i));
            dw_add(w.y, wl.y, kI * __ldcs(a.torque32 + n + i));
            dw_add(w.z, wl.z, kI * __ldcs(a.torque32 + 2 * n + i));
        }
        if (remap) {
            // remap x scales a cell-relative offset with the box: o += o * eps
            dw_add(p.x, pl.x, p.x * e->eps_hi[0] + (p.x * e->eps_lo[0] + pl.x * e->eps_hi[0]));
            dw_add(p.y, pl.y, p.y * e->eps_hi[1] + (p.y * e->eps_lo[1] + pl.y * e->eps_hi[1]));
            dw_add(p.z, pl.z, p.z * e->eps_hi[2] + (p.z * e->eps_lo[2] + pl.z * e->eps_hi[2]));
        }
        // drift o += dt * v in double words
        dw_add_prod(p.x, pl.x, dth, dtl, v.x, vl.x);
        dw_add_prod(p.y, pl.y, dth, dtl, v.y, vl.y);
        dw_add_prod(p.z, pl.z, dth, dtl, v.z, vl.z);
        st4f(a.pos32, i, p);
        st4f_cs(a.pos32lo, i, pl);
        store_vw<true>(a, i, v, vl, w, wl);
        // displacement since the build: offset change + cell origin change
        const float d0 = ((p.x - o0x) + pl.x) + (float)cell_x(c) * e->dh32[0] + e->dlo32[0];
        const float d1 = ((p.y - o0y) + pl.y) + (float)cell_y(c) * e->dh32[1] + e->dlo32[1];
        const float d2 = ((p.z - o0z) + pl.z) + (float)cell_z(c) * e->dh32[2] + e->dlo32[2];
        const float q = (d0 * d0 + d1 * d1) + d2 * d2;
        hit = hit || !(q <= e->trigger32);  // NaN included (see a64_body)
        dd = q == q ? fmaxf(dd, q) : __int_as_float(0x7fffffff);
        // kinetic term from the high words (vel32.w = m)
        const float kin[6] = {(v.w * v.x) * v.x, (v.w * v.y) * v.y, (v.w * v.z) * v.z,
                              (v.w * v.x) * v.y, (v.w * v.x) * v.z, (v.w * v.y) * v.z};
#pragma unroll
        for (int k = 0; k < 6; ++k) dw_add(Kh[k], Kl[k], kin[k]);
    }
    if (__any_sync(0xffffffffu, hit) && lane == 0) e->disp_stamp = s;
    note_displacement(e, dd);
    block_sum_dw<6, kBlockA>(Kh, Kl, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k) reinterpret_cast<float2*>(part)[(size_t)k * nb + bid] = make_float2(Kh[k], Kl[k]);
    }
}

// Three resident blocks per SM (80 registers, no spill): measured 2-3 % faster
// in the step than four at 64 registers, which spilled.
__global__ void __launch_bounds__(kBlockA, 3) k_a32(tmps_atoms a, const tmps_box* __restrict__ b,
                                                     tmps_engine* __restrict__ e, const uint32_t* __restrict__ flags,
                                                     double* __restrict__ part) {
    a32_body(a, b, e, flags, part, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------- C

constexpr int kLive = 8;  // live groups a warp screens together (8 measured best: 4 and 12 are slower)

// Position of the k-th (from 0) set bit of m (k < popc(m)).
__device__ __forceinline__ int nth_bit(uint32_t m, int k) {
    int pos = 0;
#pragma unroll
    for (int sh = 16; sh > 0; sh >>= 1) {
        const int c = __popc(m & ((1u << sh) - 1u));
        if (k >= c) {
            k -= c;
            m >>= sh;
            pos += sh;
        }
    }
    return pos;
}

template <bool MIXED>
__device__ __forceinline__ void zero_force(const tmps_atoms& A, int i) {
    const int n = A.n;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if constexpr (MIXED) {
            A.f32[c * n + i] = 0.0f;
            A.torque32[c * n + i] = 0.0f;
        } else {
            A.f[c * n + i] = 0.0;
            A.torque[c * n + i] = 0.0;
        }
    }
}

// Contact bounds at the reference positions x0 (the positions of the last
// build): per atom and per 32-atom group, the smallest gap |d| - (ri + rj)
// over the rows, rounded down to FP32; -inf for an atom holding a live
// contact (and its group) or when a periodic dimension has a single bin (the
// image is then not fixed by the stencil).  Every atom's flag bit is set:
// its force may be nonzero.
__global__ void __launch_bounds__(kBlockA) k_bounds(tmps_atoms A, tmps_nlist L, const tmps_box* __restrict__ B,
                                                     tmps_engine* __restrict__ E, int hist, int cull, uint32_t* flags,
                                                     float* gap, float* agap) {
    const int n = A.n;
    const int lane = threadIdx.x & 31;
    const int ngroups = (n + 31) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    int per[3];
    double prd[3], iprd[3];
    bool single = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        per[c] = B->per[c];
        prd[c] = B->prd[c];
        iprd[c] = B->inv_prd[c];
        single = single || (per[c] == 1 && B->g[c] == 1);
    }
    // The bound only has to be a lower bound.  The separation is the FP64
    // difference of the positions, taken to FP32 by truncation (approx_f32:
    // integer operations, no FP64 conversion), its periodic image and the
    // distance and gap then in FP32, and the gap is lowered by 3e-6 of the
    // magnitudes involved -- the separation before the image, the image shift,
    // r and the radii: over twice the error (2^-20 of each truncated value plus
    // FP32 rounding, ~1.2e-6 of them), while a pair away from the boundary
    // keeps a margin of ~1e-5 (a listed pair is never near half a box, so the
    // image is the FP64 one).  A bound a little low only culls a little less.
    float prd32[3], iprd32[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        prd32[c] = approx_f32(prd[c]);
        iprd32[c] = approx_f32(iprd[c]);
    }
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += nwarps) {
        const int i = (g << 5) + lane;
        float gmin = 3e38f;
        if (i < n) {
            const double xi[3] = {A.x0[i], A.x0[n + i], A.x0[2 * n + i]};
            const float ri = approx_f32(A.xr[4 * (size_t)i + 3]);
            const int nn = L.nnb[i];
            for (int k = 0; k < nn; ++k) {
                const int j = L.nbr[(size_t)k * n + i] & kNbrIndexMask;
                const double dd[3] = {xi[0] - A.x0[j], xi[1] - A.x0[n + j], xi[2] - A.x0[2 * n + j]};
                float d[3], mag = 0.0f;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    d[c] = approx_f32(dd[c]);
                    mag += fabsf(d[c]);
                    if (per[c] == 1) {
                        const float nimg = rintf(d[c] * iprd32[c]);
                        d[c] -= nimg * prd32[c];
                        mag += fabsf(nimg) * prd32[c];
                    }
                }
                const float r = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
                const float rs = ri + approx_f32(A.xr[4 * (size_t)j + 3]);
                const float gp = (r - rs) - 3e-6f * ((mag + r) + rs);
                gmin = gp == gp ? fminf(gmin, gp) : -3e38f;  // a NaN pair pins the group
            }
            if ((hist && L.touch[i] != 0ull) || single) gmin = -3e38f;
            agap[i] = gmin;
        }
        {
            const int t = __popc(__ballot_sync(0xffffffffu, i < n && !(gmin > 0.0f)));
            if (lane == 0 && t) atomicAdd(&E->touching, t);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gmin = fminf(gmin, __shfl_down_sync(0xffffffffu, gmin, o));
        if (lane == 0) {
            gap[g] = gmin;
            // bits of existing atoms only: a set bit makes C clear that atom's force
            const int rem = n - (g << 5);
            flags[g] = rem >= 32 ? 0xffffffffu : (1u << rem) - 1u;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float hmin = (float)B->hcell[0];
        hmin = fminf(hmin, (float)B->hcell[1]);
        hmin = fminf(hmin, (float)B->hcell[2]);
        E->cull_tol = 1e-5f * hmin;
        E->maxd2_bits = 0u;
        E->shift_bound = 0.0f;
        for (int c = 0; c < 3; ++c) E->prd_ref[c] = B->prd[c];
        E->cull = (cull && !single) ? 1 : 0;
        E->order_ready = 0;  // the first pass after the bounds visits every group
    }
}

// Groups in ascending order of their gap bound, for C's ordered pass.  Key:
// the gap's bits made to order as unsigned (a NaN first), then the group.
// Deterministic: a bitonic sort of distinct keys.
__global__ void __launch_bounds__(256) k_gap_keys(const float* __restrict__ gap, int ng, int npad,
                                                  uint64_t* __restrict__ keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    if (i >= ng) {
        keys[i] = ~0ull;
        return;
    }
    const uint32_t u = __float_as_uint(gap[i]);
    uint32_t k;
    if ((u & 0x7fffffffu) > 0x7f800000u) k = 0u;  // NaN: culls nothing, so first
    else k = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    keys[i] = ((uint64_t)k << 32) | (uint32_t)i;
}

__global__ void __launch_bounds__(256) k_bitonic_global(uint64_t* __restrict__ keys, int npad, int j, int k) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    const int l = i ^ j;
    if (l <= i) return;
    const uint64_t a = keys[i], b = keys[l];
    if ((a > b) == ((i & k) == 0)) {
        keys[i] = b;
        keys[l] = a;
    }
}

// Stages k_lo..k_hi of the bitonic sort inside chunks of `chunk` keys (the
// first stage from j = j_first), one block of chunk / 2 threads per chunk.
// (Measured: 2048-key chunks, one pair per thread and stage, beat 16384-key
// chunks in 128 KB of shared memory -- fewer launches, but each block then
// runs 91 barrier-separated stages at four pairs per thread.)
constexpr int kSortChunk = 2048;
__global__ void __launch_bounds__(kSortChunk / 2) k_bitonic_shared(uint64_t* __restrict__ keys, int chunk, int k_lo,
                                                                 int k_hi, int j_first) {
    __shared__ uint64_t sk[kSortChunk];
    const int c0 = blockIdx.x * chunk;
    for (int t = threadIdx.x; t < chunk; t += blockDim.x) sk[t] = keys[c0 + t];
    __syncthreads();
    for (int k = k_lo; k <= k_hi; k <<= 1) {
        for (int j = (k == k_lo ? j_first : k >> 1); j > 0; j >>= 1) {
            const int t = threadIdx.x;
            const int i = 2 * t - (t & (j - 1));  // lower element of the pair
            const int l = i + j;
            const uint64_t a = sk[i], b = sk[l];
            if ((a > b) == (((c0 + i) & k) == 0)) {
                sk[i] = b;
                sk[l] = a;
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < chunk; t += blockDim.x) keys[c0 + t] = sk[t];
}

__global__ void __launch_bounds__(256) k_gap_order(const uint64_t* __restrict__ keys, const float* __restrict__ gap,
                                                   int ng, int32_t* __restrict__ order, float* __restrict__ sgap) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ng) return;
    const int g = (int)(uint32_t)keys[p];
    order[p] = g;
    sgap[p] = gap[g];
}

// C: the contact forces of one step.  Per warp, 32 groups strided over the
// system (warp w owns positions w, w + nwarps, ...; warps numbered across
// blocks first).  The first pass after the bounds takes the groups in index
// order (neighbouring groups -- atoms are in Morton order -- go to different
// SMs); every later pass takes them in ascending order of their gap bound, in
// which the live groups are a prefix, so each warp gets the same number of
// live groups and stops at its first ruled-out position:
//  1. bound check, one group per lane: a group whose smallest gap at the
//     reference positions (tmps_fused_bounds) exceeds 2 max|x - x0| + the
//     change of the periodic image shifts + a rounding slack cannot touch
//     (triangle inequality; both running maxima only grow, so it has had no
//     contact since the reference and its history is clear): its atoms are
//     finished with no row read;
//  2. rosters: the atoms of up to kLive live groups whose own gap bound does
//     not rule contact out, in group then atom order, 32 at a time.  A
//     roster's state words go to shared memory (CfWarp), then
//  3. near test: its (atom, slot) entries laid across the lanes, two passes
//     of 32 at once -- is the partner within reach of contact? (the contact
//     test itself in FP64; a conservative FP32 version in the mixed form).
//     Near entries join a ring of queued contacts in shared memory;
//  4. contact law: 32 queued contacts at a time, one per lane, so the law
//     runs with full lanes however the contacts fall over the rows; each
//     contact's force, torque and virial go to shared memory and the first
//     lane of each atom's run of contacts adds them to the atom's sums in
//     slot order -- the order of a one-thread-per-atom loop, whatever the
//     batching (so culling changes no bit of a force);
//  5. finish, one lane per roster atom: an atom with a near entry is flagged
//     (its bit in the group's new flag word), gets Cundall damping, its force
//     and torque written and its virial and kinetic terms summed; every
//     roster atom's touch mask is rewritten if it changed (cleared when it
//     has no near entry).
// The flag words double as "force may be nonzero": an atom's force and
// torque are written as zeros only when it was flagged the step before, so
// every unflagged atom holds an exact zero, which A relies on to skip
// loading them.  None of the skipping changes a result.  The per-block
// virial partials depend only on the flag words, the group order and the
// grid, not on scheduling; the kinetic term of an unflagged atom is A's.
constexpr int kRing = 128;  // queued contacts per warp: < 32 waiting + 64 from one near-test step

template <bool MIXED>
struct CfWarp;

// mixed form: FP32 state words; a queued entry keeps the partner's high
// position word the near test loaded
template <>
struct CfWarp<true> {
    float4 p[32], pl[32], v[32], w[32];  // pos32, pos32lo, vel32, om32 of the roster atoms
    float4 red[3][32];                   // one contact per lane: f.xyz t.x | t.yz V0 V1 | V2..V5
    float4 acc[3][32];                   // per roster atom, the same packing
    float4 qp[kRing];                    // queued: partner pos32
    uint64_t touch[32], ntouch[32];      // touch mask at entry / of this step's contacts
    int32_t start[33], idx[32], cell[32], qe[kRing];
    uint32_t near[32], qak[kRing];       // queued: roster atom | slot << 5
};

template <>
struct CfWarp<false> {
    double4 p[32], v[32], w[32];  // xr, vm, om of the roster atoms
    double2 red[6][32];           // f.xy | f.z t.x | t.yz | V0 V1 | V2 V3 | V4 V5
    double2 acc[6][32];
    uint64_t touch[32], ntouch[32];
    int32_t start[33], idx[32], qe[kRing];
    uint32_t near[32], qak[kRing];
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// The partner-side words of one contact (partner j of row atom i at slot k):
// its state words and the contact's history as it enters the step.
template <bool MIXED>
struct CfLoad {
    using S4 = typename std::conditional<MIXED, float4, double4>::type;
    using HT = typename std::conditional<MIXED, DW, double>::type;
    S4 pj, v2, w2;
    float4 jl;
    int32_t cj;
    bool was;
    HT shr[3], rlr[3];
};

template <int STYLE, bool MIXED, bool DENSE>
__device__ __forceinline__ void cf_body(const tmps_atoms& A, const tmps_nlist& L, const tmps_pair_params& P,
                                        const tmps_box* __restrict__ B, tmps_engine* __restrict__ E,
                                        uint32_t* __restrict__ flags, const float* __restrict__ gap,
                                        const float* __restrict__ agap, const int32_t* __restrict__ order,
                                        const float* __restrict__ sgap, double* __restrict__ part, const int bid,
                                        const int nblk) {
    using T = typename std::conditional<MIXED, float, double>::type;
    // histories: doubles in the FP64 form, FP32 double words in the mixed form
    using HT = typename std::conditional<MIXED, DW, double>::type;
    using S4 = typename std::conditional<MIXED, float4, double4>::type;  // a state word
    __shared__ double smem[6 * (kBlockC / 32)];
    __shared__ uint32_t cwords[kBlockC / 32][kLive];
    // the kLive groups of the batch in hand: group, old and near words (warp-uniform)
    __shared__ int32_t bgrp[kBlockC / 32][kLive];
    __shared__ uint32_t bold[kBlockC / 32][kLive], bnear[kBlockC / 32][kLive];
    __shared__ CfWarp<MIXED> cwarp[DENSE ? 1 : kBlockC / 32];
    pdl_enter();
    if (E->aborted || E->step >= E->stop_step) return;
    const int64_t s = E->step + 1;
    if (rebuild_due(E, s)) return;  // S marks the step aborted; the host rebuilds
    const int nb = E->nblocks;      // partials are component-major, [6][nb]
    part += nb - nblk;              // C's blocks follow A's
    constexpr bool kHist = STYLE == STYLE_HOOKE_HISTORY || STYLE == STYLE_HERTZ_HISTORY || STYLE == STYLE_GRANULAR;
    const bool hist = kHist && (STYLE != STYLE_GRANULAR || P.tangential_id >= 2 || P.rolling_id != 0);
    const bool roll = STYLE == STYLE_GRANULAR && P.rolling_id != 0;
    const int n = A.n;
    T dt;
    if constexpr (MIXED) dt = E->dt_hi;
    else dt = E->dt;
    // per-step constants
    T hh[3] = {0, 0, 0}, prd[3], iprd[3];
    float hlo[3] = {0, 0, 0}, prdlo[3] = {0, 0, 0};
    int per[3], single[3], gdim[3];
    T hrate[3] = {0, 0, 0}, hshear[3] = {0, 0, 0};
    const bool vremap = B->vremap != 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        per[c] = B->per[c];
        gdim[c] = B->g[c];
        if constexpr (MIXED) {
            hh[c] = E->h32[c];
            hlo[c] = E->hlo32[c];
            prd[c] = E->prd32[c];
            prdlo[c] = E->prdlo32[c];
            iprd[c] = E->iprd32[c];
            single[c] = E->single_bin[c];
        } else {
            prd[c] = B->prd[c];
            iprd[c] = B->inv_prd[c];
            single[c] = 0;
        }
    }
    if (vremap) {
        // n . h_rate for the image count n = (n0, n1, n2) of the partner
        hrate[0] = (T)B->h_rate[0]; hrate[1] = (T)B->h_rate[1]; hrate[2] = (T)B->h_rate[2];
        hshear[0] = (T)B->h_rate[3]; hshear[1] = (T)B->h_rate[4]; hshear[2] = (T)B->h_rate[5];
    }
    // mixed form: the 27 stencil offsets (ox, oy, oz) in {-1, 0, 1} times the
    // cell edge, both words (exact products), by the code a list entry carries
    __shared__ float4 soff[MIXED ? 27 : 1], sofl[MIXED ? 27 : 1];
    __shared__ PairParams32 sP;  // the mixed law's coefficients, converted once per block
    if constexpr (MIXED) {
        if (threadIdx.x == 32) params32(P, sP);
        if (threadIdx.x < 27) {
            const int code = threadIdx.x;
            const float ox = (float)(code % 3 - 1), oy = (float)((code / 3) % 3 - 1), oz = (float)(code / 9 - 1);
            soff[code] = make_float4(ox * hh[0], oy * hh[1], oz * hh[2], 0.0f);
            sofl[code] = make_float4(ox * hlo[0], oy * hlo[1], oz * hlo[2], 0.0f);
        }
        __syncthreads();
    }
    double Vd[6] = {0, 0, 0, 0, 0, 0};
    float Vh[6] = {0, 0, 0, 0, 0, 0}, Vl[6] = {0, 0, 0, 0, 0, 0};  // mixed: per-thread double words
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    CfWarp<MIXED>& W = cwarp[DENSE ? 0 : wib];
    const int ngroups = (n + 31) >> 5;
    const int nwarps = (nblk * blockDim.x) >> 5;
    const size_t ss = (size_t)L.slots * n;
    // consecutive groups (neighbours in space) go to consecutive blocks
    const int gw = bid + nblk * wib;
    const bool cull = E->cull != 0;
    float thr = 0.0f;
    if (cull) {
        // a NaN displacement makes thr NaN and culls nothing
        const float md = sqrtf(__uint_as_float(E->maxd2_bits));
        thr = ((2.0f * md) * 1.0001f + E->shift_bound) + E->cull_tol;
    }

    // The contact of row atom ia (its state words Pi, PLi (mixed: low words and
    // radius lo), Vi, Wi and packed cell Ci) with the partner of row entry e at
    // slot k (its high position word Pj), `was` its touch bit: whether they
    // touch, and if so the row atom's force, torque and pair virial terms in
    // fc, tc, vc; the contact's history is updated in place.  Every other load
    // of the contact is issued here together (one round trip).
    // The loads of a contact (row atom ia, row entry e at slot k, touch bit
    // `was`, partner high position word Pj), all issued at once: one round trip.
    auto contact_fetch = [&](const int ia, const int e, const int k, const bool was, const S4 Pj) {
        CfLoad<MIXED> cl;
        const int j = e & kNbrIndexMask;
        const size_t so = (size_t)k * n + ia;
        cl.pj = Pj;
        cl.was = was;
        cl.cj = 0;
        if constexpr (MIXED) {
            cl.jl = ld4f(A.pos32lo, j);
            cl.v2 = ld4f(A.vel32, j);
            cl.w2 = ld4f(A.om32, j);
            if (vremap) cl.cj = A.cell32[j];
        } else {
            cl.jl = make_float4(0.f, 0.f, 0.f, 0.f);
            cl.v2 = ld4(A.vm, j);
            cl.w2 = ld4(A.om, j);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cl.shr[c] = HT{};
            cl.rlr[c] = HT{};
        }
        if (hist && was) {
            const HT* hs = reinterpret_cast<const HT*>(L.shear);
            cl.shr[0] = hs[so];
            cl.shr[1] = hs[ss + so];
            cl.shr[2] = hs[2 * ss + so];
            if (roll) {
                const HT* hr = reinterpret_cast<const HT*>(L.rolling);
                cl.rlr[0] = hr[so];
                cl.rlr[1] = hr[ss + so];
                cl.rlr[2] = hr[2 * ss + so];
            }
        }
        return cl;
    };

    // The contact of row atom ia (its state words Pi, PLi (mixed: low words and
    // radius lo), Vi, Wi and packed cell Ci) with the partner of row entry e at
    // slot k, from its loads `cl`: whether they touch, and if so the row atom's
    // force, torque and pair virial terms in fc, tc, vc; the contact's history
    // is updated in place.
    auto contact_eval = [&](const int ia, const int e, const int k, const S4 Pi, const float4 PLi, const S4 Vi,
                            const S4 Wi, const int32_t Ci, const CfLoad<MIXED>& cl, T (&fc)[3], T (&tc)[3],
                            T (&vc)[6]) -> bool {
        (void)PLi;
        (void)Ci;
        const int j = e & kNbrIndexMask;
        const bool lo = ia < j;
        const size_t so = (size_t)k * n + ia;
        const bool was = cl.was;
        T xi[3], xj[3], ri, rj;
        int32_t ci = 0, cj = 0;
        float4 il = make_float4(0.f, 0.f, 0.f, 0.f), jl = il;
        T vi[3], wi[3], mi, vj[3], wj[3], mj;
        HT shr[3], rlr[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            shr[c] = cl.shr[c];
            rlr[c] = cl.rlr[c];
        }
        if constexpr (MIXED) {
            const float4 pi = Pi, pj = cl.pj;
            il = PLi;
            jl = cl.jl;
            const float4 v = Vi, w = Wi;
            const float4 v2 = cl.v2, w2 = cl.w2;
            if (vremap) {
                ci = Ci;
                cj = cl.cj;
            }
            xi[0] = pi.x; xi[1] = pi.y; xi[2] = pi.z; ri = pi.w;
            xj[0] = pj.x; xj[1] = pj.y; xj[2] = pj.z; rj = pj.w;
            vi[0] = v.x; vi[1] = v.y; vi[2] = v.z; mi = v.w;
            wi[0] = w.x; wi[1] = w.y; wi[2] = w.z;
            vj[0] = v2.x; vj[1] = v2.y; vj[2] = v2.z; mj = v2.w;
            wj[0] = w2.x; wj[1] = w2.y; wj[2] = w2.z;
        } else {
            const double4 pi = Pi, pj = cl.pj;
            const double4 v = Vi, w = Wi;
            const double4 v2 = cl.v2, w2 = cl.w2;
            xi[0] = pi.x; xi[1] = pi.y; xi[2] = pi.z; ri = pi.w;
            xj[0] = pj.x; xj[1] = pj.y; xj[2] = pj.z; rj = pj.w;
            vi[0] = v.x; vi[1] = v.y; vi[2] = v.z; mi = v.w;
            wi[0] = w.x; wi[1] = w.y; wi[2] = w.z;
            vj[0] = v2.x; vj[1] = v2.y; vj[2] = v2.z; mj = v2.w;
            wj[0] = w2.x; wj[1] = w2.y; wj[2] = w2.z;
        }
        // separation x_i - x_j
        T d[3];
        T nimg[3] = {0, 0, 0};
        const int code = (unsigned)e >> kNbrIndexBits;
        float offh[3] = {0.f, 0.f, 0.f}, offl[3] = {0.f, 0.f, 0.f};
        if constexpr (MIXED) {
            const float4 so = soff[code], sl = sofl[code];
            offh[0] = so.x; offh[1] = so.y; offh[2] = so.z;
            offl[0] = sl.x; offl[1] = sl.y; offl[2] = sl.z;
            // offsets are relative to each atom's own cell: j's cell is
            // the stencil offset (ox, oy, oz) away from i's, so
            // x_i - x_j = (o_i - o_j) - offset * h
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                d[c] = (xi[c] - xj[c]) - offh[c];
                if (single[c]) {
                    nimg[c] = rintf(d[c] * iprd[c]);
                    d[c] -= nimg[c] * prd[c];
                }
            }
            if (vremap) {  // image count for the partner velocity shift
                const int off[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
                const int cc[3] = {cell_x(ci) + off[0] - cell_x(cj), cell_y(ci) + off[1] - cell_y(cj),
                                   cell_z(ci) + off[2] - cell_z(cj)};
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    if (!single[c] && per[c] == 1) nimg[c] = (T)(cc[c] / gdim[c]);
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                d[c] = xi[c] - xj[c];
                if (per[c] == 1) {
                    nimg[c] = rint(d[c] * iprd[c]);
                    d[c] = image_sub64(d[c], nimg[c], prd[c]);
                }
            }
        }
        PairIn<T> in;
        const T sg = lo ? T(1) : T(-1);
        in.ra = lo ? ri : rj;
        in.rb = lo ? rj : ri;
        bool near;
        if constexpr (MIXED) {
            // separation, |d|^2, |d| and the overlap from the high and
            // low FP32 words, so the overlap keeps ~2^-48 of |d| (an
            // FP32 difference of two unit-size numbers keeps 2^-24)
            const float xil[3] = {il.x, il.y, il.z}, xjl[3] = {jl.x, jl.y, jl.z};
            float dh[3], dl[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float s1, e1, s2, e2;
                two_sum(xi[c], -xj[c], s1, e1);
                two_sum(s1, -offh[c], s2, e2);
                const float low = __fadd_rn(__fsub_rn(__fsub_rn(xil[c], xjl[c]), offl[c]), __fadd_rn(e1, e2));
                two_sum(s2, low, dh[c], dl[c]);
                if (single[c]) {
                    const float ni = rintf(dh[c] * iprd[c]);
                    float s3, e3;
                    two_sum(dh[c], -ni * prd[c], s3, e3);
                    two_sum(s3, __fadd_rn(__fsub_rn(dl[c], ni * prdlo[c]), e3), dh[c], dl[c]);
                }
                dh[c] = sg * dh[c];
                dl[c] = sg * dl[c];
            }
            // |d|^2 = sum hi^2 (exact via FMA) + 2 hi lo
            float pp[3], pe[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pp[c] = __fmul_rn(dh[c], dh[c]);
                pe[c] = __fmaf_rn(dh[c], dh[c], -pp[c]);
            }
            float t1, te1, rh, re;
            two_sum(pp[0], pp[1], t1, te1);
            two_sum(t1, pp[2], rh, re);
            const float cross = __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dh[0], dl[0]),
                                                                    __fmul_rn(dh[1], dl[1])),
                                                         __fmul_rn(dh[2], dl[2])));
            const float rl0 = __fadd_rn(__fadd_rn(__fadd_rn(te1, re), __fadd_rn(__fadd_rn(pe[0], pe[1]), pe[2])),
                                        cross);
            float rsh, rsl;
            two_sum(rh, rl0, rsh, rsl);
            // r_hi need not be the rounded root: the residual rsh - r_hi^2 (one FMA,
            // within an ulp of exact for an r_hi a few ulp off) corrects it in r_lo
            const float r_hi = lsqrt(rsh);
            const float res = __fmaf_rn(-r_hi, r_hi, rsh);
            const float r_lo = __fdividef(__fadd_rn(res, rsl), __fmul_rn(2.0f, r_hi));
            // ra + rb, both words
            const float4 al = lo ? il : jl, bl = lo ? jl : il;
            float sh_, se_;
            two_sum(in.ra, in.rb, sh_, se_);
            const float rad_lo = __fadd_rn(__fadd_rn(al.w, bl.w), se_);
            const float delta = __fadd_rn(__fsub_rn(sh_, r_hi), __fsub_rn(rad_lo, r_lo));
            near = delta > 0.0f && rsh > 1e-28f;
#pragma unroll
            for (int c = 0; c < 3; ++c) in.d[c] = dh[c];
            in.rsq = rsh;
            in.r = r_hi;
            in.delta = delta;
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) in.d[c] = sg * d[c];
            in.rsq = rsq64(in.d);
            const T radsum = in.ra + in.rb;
            near = in.rsq < __dmul_rn(radsum, radsum) && in.rsq > T(1e-28);
            if (near) {
                in.r = sqrt(in.rsq);
                in.delta = radsum - in.r;
            }
        }
        if (near) {
            T dv[3] = {0, 0, 0};
            if (vremap) {
                // image count of x_a - x_b, then n . h_rate for partner b
                T na[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) na[c] = sg * nimg[c];
                dv[0] = (na[0] * hrate[0] + na[1] * hshear[2]) + na[2] * hshear[1];
                dv[1] = na[1] * hrate[1] + na[2] * hshear[0];
                dv[2] = na[2] * hrate[2];
            }
            in.ma = lo ? mi : mj;
            in.mb = lo ? mj : mi;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                in.va[c] = lo ? vi[c] : vj[c];
                in.vb[c] = (lo ? vj[c] : vi[c]) + dv[c];
                in.wa[c] = lo ? wi[c] : wj[c];
                in.wb[c] = lo ? wj[c] : wi[c];
            }
            HT sh[3] = {}, rl[3] = {};
            if (hist && was) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    sh[c] = hsign(shr[c], lo);
                    rl[c] = hsign(rlr[c], lo);
                }
            }
            PairOut<T> out;
            if constexpr (MIXED) contact_law<T, STYLE>(sP, dt, 1, in, sh, rl, out);
            else contact_law<T, STYLE>(P, dt, 1, in, sh, rl, out);
            if (hist) {
                HT* hs = reinterpret_cast<HT*>(L.shear);
                hs[so] = hsign(sh[0], lo);
                hs[ss + so] = hsign(sh[1], lo);
                hs[2 * ss + so] = hsign(sh[2], lo);
                if (roll) {
                    HT* hr = reinterpret_cast<HT*>(L.rolling);
                    hr[so] = hsign(rl[0], lo);
                    hr[ss + so] = hsign(rl[1], lo);
                    hr[2 * ss + so] = hsign(rl[2], lo);
                }
            }
            const T arm = lo ? out.arm_a : out.arm_b;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                fc[c] = sg * out.f[c];
                // rounded as written: both products may be fused into the sum, and which one is
                // must not depend on the path the contact is inlined into
                tc[c] = add_rn(mul_rn(arm, out.tor[c]), sg * out.troll[c]);
            }
            vc[0] = T(0.5) * (in.d[0] * out.f[0]);
            vc[1] = T(0.5) * (in.d[1] * out.f[1]);
            vc[2] = T(0.5) * (in.d[2] * out.f[2]);
            vc[3] = T(0.5) * (in.d[0] * out.f[1]);
            vc[4] = T(0.5) * (in.d[0] * out.f[2]);
            vc[5] = T(0.5) * (in.d[1] * out.f[2]);
        }
        return near;
    };

    // 4. the contact law for `cnt` (<= 32) queued contacts from ring position
    // qhead, one per lane, and their in-order reduction onto the roster atoms
    auto law = [&](int cnt, int qhead) {
        __syncwarp();
        const bool live = lane < cnt;
        const int slot = (qhead + lane) & (kRing - 1);
        int a = 32 + lane, k = 0, e = 0;  // a >= 32: no roster atom (a run of its own)
        if (live) {
            const uint32_t ak = W.qak[slot];
            a = (int)(ak & 31u);
            k = (int)(ak >> 5);
            e = W.qe[slot];
        }
        bool contact = false;
        T fc[3] = {0, 0, 0}, tc[3] = {0, 0, 0}, vc[6] = {0, 0, 0, 0, 0, 0};
        if (live) {
            const int ia = W.idx[a];
            const bool was = ((W.touch[a] >> k) & 1ull) != 0;
            if constexpr (MIXED) {
                const CfLoad<MIXED> cl = contact_fetch(ia, e, k, was, W.qp[slot]);
                contact = contact_eval(ia, e, k, W.p[a], W.pl[a], W.v[a], W.w[a], vremap ? W.cell[a] : 0, cl, fc,
                                       tc, vc);
            } else {
                const CfLoad<MIXED> cl = contact_fetch(ia, e, k, was, ld4(A.xr, e & kNbrIndexMask));
                contact = contact_eval(ia, e, k, W.p[a], make_float4(0.f, 0.f, 0.f, 0.f), W.v[a], W.w[a], 0, cl,
                                       fc, tc, vc);
            }
        }
        if (contact) atomicOr(reinterpret_cast<unsigned long long*>(&W.ntouch[a]), 1ull << k);
        if constexpr (MIXED) {
            W.red[0][lane] = make_float4(fc[0], fc[1], fc[2], tc[0]);
            W.red[1][lane] = make_float4(tc[1], tc[2], vc[0], vc[1]);
            W.red[2][lane] = make_float4(vc[2], vc[3], vc[4], vc[5]);
        } else {
            W.red[0][lane] = make_double2(fc[0], fc[1]);
            W.red[1][lane] = make_double2(fc[2], tc[0]);
            W.red[2][lane] = make_double2(tc[1], tc[2]);
            W.red[3][lane] = make_double2(vc[0], vc[1]);
            W.red[4][lane] = make_double2(vc[2], vc[3]);
            W.red[5][lane] = make_double2(vc[4], vc[5]);
        }
        // each roster atom's contacts form one run of lanes; its first lane
        // adds them to the atom's sums in slot order
        const int ap = __shfl_up_sync(0xffffffffu, a, 1), an = __shfl_down_sync(0xffffffffu, a, 1);
        const uint32_t ends = __ballot_sync(0xffffffffu, lane == 31 || an != a);
        __syncwarp();
        if (live && (lane == 0 || ap != a)) {
            const int last = __ffs(ends & ~lanemask_lt()) - 1;
            if constexpr (MIXED) {
                float4 s0 = W.acc[0][a], s1 = W.acc[1][a], s2 = W.acc[2][a];
                for (int t = lane; t <= last; ++t) {
                    const float4 r0 = W.red[0][t], r1 = W.red[1][t], r2 = W.red[2][t];
                    s0.x += r0.x; s0.y += r0.y; s0.z += r0.z; s0.w += r0.w;
                    s1.x += r1.x; s1.y += r1.y; s1.z += r1.z; s1.w += r1.w;
                    s2.x += r2.x; s2.y += r2.y; s2.z += r2.z; s2.w += r2.w;
                }
                W.acc[0][a] = s0; W.acc[1][a] = s1; W.acc[2][a] = s2;
            } else {
                double2 sacc[6];
#pragma unroll
                for (int c = 0; c < 6; ++c) sacc[c] = W.acc[c][a];
                for (int t = lane; t <= last; ++t) {
#pragma unroll
                    for (int c = 0; c < 6; ++c) {
                        const double2 r = W.red[c][t];
                        sacc[c].x += r.x;
                        sacc[c].y += r.y;
                    }
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) W.acc[c][a] = sacc[c];
            }
        }
        __syncwarp();
    };

    // 2-5: one roster of `count` atoms; this lane's atom is i (group word uq, bit)
    auto roster = [&](int count, int i, int uq, int bit) {
        __syncwarp();
        const bool mine = lane < count;
        const int nn = mine ? L.nnb[i] : 0;
        const uint64_t touch = (hist && mine) ? L.touch[i] : 0ull;
        if (mine) {
            if constexpr (MIXED) {
                W.p[lane] = ld4f(A.pos32, i);
                W.pl[lane] = ld4f(A.pos32lo, i);
                W.v[lane] = ld4f(A.vel32, i);
                W.w[lane] = ld4f(A.om32, i);
                if (vremap) W.cell[lane] = A.cell32[i];
            } else {
                W.p[lane] = ld4(A.xr, i);
                W.v[lane] = ld4(A.vm, i);
                W.w[lane] = ld4(A.om, i);
            }
        }
        W.idx[lane] = i;
        W.touch[lane] = touch;
        W.ntouch[lane] = 0ull;
        W.near[lane] = 0u;
        if constexpr (MIXED) {
#pragma unroll
            for (int c = 0; c < 3; ++c) W.acc[c][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
#pragma unroll
            for (int c = 0; c < 6; ++c) W.acc[c][lane] = make_double2(0.0, 0.0);
        }
        int incl = nn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        W.start[lane] = incl - nn;  // atoms past `count` start at `total`: the search never picks them
        if (lane == 0) W.start[32] = total;
        __syncwarp();
        int qhead = 0, qtail = 0, p0 = 0;  // ring positions and next entry (warp-uniform)
        while (true) {
            const int pending = qtail - qhead;
            if (pending >= 32 || (p0 >= total && pending > 0)) {
                const int cnt = pending < 32 ? pending : 32;
                law(cnt, qhead);
                qhead += cnt;
                continue;
            }
            if (p0 >= total) break;
            // 3. near test of entries p0 .. p0 + 63, two per lane, all loads in flight together
            int ea[2], aa[2], ka[2];
            bool va[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int idx = p0 + 32 * u + lane;
                va[u] = idx < total;
                int a = 0;
                if (va[u]) {
#pragma unroll
                    for (int st = 16; st > 0; st >>= 1)
                        if (W.start[a + st] <= idx) a += st;
                }
                aa[u] = a;
                ka[u] = idx - W.start[a];
                ea[u] = va[u] ? L.nbr[(size_t)ka[u] * n + W.idx[a]] : 0;
            }
            p0 += 64;
            if constexpr (MIXED) {
                float4 pj[2];
#pragma unroll
                for (int u = 0; u < 2; ++u)
                    if (va[u]) pj[u] = ld4f(A.pos32, ea[u] & kNbrIndexMask);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    bool nr = false;
                    if (va[u]) {
                        const float4 pi = W.p[aa[u]];
                        const float4 so = soff[(unsigned)ea[u] >> kNbrIndexBits];
                        const float xi[3] = {pi.x, pi.y, pi.z}, xj[3] = {pj[u].x, pj[u].y, pj[u].z};
                        const float oh[3] = {so.x, so.y, so.z};
                        float d[3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            d[c] = (xi[c] - xj[c]) - oh[c];
                            if (single[c]) d[c] -= rintf(d[c] * iprd[c]) * prd[c];
                        }
                        const float rq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
                        const float rs = (pi.w + pj[u].w) * 1.00001f;
                        nr = rq < rs * rs;
                    }
                    const uint32_t bal = __ballot_sync(0xffffffffu, nr);
                    if (nr) {
                        const int q = (qtail + __popc(bal & lanemask_lt())) & (kRing - 1);
                        W.qe[q] = ea[u];
                        W.qak[q] = (uint32_t)aa[u] | ((uint32_t)ka[u] << 5);
                        W.qp[q] = pj[u];
                        W.near[aa[u]] = 1u;
                    }
                    qtail += __popc(bal);
                }
            } else {
                double4 pj[2];
#pragma unroll
                for (int u = 0; u < 2; ++u)
                    if (va[u]) pj[u] = ld4(A.xr, ea[u] & kNbrIndexMask);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    bool nr = false;
                    if (va[u]) {
                        const double4 pi = W.p[aa[u]];
                        double d[3] = {pi.x - pj[u].x, pi.y - pj[u].y, pi.z - pj[u].z};
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            if (per[c] == 1) d[c] = image_sub64(d[c], rint(d[c] * iprd[c]), prd[c]);
                        // the contact test itself, as the law makes it (|d|^2 of either orientation)
                        const double rsq = rsq64(d);
                        const double radsum = pi.w + pj[u].w;
                        nr = rsq < __dmul_rn(radsum, radsum) && rsq > 1e-28;
                    }
                    const uint32_t bal = __ballot_sync(0xffffffffu, nr);
                    if (nr) {
                        const int q = (qtail + __popc(bal & lanemask_lt())) & (kRing - 1);
                        W.qe[q] = ea[u];
                        W.qak[q] = (uint32_t)aa[u] | ((uint32_t)ka[u] << 5);
                        W.near[aa[u]] = 1u;
                    }
                    qtail += __popc(bal);
                }
            }
            __syncwarp();
        }
        // 5. finish the roster atoms
        __syncwarp();
        if (mine) {
            const uint64_t nt = W.ntouch[lane];
            if (hist && nt != touch) L.touch[i] = nt;
            if (W.near[lane]) {
                atomicOr(&cwords[wib][uq], 1u << bit);
                T F[3], Tq[3], V[6], vi[3], wi[3], mi;
                if constexpr (MIXED) {
                    const float4 s0 = W.acc[0][lane], s1 = W.acc[1][lane], s2 = W.acc[2][lane];
                    F[0] = s0.x; F[1] = s0.y; F[2] = s0.z; Tq[0] = s0.w;
                    Tq[1] = s1.x; Tq[2] = s1.y; V[0] = s1.z; V[1] = s1.w;
                    V[2] = s2.x; V[3] = s2.y; V[4] = s2.z; V[5] = s2.w;
                    const float4 v = W.v[lane], w = W.w[lane];
                    vi[0] = v.x; vi[1] = v.y; vi[2] = v.z; mi = v.w;
                    wi[0] = w.x; wi[1] = w.y; wi[2] = w.z;
                } else {
                    const double2 s0 = W.acc[0][lane], s1 = W.acc[1][lane], s2 = W.acc[2][lane],
                                  s3 = W.acc[3][lane], s4 = W.acc[4][lane], s5 = W.acc[5][lane];
                    F[0] = s0.x; F[1] = s0.y; F[2] = s1.x; Tq[0] = s1.y; Tq[1] = s2.x; Tq[2] = s2.y;
                    V[0] = s3.x; V[1] = s3.y; V[2] = s4.x; V[3] = s4.y; V[4] = s5.x; V[5] = s5.y;
                    const double4 v = W.v[lane], w = W.w[lane];
                    vi[0] = v.x; vi[1] = v.y; vi[2] = v.z; mi = v.w;
                    wi[0] = w.x; wi[1] = w.y; wi[2] = w.z;
                }
                if (E->cundall) {  // FixDampingCundall.post_force_kernel
                    T gl, ga;
                    if constexpr (MIXED) {
                        gl = E->gamma_lin32;
                        ga = E->gamma_ang32;
                    } else {
                        gl = E->gamma_lin;
                        ga = E->gamma_ang;
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const T sf = F[c] * vi[c] >= T(0) ? T(1) : T(-1);
                        F[c] *= T(1) - gl * sf;
                        const T st = Tq[c] * wi[c] >= T(0) ? T(1) : T(-1);
                        Tq[c] *= T(1) - ga * st;
                    }
                }
                if constexpr (MIXED) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        A.f32[c * n + i] = F[c];
                        A.torque32[c * n + i] = Tq[c];
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        A.f[c * n + i] = F[c];
                        A.torque[c * n + i] = Tq[c];
                    }
                }
                // kinetic part of the virial with the end-of-step velocity
                // v(t+dt) = v(t+dt/2) + dt/2 f/m (thermo.py:94-101): A counted
                // m v(t+dt/2) v(t+dt/2) for every atom; the difference goes here
                // (the same products from the same words, so a zero force adds an
                // exact zero)
                T im;
                if constexpr (MIXED) im = __fdividef(1.0f, mi);
                else im = A.rinv[i];
                const T hdt = T(0.5) * dt;
                T vf[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) vf[c] = vi[c] + hdt * (F[c] * im);
                const T kin[6] = {(mi * vf[0]) * vf[0], (mi * vf[1]) * vf[1], (mi * vf[2]) * vf[2],
                                  (mi * vf[0]) * vf[1], (mi * vf[0]) * vf[2], (mi * vf[1]) * vf[2]};
                const T kh[6] = {(mi * vi[0]) * vi[0], (mi * vi[1]) * vi[1], (mi * vi[2]) * vi[2],
                                 (mi * vi[0]) * vi[1], (mi * vi[0]) * vi[2], (mi * vi[1]) * vi[2]};
                if constexpr (MIXED) {
                    // kin - kh is exact where the force changed v little (Sterbenz); elsewhere
                    // kh is the smaller term and the difference rounds once, as kin did
#pragma unroll
                    for (int c = 0; c < 6; ++c) dw_add(Vh[c], Vl[c], V[c] + (kin[c] - kh[c]));
                } else {
#pragma unroll
                    for (int c = 0; c < 6; ++c) Vd[c] += (V[c] + kin[c]) - kh[c];
                }
            }
        }
    };

    if constexpr (DENSE) {
        // Per-atom rows (the contact-dense path): every atom, one lane each,
        // whole 32-atom groups per warp.  Its row entries are loaded four at a
        // time (coalesced over the lanes) with their partners' high position
        // words, and the near test (the screened path's, word for word) marks
        // the near slots; the contacts of the near slots then run in ascending
        // slot order, each lane on its own atom, summed into the atom's force,
        // torque and virial in that order -- the sums the screened path forms
        // for the same atom.  Nothing is staged in shared memory and no group
        // is ruled out, which suits a state where nearly every atom touches.
        for (int base = bid * (int)blockDim.x + (int)(threadIdx.x & ~31u); base < n; base += nblk * (int)blockDim.x) {
            const int i = base + lane;
            const bool mine = i < n;
            S4 Pi{}, Vi{}, Wi{};
            float4 PLi = make_float4(0.f, 0.f, 0.f, 0.f);
            int32_t Ci = 0;
            int nn = 0;
            uint64_t touch = 0ull;
            if (mine) {
                nn = L.nnb[i];
                if (hist) touch = L.touch[i];
                if constexpr (MIXED) {
                    Pi = ld4f(A.pos32, i);
                    PLi = ld4f(A.pos32lo, i);
                    Vi = ld4f(A.vel32, i);
                    Wi = ld4f(A.om32, i);
                    if (vremap) Ci = A.cell32[i];
                } else {
                    Pi = ld4(A.xr, i);
                    Vi = ld4(A.vm, i);
                    Wi = ld4(A.om, i);
                }
            }
            const uint32_t old = flags[base >> 5];
            // near test of the row, four entries at a time
            uint64_t nmask = 0ull;
            for (int k0 = 0; k0 < nn; k0 += 4) {
                int ee[4];
                S4 pj[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) ee[u] = k0 + u < nn ? L.nbr[(size_t)(k0 + u) * n + i] : 0;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (k0 + u < nn) {
                        if constexpr (MIXED) pj[u] = ld4f(A.pos32, ee[u] & kNbrIndexMask);
                        else pj[u] = ld4(A.xr, ee[u] & kNbrIndexMask);
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (k0 + u >= nn) continue;
                    bool nr;
                    if constexpr (MIXED) {
                        const float4 so = soff[(unsigned)ee[u] >> kNbrIndexBits];
                        const float xi[3] = {Pi.x, Pi.y, Pi.z}, xj[3] = {pj[u].x, pj[u].y, pj[u].z};
                        const float oh[3] = {so.x, so.y, so.z};
                        float d[3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            d[c] = (xi[c] - xj[c]) - oh[c];
                            if (single[c]) d[c] -= rintf(d[c] * iprd[c]) * prd[c];
                        }
                        const float rq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
                        const float rs = (Pi.w + pj[u].w) * 1.00001f;
                        nr = rq < rs * rs;
                    } else {
                        double d[3] = {Pi.x - pj[u].x, Pi.y - pj[u].y, Pi.z - pj[u].z};
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            if (per[c] == 1) d[c] = image_sub64(d[c], rint(d[c] * iprd[c]), prd[c]);
                        const double rsq = rsq64(d);
                        const double radsum = Pi.w + pj[u].w;
                        nr = rsq < __dmul_rn(radsum, radsum) && rsq > 1e-28;
                    }
                    if (nr) nmask |= 1ull << (k0 + u);
                }
            }
            // the near slots' contacts in ascending slot order (each contact's
            // loads issued together, then its evaluation; issuing the next
            // contact's loads before evaluating the current one was measured
            // slower: the second set of registers spills)
            T F[3] = {0, 0, 0}, Tq[3] = {0, 0, 0}, V[6] = {0, 0, 0, 0, 0, 0};
            uint64_t nt = 0ull;
            for (uint64_t m = nmask; m; m &= m - 1ull) {
                const int k = __ffsll((long long)m) - 1;
                const int e = L.nbr[(size_t)k * n + i];
                S4 Pj;
                if constexpr (MIXED) Pj = ld4f(A.pos32, e & kNbrIndexMask);
                else Pj = ld4(A.xr, e & kNbrIndexMask);
                const CfLoad<MIXED> cl = contact_fetch(i, e, k, ((touch >> k) & 1ull) != 0, Pj);
                T fc[3] = {0, 0, 0}, tc[3] = {0, 0, 0}, vc[6] = {0, 0, 0, 0, 0, 0};
                if (contact_eval(i, e, k, Pi, PLi, Vi, Wi, Ci, cl, fc, tc, vc)) nt |= 1ull << k;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    F[c] += fc[c];
                    Tq[c] += tc[c];
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) V[c] += vc[c];
            }
            // finish the atom (the screened path's step 5)
            if (mine) {
                if (hist && nt != touch) L.touch[i] = nt;
                if (nmask != 0ull) {
                    const T vi[3] = {Vi.x, Vi.y, Vi.z}, wi[3] = {Wi.x, Wi.y, Wi.z};
                    const T mi = Vi.w;
                    if (E->cundall) {  // FixDampingCundall.post_force_kernel
                        T gl, ga;
                        if constexpr (MIXED) {
                            gl = E->gamma_lin32;
                            ga = E->gamma_ang32;
                        } else {
                            gl = E->gamma_lin;
                            ga = E->gamma_ang;
                        }
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const T sf = F[c] * vi[c] >= T(0) ? T(1) : T(-1);
                            F[c] *= T(1) - gl * sf;
                            const T st = Tq[c] * wi[c] >= T(0) ? T(1) : T(-1);
                            Tq[c] *= T(1) - ga * st;
                        }
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        if constexpr (MIXED) {
                            A.f32[c * n + i] = F[c];
                            A.torque32[c * n + i] = Tq[c];
                        } else {
                            A.f[c * n + i] = F[c];
                            A.torque[c * n + i] = Tq[c];
                        }
                    }
                    T im;
                    if constexpr (MIXED) im = __fdividef(1.0f, mi);
                    else im = A.rinv[i];
                    const T hdt = T(0.5) * dt;
                    T vf[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) vf[c] = vi[c] + hdt * (F[c] * im);
                    const T kin[6] = {(mi * vf[0]) * vf[0], (mi * vf[1]) * vf[1], (mi * vf[2]) * vf[2],
                                      (mi * vf[0]) * vf[1], (mi * vf[0]) * vf[2], (mi * vf[1]) * vf[2]};
                    const T kh[6] = {(mi * vi[0]) * vi[0], (mi * vi[1]) * vi[1], (mi * vi[2]) * vi[2],
                                     (mi * vi[0]) * vi[1], (mi * vi[0]) * vi[2], (mi * vi[1]) * vi[2]};
                    if constexpr (MIXED) {
#pragma unroll
                        for (int c = 0; c < 6; ++c) dw_add(Vh[c], Vl[c], V[c] + (kin[c] - kh[c]));
                    } else {
#pragma unroll
                        for (int c = 0; c < 6; ++c) Vd[c] += (V[c] + kin[c]) - kh[c];
                    }
                }
            }
            // the group's new flag word; stale forces of atoms no longer flagged
            const uint32_t w = __ballot_sync(0xffffffffu, mine && nmask != 0ull);
            if (lane == 0 && w != old) flags[base >> 5] = w;
            if (mine && ((old >> lane) & 1u) && !((w >> lane) & 1u)) zero_force<MIXED>(A, i);
        }
    } else {
    if (lane < kLive) cwords[wib][lane] = 0u;
    __syncwarp();
    // Ordered pass: after the first pass that follows the bounds (which
    // visits every group, clears the flags of those it rules out and their
    // stale forces), thr only grows until the next bounds, so a group ruled
    // out stays out with its flags clear, and the live groups are a prefix of
    // the ascending gap order.  Walking that order instead of the group
    // index gives every warp the same number of live groups (+-1).
    const bool ordered = cull && E->order_ready != 0;
    for (int base = gw; base < ngroups; base += 32 * nwarps) {
        const int k = base + lane * nwarps;
        int mygrp = k;
        uint32_t myold = 0u;
        bool live = false;
        if (k < ngroups) {
            if (ordered) {
                mygrp = order[k];
                live = !(sgap[k] > thr);
            } else {
                myold = flags[mygrp];
                live = !(cull && gap[mygrp] > thr);
                if (!live && myold != 0u) {
                    // ruled out now, flagged last step: clear the stale forces
                    for (uint32_t w = myold; w; w &= w - 1) zero_force<MIXED>(A, (mygrp << 5) + __ffs(w) - 1);
                    flags[mygrp] = 0u;
                }
            }
        }
        uint32_t pending = __ballot_sync(0xffffffffu, live);
        if (ordered && pending == 0u) break;  // no later position of this warp is live
        while (pending) {
            // up to kLive live groups at once
            int gq[kLive];
            uint32_t oq[kLive], nw[kLive];
            int nq = 0;
#pragma unroll
            for (int u = 0; u < kLive; ++u) {
                gq[u] = 0;
                oq[u] = 0u;
                if (pending) {
                    const int src = __ffs(pending) - 1;
                    pending &= pending - 1;
                    gq[u] = __shfl_sync(0xffffffffu, mygrp, src);
                    oq[u] = __shfl_sync(0xffffffffu, myold, src);
                    nq = u + 1;
                }
            }
            // the atoms' own bounds (and, in the ordered pass, the groups'
            // flag words), all issued at once
            float ag[kLive];
#pragma unroll
            for (int u = 0; u < kLive; ++u) {
                const int i = (gq[u] << 5) + lane;
                ag[u] = (u < nq && i < n) ? agap[i] : 0.0f;
                if (ordered && u < nq) oq[u] = flags[gq[u]];
            }
            int near_total = 0;
#pragma unroll
            for (int u = 0; u < kLive; ++u) {
                const int i = (gq[u] << 5) + lane;
                nw[u] = __ballot_sync(0xffffffffu, u < nq && i < n && !(cull && ag[u] > thr));
                near_total += __popc(nw[u]);
            }
            // park the batch in shared memory while its rosters run (registers go to the law)
            if (lane < kLive) {
#pragma unroll
                for (int u = 0; u < kLive; ++u) {
                    if (u == lane) {
                        bgrp[wib][u] = gq[u];
                        bold[wib][u] = oq[u];
                        bnear[wib][u] = nw[u];
                    }
                }
            }
            __syncwarp();
            // the near atoms, 32 at a time, in group then atom order: one roster each
            for (int r0 = 0; r0 < near_total; r0 += 32) {
                const int idx = r0 + lane;
                int uq = -1, bit = 0, acc = 0, g = 0;
                for (int u = 0; u < nq; ++u) {
                    const uint32_t w = bnear[wib][u];
                    const int c = __popc(w);
                    if (uq < 0 && idx < acc + c) {
                        uq = u;
                        bit = nth_bit(w, idx - acc);
                        g = bgrp[wib][u];
                    }
                    acc += c;
                }
                const int count = near_total - r0 < 32 ? near_total - r0 : 32;
                roster(count, uq >= 0 ? (g << 5) + bit : 0, uq < 0 ? 0 : uq, bit);
            }
            __syncwarp();
            // new flag words; stale forces of atoms no longer flagged
            for (int u = 0; u < nq; ++u) {
                const uint32_t w = cwords[wib][u], old = bold[wib][u];
                const int g = bgrp[wib][u];
                const int i = (g << 5) + lane;
                if (lane == 0 && w != old) flags[g] = w;
                if (i < n && ((old >> lane) & 1u) && !((w >> lane) & 1u)) zero_force<MIXED>(A, i);
            }
            __syncwarp();
            if (lane < kLive) cwords[wib][lane] = 0u;
            __syncwarp();
        }
    }
    }  // screened path
    if constexpr (MIXED) {
        block_sum_dw<6, kBlockC>(Vh, Vl, reinterpret_cast<float2*>(smem));
        if (threadIdx.x == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) reinterpret_cast<float2*>(part)[(size_t)c * nb + bid] = make_float2(Vh[c], Vl[c]);
        }
    } else {
        block_sum<6, kBlockC>(Vd, smem);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) part[(size_t)c * nb + bid] = Vd[c];
        }
    }
    if (threadIdx.x == 0 && bid == 0) E->final_pending = 1;
}

template <int STYLE, bool MIXED, bool DENSE = false>
__global__ void __launch_bounds__(kBlockC, MIXED ? 4 : 3)
    k_cf(tmps_atoms A, tmps_nlist L, tmps_pair_params P, const tmps_box* __restrict__ B,
         tmps_engine* __restrict__ E, uint32_t* __restrict__ flags, const float* __restrict__ gap,
         const float* __restrict__ agap, double* __restrict__ part) {
    const char* sc = reinterpret_cast<const char*>(flags);  // the scratch base
    cf_body<STYLE, MIXED, DENSE>(A, L, P, B, E, flags, gap, agap, reinterpret_cast<const int32_t*>(sc + lay_order(A.n)),
                          reinterpret_cast<const float*>(sc + lay_sgap(A.n)), part, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------- S

__device__ double limit_rate_f(double rate, double ptarget, int normalize, double max_rate) {
    double out = rate;
    if (normalize) {
        if (ptarget == 0.0) {
            if (out != 0.0) out = copysign(max_rate, out);
        } else {
            out = out / fabs(ptarget);
        }
    }
    if (max_rate != 0.0 && fabs(out) > max_rate) out = copysign(max_rate, out);
    return out;
}

constexpr int kBlockS = 768;  // four warps per virial component

// The servo's arithmetic on staged copies of the three structs.  On this
// part an FP64 instruction costs ~64 cycles of latency and a division ~670,
// however few lanes are active, so the work is laid out for the SM's four
// FP64 units: warp 0 runs the serial chain (pressure -> rate -> new box,
// lane k < 6 one pressure component, lane d < 3 one dimension), then the
// independent derived quantities are spread over the block's warps.  Each
// value is the same FP64 expression as a one-thread form would compute.
struct ServoNew {
    double lo[3], hi[3], prd[3];   // new box
    double olo[3], oprd[3];        // old box
    int bad;
};

__device__ void servo_chain_warp(const tmps_box& b, tmps_servo& sv, const tmps_engine& e, const double* acc,
                                 ServoNew& o) {
    const int lane = threadIdx.x & 31;
    const double dt = e.dt;
    const double vol = b.prd[0] * b.prd[1] * b.prd[2];
    double t = 0.0;
    if (lane < 6) {
        t = vol > 0.0 ? acc[lane] / vol : 0.0;
        sv.pressure[lane] = t;
    }
    const double t0 = __shfl_sync(0xffffffffu, t, 0), t1 = __shfl_sync(0xffffffffu, t, 1),
                 t2 = __shfl_sync(0xffffffffu, t, 2);
    const int d = lane;
    double nprd = 1.0;
    if (lane < 3) {
        const double lo = b.lo[d], prd = b.prd[d];
        double nlo = lo, nhi = b.hi[d];
        const int st = sv.style[d];
        const double ls = sv.lo_start[d], hs = sv.hi_start[d];
        if (st >= 1 && st <= 4) {
            const double elapsed = (double)sv.nsteps * dt;
            if (st == 1) {
                const double shift = ((0.5 * elapsed) * sv.rate[d]) * (hs - ls);
                nlo = ls - shift; nhi = hs + shift;
            } else if (st == 2) {
                const double mid = 0.5 * (ls + hs);
                const double half = (0.5 * (hs - ls)) * exp(sv.rate[d] * elapsed);
                nlo = mid - half; nhi = mid + half;
            } else if (st == 3) {
                const double shift = (0.5 * elapsed) * sv.vel[d];
                nlo = ls - shift; nhi = hs + shift;
            } else {
                const double shift = (0.5 * sv.amp[d]) * sin(((2.0 * 3.14159265358979323846) * elapsed) / sv.tper[d]);
                nlo = ls - shift; nhi = hs + shift;
            }
        } else if (st >= 5 && st <= 7) {
            const double frac = sv.nsteps_total > 0 ? (double)sv.nsteps / (double)sv.nsteps_total : 0.0;
            if (st == 5) {
                nlo = ls + frac * (sv.flo[d] - ls);
                nhi = hs + frac * (sv.fhi[d] - hs);
            } else if (st == 6) {
                const double lo_stop = ls + sv.dlo[d], hi_stop = hs + sv.dhi[d];
                nlo = ls + frac * (lo_stop - ls);
                nhi = hs + frac * (hi_stop - hs);
            } else {
                const double mid = 0.5 * (ls + hs);
                const double half = (0.5 * sv.scale[d]) * (hs - ls);
                nlo = ls + frac * ((mid - half) - ls);
                nhi = hs + frac * ((mid + half) - hs);
            }
        } else if (st == 8 || st == 9) {
            // coupled axes share their mean pressure; style 9 (pressure/scalar)
            // with no coupling uses the scalar pressure
            const double scalar = ((t0 + t1) + t2) / 3.0;
            double pd = d == 0 ? t0 : (d == 1 ? t1 : t2);
            if (sv.couple == 1) pd = scalar;
            else if (sv.couple == 2 && d < 2) pd = (t0 + t1) / 2.0;
            else if (sv.couple == 3 && d > 0) pd = (t1 + t2) / 2.0;
            else if (sv.couple == 4 && d != 1) pd = (t0 + t2) / 2.0;
            if (sv.couple == 0 && st == 9) pd = scalar;
            const double tgt = sv.ptarget[d];
            const double rate = limit_rate_f(sv.pgain[d] * (pd - tgt), tgt, sv.normalize, sv.max_rate);
            sv.cum[d] += (dt * rate) * prd;
            nlo = ls - 0.5 * sv.cum[d];
            nhi = hs + 0.5 * sv.cum[d];
        }
        o.lo[d] = nlo;
        o.hi[d] = nhi;
        o.olo[d] = lo;
        o.oprd[d] = prd;
    }
    if (sv.post) {
        // volume and box styles: one lane over the three axes' targets
        __syncwarp();
        if (lane == 0) {
            const double tt[6] = {t0, t1, t2, 0.0, 0.0, 0.0};
            servo_post(sv, o.oprd, tt, dt, o.lo, o.hi);
        }
        __syncwarp();
    }
    if (lane < 3) {
        nprd = o.hi[d] - o.lo[d];
        o.prd[d] = nprd;
    }
    const bool bad = __any_sync(0xffffffffu, !(nprd > 0.0));
    if (lane == 0) o.bad = bad ? 1 : 0;
}

// The quantities derived from the new box, one kind per warp (lanes 0..2 =
// dimensions); nothing is written when the new box is not positive.
__device__ void servo_derive(tmps_box& b, const tmps_servo& sv, tmps_engine& e, const ServoNew& o) {
    if (o.bad) return;
    const int warp = threadIdx.x >> 5, d = threadIdx.x & 31;
    if (d >= 3) return;
    const double nprd = o.prd[d], prd = o.oprd[d];
    switch (warp) {
        case 0:
            b.inv_prd[d] = 1.0 / nprd;
            if (e.mixed) e.iprd32[d] = (float)b.inv_prd[d];
            break;
        case 1: {
            const double hc = nprd / (double)b.g[d];
            b.hcell[d] = hc;
            if (e.mixed) {
                split(hc, e.h32[d], e.hlo32[d]);
                e.dh32[d] = (float)(hc - e.h0[d]);
            }
            break;
        }
        case 2:
            b.h_rate[d] = (nprd - prd) / e.dt;
            b.h_rate[3 + d] = 0.0;
            break;
        case 3:
            if (e.mixed) split((nprd - prd) / prd, e.eps_hi[d], e.eps_lo[d]);
            else e.remap_scale[d] = nprd / prd;
            break;
        case 4:
            if (e.mixed) {
                split(nprd, e.prd32[d], e.prdlo32[d]);
                e.dlo32[d] = (float)(o.lo[d] - e.lo0[d]);
            }
            break;
        case 5: {
            b.old_lo[d] = o.olo[d];
            b.old_prd[d] = prd;
            b.lo[d] = o.lo[d];
            b.hi[d] = o.hi[d];
            b.prd[d] = nprd;
            if (e.cull) {
                // change of the periodic image shifts since the contact bounds' reference
                const double dd = fabs(nprd - e.prd_ref[d]);
                const double d1 = __shfl_sync(0x7u, dd, 1), d2 = __shfl_sync(0x7u, dd, 2);
                if (d == 0) e.shift_bound = fmaxf(e.shift_bound, __double2float_ru((dd + d1) + d2));
            }
            if (d == 0) {
                b.vremap = sv.remap == 2 ? 1 : 0;
                b.remap_pending = sv.remap == 1 ? 1 : 0;
            }
            break;
        }
        default:
            break;
    }
}

template <typename S>
__device__ __forceinline__ void copy_words(S* dst, const S* src) {
    static_assert(sizeof(S) % 4 == 0, "struct size");
    const uint32_t* a = reinterpret_cast<const uint32_t*>(src);
    uint32_t* o = reinterpret_cast<uint32_t*>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(S) / 4); k += blockDim.x) o[k] = a[k];
}

// S: finish the step.  Decide the rebuild, sum the virial partials of A and
// C in a fixed order, run the servo.  The box and servo structs are written
// by S alone, and the previous step's S has completed before this one can
// start, so they are staged before the dependency wait; the engine struct
// (A and C write parts of it) after.  The partials are component-major,
// [6][nblocks]: four warps per component each take every fourth run of 32
// blocks (coalesced, all loads of a lane in flight at once), then a shuffle
// tree and the four warp sums in order.  The mixed form's partials are
// double words and are summed as such; only the six totals become FP64.
constexpr int kWarpsS = kBlockS / 32;
static_assert(kWarpsS == 24, "four warps per virial component");
constexpr int kPartLoads = 10;  // per lane: up to 32 * 4 * 10 = 1280 partial blocks in one round

template <typename V, typename Add>
__device__ __forceinline__ V sum_component(const V* row, int nb, int q, int lane, V zero, Add add) {
    V acc = zero;
    for (int k0 = q * 32 + lane; k0 < nb; k0 += 128 * kPartLoads) {
        V v[kPartLoads];
#pragma unroll
        for (int u = 0; u < kPartLoads; ++u) {
            const int k = k0 + 128 * u;
            v[u] = k < nb ? row[k] : zero;
        }
#pragma unroll
        for (int u = 0; u < kPartLoads; ++u) acc = add(acc, v[u]);
    }
    return acc;
}

__device__ __forceinline__ void s_body(tmps_box* b, tmps_servo* sv, tmps_engine* e, const char* scratch,
                                       int32_t* status) {
    __shared__ double tot[6];
    __shared__ double wsum[kWarpsS];
    __shared__ float2 wsumf[kWarpsS];
    __shared__ tmps_box sb;
    __shared__ tmps_servo ssv;
    __shared__ tmps_engine se;
    __shared__ ServoNew snew;
    copy_words(&sb, b);
    copy_words(&ssv, sv);
    // run constants of the engine record (only the host changes them, between
    // launches), so the partial sums can be fetched with this step's words
    const int nb = e->nblocks;
    const int64_t part_off = e->part_off;
    const bool mixed = e->mixed != 0, servo = e->servo != 0;
    __syncthreads();
    const bool servo_now = servo && ((ssv.step_count + 1) % ssv.nevery == 0);
    pdl_enter();
    // this step's engine words (A and C write some) and the virial partials in
    // flight together; one word per thread (the batched S has 192 threads)
    constexpr int kEngineWords = (int)(sizeof(tmps_engine) / 4);
    static_assert(kEngineWords <= 192, "one engine word per thread of the batched S");
    const uint32_t ew = (int)threadIdx.x < kEngineWords ? reinterpret_cast<const uint32_t*>(e)[threadIdx.x] : 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (servo_now) {
        const double* part = reinterpret_cast<const double*>(scratch + part_off);
        // kWarpsS virtual warps, four per component; a block of fewer warps
        // runs several in turn, with the same arithmetic each
        if (mixed) {
            for (int vw = warp; vw < kWarpsS; vw += (int)(blockDim.x >> 5)) {
                const int c = vw >> 2, q = vw & 3;
                const float2* row = reinterpret_cast<const float2*>(part) + (size_t)c * nb;
                float2 acc = sum_component(row, nb, q, lane, make_float2(0.0f, 0.0f), [](float2 x, float2 y) {
                    dw_add2(x.x, x.y, y.x, y.y);
                    return x;
                });
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float bh = __shfl_down_sync(0xffffffffu, acc.x, o),
                                bl = __shfl_down_sync(0xffffffffu, acc.y, o);
                    dw_add2(acc.x, acc.y, bh, bl);
                }
                if (lane == 0) wsumf[vw] = acc;
            }
        } else {
            for (int vw = warp; vw < kWarpsS; vw += (int)(blockDim.x >> 5)) {
                const int c = vw >> 2, q = vw & 3;
                const double* row = part + (size_t)c * nb;
                double t = sum_component(row, nb, q, lane, 0.0, [](double x, double y) { return x + y; });
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
                if (lane == 0) wsum[vw] = t;
            }
        }
    }
    if ((int)threadIdx.x < kEngineWords) reinterpret_cast<uint32_t*>(&se)[threadIdx.x] = ew;
    __syncthreads();
    if (se.aborted || se.step >= se.stop_step) return;
    const int64_t s = se.step + 1;
    if (rebuild_due(&se, s)) {
        if (threadIdx.x == 0) e->aborted = 1;
        return;
    }
    if (servo_now) {
        if (threadIdx.x < 6) {
            if (mixed) {
                float h = 0.0f, l = 0.0f;
#pragma unroll
                for (int w = 0; w < 4; ++w) dw_add2(h, l, wsumf[4 * threadIdx.x + w].x, wsumf[4 * threadIdx.x + w].y);
                tot[threadIdx.x] = (double)h + (double)l;
            } else {
                tot[threadIdx.x] = ((wsum[4 * threadIdx.x] + wsum[4 * threadIdx.x + 1]) + wsum[4 * threadIdx.x + 2]) +
                                   wsum[4 * threadIdx.x + 3];
            }
        }
        __syncthreads();
    }
    if (warp == 0) {
        if (lane == 0) {
            se.step = s;
            se.order_ready = se.cull;  // C has had its first pass since the bounds
            sb.remap_pending = 0;
            if (se.servo) {
                ssv.step_count += 1;
                ssv.nsteps += 1;
            }
        }
        __syncwarp();
        if (servo_now) {
            servo_chain_warp(sb, ssv, se, tot, snew);
            if (lane == 0 && snew.bad) atomicOr(status, TMPS_STATUS_BOX_NONPOSITIVE);
            if (se.plog != nullptr && se.plog_len > 0 && lane < 6)
                se.plog[(size_t)(s % se.plog_len) * 6 + lane] = ssv.pressure[lane];
        }
    }
    __syncthreads();
    if (servo_now) {
        servo_derive(sb, ssv, se, snew);
        __syncthreads();
    }
    copy_words(e, &se);
    copy_words(b, &sb);
    copy_words(sv, &ssv);
}

__global__ void __launch_bounds__(kBlockS) k_s(tmps_box* b, tmps_servo* sv, tmps_engine* e, const char* scratch,
                                               int32_t* status) {
    s_body(b, sv, e, scratch, status);
}

// ---------------------------------------------------------------- batched
// Every block of a batched grid belongs to one instance (block_inst) and runs
// that instance's single-instance body with its instance-local block index,
// over the instance's own arrays.  The descriptors are written by the host
// between chunks, never by these kernels, so they are read before the
// dependency wait.

// The block's descriptor, staged in shared memory: the bodies then read its
// fields with shared loads instead of holding a register copy of every one.
__device__ __forceinline__ const tmps_instance& stage_instance(tmps_instance& si, const tmps_instance* inst, int i) {
    copy_words(&si, &inst[i]);
    __syncthreads();
    return si;
}

__global__ void __launch_bounds__(kBlockA) kb_a64(const tmps_instance* __restrict__ inst,
                                                   const int32_t* __restrict__ block_inst) {
    __shared__ tmps_instance si;
    const tmps_instance& I = stage_instance(si, inst, block_inst[blockIdx.x]);
    char* sc = static_cast<char*>(I.scratch);
    a64_body(I.a, I.box, I.eng, reinterpret_cast<const uint32_t*>(sc), reinterpret_cast<double*>(sc + lay_part(I.a.n)),
             (int)blockIdx.x - I.a_first, I.a_blocks);
}

__global__ void __launch_bounds__(kBlockA, 4) kb_a32(const tmps_instance* __restrict__ inst,
                                                      const int32_t* __restrict__ block_inst) {
    __shared__ tmps_instance si;
    const tmps_instance& I = stage_instance(si, inst, block_inst[blockIdx.x]);
    char* sc = static_cast<char*>(I.scratch);
    a32_body(I.a, I.box, I.eng, reinterpret_cast<const uint32_t*>(sc), reinterpret_cast<double*>(sc + lay_part(I.a.n)),
             (int)blockIdx.x - I.a_first, I.a_blocks);
}

template <int STYLE, bool MIXED>
__global__ void __launch_bounds__(kBlockC, MIXED ? 4 : 3)
    kb_cf(const tmps_instance* __restrict__ inst, const int32_t* __restrict__ block_inst) {
    __shared__ tmps_instance si;
    const tmps_instance& I = stage_instance(si, inst, block_inst[blockIdx.x]);
    char* sc = static_cast<char*>(I.scratch);
    const int n = I.a.n;
    double* part = reinterpret_cast<double*>(sc + lay_part(n));
    cf_body<STYLE, MIXED, false>(I.a, I.nl, I.p, I.box, I.eng, reinterpret_cast<uint32_t*>(sc),
                          reinterpret_cast<const float*>(sc + lay_gap(n)), reinterpret_cast<const float*>(sc + lay_agap(n)),
                          reinterpret_cast<const int32_t*>(sc + lay_order(n)),
                          reinterpret_cast<const float*>(sc + lay_sgap(n)), part, (int)blockIdx.x - I.c_first,
                          I.c_blocks);
}

// S of a batch: one block of six warps per instance (the derived quantities
// take one warp per kind, the virial sum runs the 24 virtual warps of the
// single-instance S four at a time), so many instances fit in one wave.
constexpr int kBlockSB = 192;
__global__ void __launch_bounds__(kBlockSB) kb_s(const tmps_instance* __restrict__ inst, int32_t* status) {
    const tmps_instance& I = inst[blockIdx.x];
    s_body(I.box, I.servo, I.eng, static_cast<const char*>(I.scratch), status);
}

__global__ void kb_state(const tmps_instance* __restrict__ inst, int ninst, int64_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const tmps_engine* e = inst[i].eng;
    out[2 * i] = e->step;
    out[2 * i + 1] = e->aborted;
}

// -------------------------------------------------------- prepare / unpack

__global__ void __launch_bounds__(kBlockA) k_prepare(tmps_atoms a, const tmps_box* __restrict__ b,
                                                      tmps_engine* __restrict__ e, const int32_t* cell_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    if (i >= n) return;
    const double4 x = ld4(a.xr, i), v = ld4(a.vm, i), w = ld4(a.om, i);
    const bool mixed = e->mixed != 0;
    // every load before the first store (a store could alias them as far as
    // the compiler knows, and would hold each later load back a round trip)
    double x0[3] = {0, 0, 0}, f[3] = {0, 0, 0}, t[3] = {0, 0, 0};
    int lin = 0;
    if (mixed) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            x0[k] = a.x0[k * n + i];
            f[k] = a.f[k * n + i];
            t[k] = a.torque[k * n + i];
        }
        lin = cell_of[i];
    }
    if (a.rinv) {
        const double rm = 1.0 / v.w, rI = 1.0 / w.w;
        a.rinv[i] = rm;
        a.rinv[n + i] = rI;
        // the FP64 update leaves out a zero force's kick only where 1/m and 1/I are positive and
        // finite (0 * inf is a NaN; a negative factor would keep a negative zero velocity)
        if (!(rm > 0.0 && isfinite(rm) && rI > 0.0 && isfinite(rI))) e->kick_all = 1;
    }
    if (!mixed) return;
    const int gx = b->g[0], gxy = b->g[0] * b->g[1];
    const int cz = lin / gxy, cy = (lin - cz * gxy) / gx, cx = lin - cz * gxy - cy * gx;
    const int cc[3] = {cx, cy, cz};
    const double xx[3] = {x.x, x.y, x.z};
    float oh[3], ol[3];
    for (int k = 0; k < 3; ++k) {
        const double origin = b->lo[k] + f64_of(__int2float_rn(cc[k])) * b->hcell[k];
        split(xx[k] - origin, oh[k], ol[k]);
        // the skin check's reference: the position at the last build, as an
        // offset from the same origin (x0 is kept by the build in FP64)
        a.o0_32[k * n + i] = f32_rn(x0[k] - origin);
    }
    a.cell32[i] = cx | (cy << 10) | (cz << 20);
    // the forces in hand (the setup forces at a run's start; at a rebuild C rewrites them first)
    for (int k = 0; k < 3; ++k) {
        a.f32[k * n + i] = f32_rn(f[k]);
        a.torque32[k * n + i] = f32_rn(t[k]);
    }
    float rh, rl;
    split(x.w, rh, rl);
    st4f(a.pos32, i, make_float4(oh[0], oh[1], oh[2], rh));
    st4f(a.pos32lo, i, make_float4(ol[0], ol[1], ol[2], rl));
    float vh[3], vlo[3], wh[3], wlo[3];
    split(v.x, vh[0], vlo[0]); split(v.y, vh[1], vlo[1]); split(v.z, vh[2], vlo[2]);
    split(w.x, wh[0], wlo[0]); split(w.y, wh[1], wlo[1]); split(w.z, wh[2], wlo[2]);
    // 1/m and 1/I of the mixed form's update: FP32 reciprocals of the FP32 values (within an ulp of
    // the rounded FP64 ones; no FP64 division)
    const float m32 = f32_rn(v.w), I32 = f32_rn(w.w);
    reinterpret_cast<float2*>(a.inv32)[i] = make_float2(__frcp_rn(m32), __frcp_rn(I32));
    store_vw<false>(a, i, make_float4(vh[0], vh[1], vh[2], m32), make_float4(vlo[0], vlo[1], vlo[2], 0.0f),
                    make_float4(wh[0], wh[1], wh[2], 0.0f), make_float4(wlo[0], wlo[1], wlo[2], 0.0f));
}

__global__ void k_prepare_engine(const tmps_box* __restrict__ b, tmps_engine* e, int64_t part_off) {
    if (threadIdx.x || blockIdx.x) return;
    e->part_off = part_off;
    e->cull = 0;  // until tmps_fused_bounds sets the bounds
    e->touching = 0;
    e->kick_all = 0;  // k_prepare, launched next, sets it for an atom of odd mass or inertia
    e->maxd2_bits = 0u;
    e->shift_bound = 0.0f;
    for (int d = 0; d < 3; ++d) {
        e->lo0[d] = b->lo[d];
        e->h0[d] = b->hcell[d];
        e->dlo32[d] = 0.0f;
        e->dh32[d] = 0.0f;
        split(b->hcell[d], e->h32[d], e->hlo32[d]);
        split(b->prd[d], e->prd32[d], e->prdlo32[d]);
        e->iprd32[d] = (float)b->inv_prd[d];
        e->single_bin[d] = (b->per[d] == 1 && b->g[d] == 1) ? 1 : 0;
        e->eps_hi[d] = 0.0f;
        e->eps_lo[d] = 0.0f;
    }
    split(e->dt, e->dt_hi, e->dt_lo);
    e->trigger32 = (float)e->trigger_sq;
    e->gamma_lin32 = (float)e->gamma_lin;
    e->gamma_ang32 = (float)e->gamma_ang;
}

__global__ void __launch_bounds__(kBlockA) k_unpack(tmps_atoms a, const tmps_box* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    if (i >= n) return;
    double4 x = ld4(a.xr, i), v = ld4(a.vm, i), w = ld4(a.om, i);
    const float4 p = ld4f(a.pos32, i), pl = ld4f(a.pos32lo, i);
    float4 vv, vl, ww, wl;
    load_vw<false>(a, i, vv, vl, ww, wl);
    const int32_t c = a.cell32[i];
    // the FP32 forces with the rest, before any store (see k_prepare)
    float f32[3], t32[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f32[k] = a.f32[k * n + i];
        t32[k] = a.torque32[k * n + i];
    }
    const int cc[3] = {cell_x(c), cell_y(c), cell_z(c)};
    const float oh[3] = {p.x, p.y, p.z}, ol[3] = {pl.x, pl.y, pl.z};
    double xx[3];
    // float -> double widenings with integer operations (exact; off the FP64 pipe)
    for (int k = 0; k < 3; ++k) xx[k] = (b->lo[k] + (double)cc[k] * b->hcell[k]) + (f64_of(oh[k]) + f64_of(ol[k]));
    x.x = xx[0]; x.y = xx[1]; x.z = xx[2];
    v.x = f64_of(vv.x) + f64_of(vl.x); v.y = f64_of(vv.y) + f64_of(vl.y); v.z = f64_of(vv.z) + f64_of(vl.z);
    w.x = f64_of(ww.x) + f64_of(wl.x); w.y = f64_of(ww.y) + f64_of(wl.y); w.z = f64_of(ww.z) + f64_of(wl.z);
    st4(a.xr, i, x);
    st4(a.vm, i, v);
    st4(a.om, i, w);
    for (int k = 0; k < 3; ++k) {
        a.f[k * n + i] = f64_of(f32[k]);
        a.torque[k * n + i] = f64_of(t32[k]);
    }
}

// Settle: the pending second half-kick and remap.
template <bool MIXED>
__global__ void __launch_bounds__(kBlockA) k_settle(tmps_atoms a, const tmps_box* __restrict__ b,
                                                     const tmps_engine* __restrict__ e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    if (i >= n) return;
    if constexpr (MIXED) {
        float4 p = ld4f(a.pos32, i), pl = ld4f(a.pos32lo, i);
        float4 v, vl, w, wl;
        load_vw<false>(a, i, v, vl, w, wl);
        if (e->final_pending) {
            const float dtf = 0.5f * e->dt_hi;
            const float km = dtf * vl.w, kI = dtf * wl.w;
            dw_add(v.x, vl.x, km * a.f32[i]);
            dw_add(v.y, vl.y, km * a.f32[n + i]);
            dw_add(v.z, vl.z, km * a.f32[2 * n + i]);
            dw_add(w.x, wl.x, kI * a.torque32[i]);
            dw_add(w.y, wl.y, kI * a.torque32[n + i]);
            dw_add(w.z, wl.z, kI * a.torque32[2 * n + i]);
        }
        if (b->remap_pending) {
            dw_add(p.x, pl.x, p.x * e->eps_hi[0] + (p.x * e->eps_lo[0] + pl.x * e->eps_hi[0]));
            dw_add(p.y, pl.y, p.y * e->eps_hi[1] + (p.y * e->eps_lo[1] + pl.y * e->eps_hi[1]));
            dw_add(p.z, pl.z, p.z * e->eps_hi[2] + (p.z * e->eps_lo[2] + pl.z * e->eps_hi[2]));
        }
        st4f(a.pos32, i, p);
        st4f(a.pos32lo, i, pl);
        store_vw<false>(a, i, v, vl, w, wl);
        return;
    }
    double4 x = ld4(a.xr, i), v = ld4(a.vm, i), w = ld4(a.om, i);
    if (e->final_pending) {
        {
            const double dtf = 0.5 * e->dt, im = a.rinv[i], iI = a.rinv[n + i];
            v.x += dtf * (a.f[i] * im); v.y += dtf * (a.f[n + i] * im); v.z += dtf * (a.f[2 * n + i] * im);
            w.x += dtf * (a.torque[i] * iI); w.y += dtf * (a.torque[n + i] * iI);
            w.z += dtf * (a.torque[2 * n + i] * iI);
        }
    }
    if (b->remap_pending) {
        x.x = b->lo[0] + (x.x - b->old_lo[0]) * e->remap_scale[0];
        x.y = b->lo[1] + (x.y - b->old_lo[1]) * e->remap_scale[1];
        x.z = b->lo[2] + (x.z - b->old_lo[2]) * e->remap_scale[2];
    }
    st4(a.xr, i, x);
    st4(a.vm, i, v);
    st4(a.om, i, w);
}

__global__ void k_set_log(tmps_engine* e, double* log, int32_t len) {
    if (threadIdx.x || blockIdx.x) return;
    e->plog = log;
    e->plog_len = log ? len : 0;
}

__global__ void k_settle_flags(tmps_box* b, tmps_engine* e) {
    if (threadIdx.x || blockIdx.x) return;
    e->final_pending = 0;
    b->remap_pending = 0;
}

bool launch_ok() { return cudaPeekAtLastError() == cudaSuccess; }

// Launch with programmatic stream serialization (see pdl_enter).
template <typename... P, typename... A>
void launch_pdl(void (*kernel)(P...), int grid, int block, cudaStream_t s, A&&... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

bool mixed_ok(const tmps_atoms* a) {
    return a->pos32 && a->pos32lo && a->vel32 && a->lo32 && a->om32 && a->wlz32 && a->inv32 && a->cell32 && a->f32 &&
           a->torque32 && a->o0_32;
}

int sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            sms = v;
        else
            sms = 152;
    }
    return sms;
}
// Grids of the two passes of C: exactly one wave of resident blocks each
// (occupancy of the kernel instance x SMs), so the static grid-stride split
// leaves no partial second wave.
template <typename K>
int wave_blocks(K kernel, int block) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, block, 0) != cudaSuccess || occ < 1) occ = 1;
    return occ * sm_count();
}
int contact_wave(int style, bool mixed) {
    static int w[5][2] = {};
    if (style < 0 || style > 4) style = 4;
    int& v = w[style][mixed ? 1 : 0];
    if (!v) {
        switch (style) {
            case 0: v = mixed ? wave_blocks(k_cf<0, true>, kBlockC) : wave_blocks(k_cf<0, false>, kBlockC); break;
            case 1: v = mixed ? wave_blocks(k_cf<1, true>, kBlockC) : wave_blocks(k_cf<1, false>, kBlockC); break;
            case 2: v = mixed ? wave_blocks(k_cf<2, true>, kBlockC) : wave_blocks(k_cf<2, false>, kBlockC); break;
            case 3: v = mixed ? wave_blocks(k_cf<3, true>, kBlockC) : wave_blocks(k_cf<3, false>, kBlockC); break;
            default: v = mixed ? wave_blocks(k_cf<4, true>, kBlockC) : wave_blocks(k_cf<4, false>, kBlockC); break;
        }
    }
    return v;
}
int a_wave(bool mixed) {
    static int w[2] = {0, 0};
    int& v = w[mixed ? 1 : 0];
    if (!v) v = mixed ? wave_blocks(k_a32, kBlockA) : wave_blocks(k_a64, kBlockA);
    return v;
}
int a_blocks(int n, bool mixed) { const int b = grid_for(n, kBlockA); return b < a_wave(mixed) ? b : a_wave(mixed); }
int contact_blocks(int n, int style, bool mixed) {
    const int b = grid_for(n, kBlockC);
    return b < contact_wave(style, mixed) ? b : contact_wave(style, mixed);
}
// Grids under a launch shape of g 32-atom groups per warp: one block per
// 256 g atoms for A (g passes of its grid-stride loop), one per 128 g atoms
// for C (g groups per warp, screened kLive at a time), never more blocks than
// the default grid (g <= 0).  Both loops cover every atom for any grid; many
// small systems in one batched launch want g > 1, so that each block's fixed
// latency (descriptor, engine record, partial sums) is paid for more atoms
// and a warp of C keeps several groups in flight instead of one group per
// block wave.  The virial partials are per block, so the shape fixes the
// order of the virial sum (results depend on it at rounding level only).
int a_blocks_shaped(int n, bool mixed, int g) {
    const int d = a_blocks(n, mixed);
    if (g <= 0) return d;
    const int b = grid_for(n, kBlockA * g);
    return b < d ? b : d;
}
int contact_blocks_shaped(int n, int style, bool mixed, int g) {
    const int d = contact_blocks(n, style, mixed);
    if (g <= 0) return d;
    const int b = grid_for(n, kBlockC * g);
    return b < d ? b : d;
}
// The scratch regions (lay_*): the first three depend on n alone, so A finds
// the flag words at the base and S finds the partials through
// tmps_engine.part_off.
size_t gap_offset(int n) { return lay_gap(n); }
size_t atom_gap_offset(int n) { return lay_agap(n); }
size_t part_offset(int n) { return lay_part(n); }
// The mixed form's histories between their two storages: doubles (the FP64
// form, the per-hook kernels, the rebuild carry-over, restart) and FP32
// double words (the mixed contact pass).  Only the entries of touching slots
// hold a history; to_dw 1: double -> (hi, lo), 0: (hi, lo) -> double, exact
// both ways for values of at most 48 significant bits.
__global__ void __launch_bounds__(256) k_history_form(tmps_nlist L, int to_dw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = L.n;
    if (i >= n) return;
    const uint64_t t = L.touch[i];
    if (!t) return;
    const size_t ss = (size_t)L.slots * n;
    for (uint64_t w = t; w; w &= w - 1) {
        const int k = __ffsll((long long)w) - 1;
        if (k >= L.slots) break;
        for (int arr = 0; arr < 2; ++arr) {
            double* h = arr == 0 ? L.shear : L.rolling;
            if (!h) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                double* p = h + (size_t)c * ss + (size_t)k * n + i;
                if (to_dw) {
                    const double v = *p;
                    const float hi = __double2float_rn(v);
                    const float lo = __double2float_rn(v - (double)hi);
                    *reinterpret_cast<DW*>(p) = DW{hi, lo};
                } else {
                    const DW v = *reinterpret_cast<const DW*>(p);
                    *p = (double)v.hi + (double)v.lo;
                }
            }
        }
    }
}

}  // namespace

extern "C" {

int tmps_mixed_history(const tmps_nlist* nl, int32_t to_dw, void* stream) {
    if (!nl || nl->n < 0 || nl->slots < 1 || nl->slots > kMaxSlots) return TMPS_ERR_BAD_ARG;
    if (nl->n == 0 || !nl->touch || !nl->shear) return TMPS_OK;
    k_history_form<<<grid_for(nl->n, 256), 256, 0, (cudaStream_t)stream>>>(*nl, to_dw ? 1 : 0);
    note_launches(1);
    return cudaPeekAtLastError() == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}

int32_t tmps_fused_blocks(int32_t n, int32_t style, int32_t mixed) {
    return a_blocks(n, mixed != 0) + contact_blocks(n, style, mixed != 0);
}

int64_t tmps_fused_scratch_bytes(int32_t n, int32_t style, int32_t mixed) {
    if (n < 0) return -1;
    return (int64_t)(part_offset(n) +
                     (size_t)(a_blocks(n, mixed != 0) + contact_blocks(n, style, mixed != 0)) * 6 * sizeof(double));
}

int tmps_fused_prepare(const tmps_atoms* a, const tmps_box* d_box, tmps_engine* d_eng, const int32_t* cell_of,
                       void* stream) {
    if (!a || !d_box || !d_eng || !cell_of || a->n < 0) return TMPS_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    k_prepare_engine<<<1, 32, 0, s>>>(d_box, d_eng, (int64_t)part_offset(a->n));
    note_launches(1);
    if (a->n > 0) {
        k_prepare<<<grid_for(a->n, kBlockA), kBlockA, 0, s>>>(*a, d_box, d_eng, cell_of);
        note_launches(1);
    }
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_mixed_unpack(const tmps_atoms* a, const tmps_box* d_box, void* stream) {
    if (!a || !d_box || a->n < 0 || !mixed_ok(a)) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_unpack<<<grid_for(a->n, kBlockA), kBlockA, 0, (cudaStream_t)stream>>>(*a, d_box);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_fused_a(const tmps_atoms* a, tmps_box* d_box, tmps_engine* d_eng, int32_t a_blocks_, void* scratch,
                 void* stream) {
    if (!a || !d_box || !d_eng || !scratch || a->n < 0) return TMPS_ERR_BAD_ARG;
    if (!a->pos32 && (!a->rinv || !a->x0)) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    const int n = a->n;
    const bool mixed = a->pos32 != nullptr;
    const int gdef = a_blocks(n, mixed);
    if (a_blocks_ > gdef) return TMPS_ERR_BAD_ARG;  // the scratch holds the default grid's partials
    const int g = a_blocks_ > 0 ? a_blocks_ : gdef;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t* flags = (const uint32_t*)scratch;
    double* part = (double*)((char*)scratch + part_offset(n));  // A's partials come first
    if (mixed) {
        if (!mixed_ok(a)) return TMPS_ERR_BAD_ARG;
        launch_pdl(k_a32, g, kBlockA, s, *a, (const tmps_box*)d_box, d_eng, flags, part);
    } else {
        launch_pdl(k_a64, g, kBlockA, s, *a, (const tmps_box*)d_box, d_eng, flags, part);
    }
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_fused_c(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box, tmps_engine* d_eng,
                 const tmps_pair_params* p, int32_t c_blocks, void* scratch, int32_t rows, void* stream) {
    if (!a || !nl || !d_box || !d_eng || !p || !scratch || a->n < 0 || nl->n != a->n) return TMPS_ERR_BAD_ARG;
    if (!a->pos32 && !a->rinv) return TMPS_ERR_BAD_ARG;
    if (p->style < 0 || p->style > 4 || nl->slots < 1 || nl->slots > kMaxSlots) return TMPS_ERR_BAD_ARG;
    if (p->style == 4 && p->rolling_id != 0 && !nl->rolling) return TMPS_ERR_BAD_ARG;
    const int n = a->n;
    const bool mixed = a->pos32 != nullptr;
    const int g2def = contact_blocks(n, p->style, mixed);
    if (c_blocks > g2def) return TMPS_ERR_BAD_ARG;  // the scratch holds the default grid's partials
    const int g2 = c_blocks > 0 ? c_blocks : g2def;
    uint32_t* flags = (uint32_t*)scratch;
    const float* gap = (const float*)((char*)scratch + gap_offset(n));
    const float* agap = (const float*)((char*)scratch + atom_gap_offset(n));
    // partials are component-major, [6][nblocks]; C's blocks follow A's
    double* part2 = (double*)((char*)scratch + part_offset(n));
    cudaStream_t s = (cudaStream_t)stream;
    if (mixed && !mixed_ok(a)) return TMPS_ERR_BAD_ARG;
#define TMPS_LAUNCH_C(ST)                                                                                          \
    if (mixed && rows) launch_pdl(k_cf<ST, true, true>, g2, kBlockC, s, *a, *nl, *p, d_box, d_eng, flags, gap, agap, \
                                  part2);                                                                        \
    else if (mixed) launch_pdl(k_cf<ST, true>, g2, kBlockC, s, *a, *nl, *p, d_box, d_eng, flags, gap, agap, part2); \
    else if (rows) launch_pdl(k_cf<ST, false, true>, g2, kBlockC, s, *a, *nl, *p, d_box, d_eng, flags, gap, agap,   \
                              part2);                                                                            \
    else launch_pdl(k_cf<ST, false>, g2, kBlockC, s, *a, *nl, *p, d_box, d_eng, flags, gap, agap, part2);
    switch (p->style) {
        case 0: TMPS_LAUNCH_C(0) break;
        case 1: TMPS_LAUNCH_C(1) break;
        case 2: TMPS_LAUNCH_C(2) break;
        case 3: TMPS_LAUNCH_C(3) break;
        default: TMPS_LAUNCH_C(4) break;
    }
#undef TMPS_LAUNCH_C
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_fused_servo(tmps_box* d_box, tmps_servo* d_servo, tmps_engine* d_eng, const void* scratch,
                     int32_t* d_status, void* stream) {
    if (!d_box || !d_servo || !d_eng || !scratch || !d_status) return TMPS_ERR_BAD_ARG;
    launch_pdl(k_s, 1, kBlockS, (cudaStream_t)stream, d_box, d_servo, d_eng, (const char*)scratch, d_status);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_fused_bounds(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box, tmps_engine* d_eng,
                      const tmps_pair_params* p, int32_t cull, void* scratch, void* stream) {
    if (!a || !nl || !d_box || !d_eng || !p || !scratch || a->n < 0 || nl->n != a->n || !a->x0 || !a->xr)
        return TMPS_ERR_BAD_ARG;
    if (nl->slots < 1 || nl->slots > kMaxSlots) return TMPS_ERR_BAD_ARG;
    const int n = a->n;
    const bool has_hist = p->style == 1 || p->style == 3 ||
                          (p->style == 4 && (p->tangential_id >= 2 || p->rolling_id != 0));
    uint32_t* flags = (uint32_t*)scratch;
    float* gap = (float*)((char*)scratch + gap_offset(n));
    float* agap = (float*)((char*)scratch + atom_gap_offset(n));
    const int g = n > 0 ? grid_for(n, kBlockA) : 1;
    cudaStream_t st = (cudaStream_t)stream;
    k_bounds<<<g, kBlockA, 0, st>>>(*a, *nl, d_box, d_eng, has_hist ? 1 : 0, cull ? 1 : 0, flags, gap, agap);
    note_launches(1);
    if (cull && n > 0) {
        // the groups in ascending gap order (C's ordered pass)
        const int ng = lay_groups(n), npad = lay_npad(n);
        uint64_t* keys = (uint64_t*)((char*)scratch + lay_keys(n));
        const int bt = npad < 256 ? npad : 256;
        k_gap_keys<<<grid_for(npad, bt), bt, 0, st>>>(gap, ng, npad, keys);
        const int chunk = npad < kSortChunk ? npad : kSortChunk;
        k_bitonic_shared<<<npad / chunk, chunk / 2, 0, st>>>(keys, chunk, 2, chunk, 1);
        int launches = 2;
        for (int k = 2 * chunk; k <= npad; k <<= 1) {
            for (int j = k >> 1; j >= chunk; j >>= 1) {
                k_bitonic_global<<<grid_for(npad, bt), bt, 0, st>>>(keys, npad, j, k);
                ++launches;
            }
            k_bitonic_shared<<<npad / chunk, chunk / 2, 0, st>>>(keys, chunk, k, k, chunk / 2);
            ++launches;
        }
        k_gap_order<<<grid_for(ng, 256), 256, 0, st>>>(keys, gap, ng, (int32_t*)((char*)scratch + lay_order(n)),
                                                       (float*)((char*)scratch + lay_sgap(n)));
        note_launches(launches + 1);
    }
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_fused_pressure_log(tmps_engine* d_eng, double* h_log, int32_t len, void* stream) {
    if (!d_eng || (h_log && len < 1)) return TMPS_ERR_BAD_ARG;
    double* dptr = nullptr;
    if (h_log) {
        // only page-locked host memory the device can address
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, h_log) != cudaSuccess || at.type != cudaMemoryTypeHost ||
            at.devicePointer == nullptr) {
            (void)cudaGetLastError();
            return TMPS_ERR_BAD_ARG;
        }
        dptr = (double*)at.devicePointer;
    }
    k_set_log<<<1, 1, 0, (cudaStream_t)stream>>>(d_eng, dptr, len);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_batch_blocks(int32_t n, int32_t style, int32_t mixed, int32_t* a_b, int32_t* c_b) {
    return tmps_fused_shape(n, style, mixed, 0, 0, a_b, c_b);
}

int tmps_fused_shape(int32_t n, int32_t style, int32_t mixed, int32_t a_groups_per_warp, int32_t c_groups_per_warp,
                     int32_t* a_b, int32_t* c_b) {
    if (n < 0 || style < 0 || style > 4 || !a_b || !c_b) return TMPS_ERR_BAD_ARG;
    *a_b = n > 0 ? a_blocks_shaped(n, mixed != 0, a_groups_per_warp) : 0;
    *c_b = n > 0 ? contact_blocks_shaped(n, style, mixed != 0, c_groups_per_warp) : 0;
    return TMPS_OK;
}

int tmps_batch_a(const tmps_instance* d_inst, const int32_t* d_block_inst, int32_t nblocks, int32_t mixed,
                 void* stream) {
    if (!d_inst || !d_block_inst || nblocks < 0) return TMPS_ERR_BAD_ARG;
    if (nblocks == 0) return TMPS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (mixed) launch_pdl(kb_a32, nblocks, kBlockA, s, d_inst, d_block_inst);
    else launch_pdl(kb_a64, nblocks, kBlockA, s, d_inst, d_block_inst);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_batch_c(const tmps_instance* d_inst, const int32_t* d_block_inst, int32_t nblocks, int32_t style,
                 int32_t mixed, void* stream) {
    if (!d_inst || !d_block_inst || nblocks < 0 || style < 0 || style > 4) return TMPS_ERR_BAD_ARG;
    if (nblocks == 0) return TMPS_OK;
    cudaStream_t s = (cudaStream_t)stream;
#define TMPS_LAUNCH_BC(ST)                                                         \
    if (mixed) launch_pdl(kb_cf<ST, true>, nblocks, kBlockC, s, d_inst, d_block_inst); \
    else launch_pdl(kb_cf<ST, false>, nblocks, kBlockC, s, d_inst, d_block_inst);
    switch (style) {
        case 0: TMPS_LAUNCH_BC(0) break;
        case 1: TMPS_LAUNCH_BC(1) break;
        case 2: TMPS_LAUNCH_BC(2) break;
        case 3: TMPS_LAUNCH_BC(3) break;
        default: TMPS_LAUNCH_BC(4) break;
    }
#undef TMPS_LAUNCH_BC
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_batch_servo(const tmps_instance* d_inst, int32_t ninst, int32_t* d_status, void* stream) {
    if (!d_inst || ninst < 0 || !d_status) return TMPS_ERR_BAD_ARG;
    if (ninst == 0) return TMPS_OK;
    launch_pdl(kb_s, ninst, kBlockSB, (cudaStream_t)stream, d_inst, d_status);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_batch_state(const tmps_instance* d_inst, int32_t ninst, int64_t* d_state, void* stream) {
    if (!d_inst || ninst < 0 || !d_state) return TMPS_ERR_BAD_ARG;
    if (ninst == 0) return TMPS_OK;
    kb_state<<<grid_for(ninst, 128), 128, 0, (cudaStream_t)stream>>>(d_inst, ninst, d_state);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_fused_settle(const tmps_atoms* a, tmps_box* d_box, tmps_engine* d_eng, void* stream) {
    if (!a || !d_box || !d_eng || a->n < 0 || (!a->pos32 && !a->rinv)) return TMPS_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (a->n > 0) {
        if (a->pos32) k_settle<true><<<grid_for(a->n, kBlockA), kBlockA, 0, s>>>(*a, d_box, d_eng);
        else k_settle<false><<<grid_for(a->n, kBlockA), kBlockA, 0, s>>>(*a, d_box, d_eng);
        note_launches(1);
    }
    k_settle_flags<<<1, 1, 0, s>>>(d_box, d_eng);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

}  // extern "C"
