// Per-atom streaming kernels of the DEM step (FP64 form): velocity Verlet,
// Cundall damping, force clearing, skin check, periodic wrap, the virial
// reduction, the pressure servo and the affine remap.
//
// Each kernel restates one reference loop; the arithmetic order of every
// expression is kept so results agree with the reference to rounding.
#include <atomic>
#include <cstdio>

#include "tmps_common.cuh"
#include "tmps_servo.cuh"

using namespace tmps;

namespace {

constexpr int kBlock = 256;

// ---------------------------------------------------------------- Verlet

// FixNVESphere.initial_integrate_kernel (nve_sphere.py:44-77):
//   v += dtf * (f / m);  x = x + dtv * v;  omega += dtf * (torque / I)
__global__ void __launch_bounds__(kBlock) k_verlet_initial(tmps_atoms a, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int n = a.n;
    const double dtv = dt, dtf = 0.5 * dt;
    double4 x = ld4(a.xr, i), v = ld4(a.vm, i), w = ld4(a.om, i);
    const double m = v.w, inertia = w.w;
    v.x += dtf * (a.f[i] / m);
    v.y += dtf * (a.f[n + i] / m);
    v.z += dtf * (a.f[2 * n + i] / m);
    x.x = x.x + dtv * v.x;
    x.y = x.y + dtv * v.y;
    x.z = x.z + dtv * v.z;
    w.x += dtf * (a.torque[i] / inertia);
    w.y += dtf * (a.torque[n + i] / inertia);
    w.z += dtf * (a.torque[2 * n + i] / inertia);
    st4(a.xr, i, x);
    st4(a.vm, i, v);
    st4(a.om, i, w);
}

// FixNVESphere.final_integrate_kernel (nve_sphere.py:79-96)
__global__ void __launch_bounds__(kBlock) k_verlet_final(tmps_atoms a, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int n = a.n;
    const double dtf = 0.5 * dt;
    double4 v = ld4(a.vm, i), w = ld4(a.om, i);
    const double m = v.w, inertia = w.w;
    v.x += dtf * (a.f[i] / m);
    v.y += dtf * (a.f[n + i] / m);
    v.z += dtf * (a.f[2 * n + i] / m);
    w.x += dtf * (a.torque[i] / inertia);
    w.y += dtf * (a.torque[n + i] / inertia);
    w.z += dtf * (a.torque[2 * n + i] / inertia);
    st4(a.vm, i, v);
    st4(a.om, i, w);
}

// a * b >= 0.0, as the FP64 product compares: from the sign bits where the
// exponents keep the product clear of underflow (and neither is a NaN), the
// product itself otherwise.
__device__ __forceinline__ bool prod_nonneg(double a, double b) {
    const int ha = __double2hiint(a), hb = __double2hiint(b);
    const int ea = (ha >> 20) & 0x7ff, eb = (hb >> 20) & 0x7ff;
    if (ea > 0x200 && ea < 0x600 && eb > 0x200 && eb < 0x600) return (ha ^ hb) >= 0;
    return a * b >= 0.0;
}

// FixDampingCundall.post_force (damping_cundall.py:36-53):
//   f_d *= 1 - gamma_lin sign(f_d v_d),  torque_d *= 1 - gamma_ang sign(torque_d omega_d)
// The factors 1 -+ gamma are the same two roundings for every atom (gamma *
// sign is exact), so they are formed once; each component then costs one
// FP64 multiply.
__global__ void __launch_bounds__(kBlock) k_cundall(tmps_atoms a, double gl, double ga) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int n = a.n;
    const double lp = 1.0 - gl, lm = 1.0 + gl, ap = 1.0 - ga, am = 1.0 + ga;
    const double4 v = ld4(a.vm, i), w = ld4(a.om, i);
    const double vv[3] = {v.x, v.y, v.z}, ww[3] = {w.x, w.y, w.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double fd = a.f[d * n + i];
        a.f[d * n + i] = __dmul_rn(fd, prod_nonneg(fd, vv[d]) ? lp : lm);
        const double td = a.torque[d * n + i];
        a.torque[d * n + i] = __dmul_rn(td, prod_nonneg(td, ww[d]) ? ap : am);
    }
}

// NeighborList.check_displacement (neighbor.py:242-245): stamp the flag when
// |x - x0|^2 > trigger.  Exact FP64 (no contraction) so the decision matches
// the reference for the same positions.  A non-finite displacement stamps it
// too (the reference's test lets a NaN through): the rebuild that follows
// bins the atom and reports TMPS_STATUS_NONFINITE.
__global__ void __launch_bounds__(kBlock) k_skin_check(tmps_atoms a, double trig, int32_t stamp,
                                                        int32_t* flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool hit = false;
    if (i < a.n) {
        const int n = a.n;
        double4 x = ld4(a.xr, i);
        double d0 = __dsub_rn(x.x, a.x0[i]);
        double d1 = __dsub_rn(x.y, a.x0[n + i]);
        double d2 = __dsub_rn(x.z, a.x0[2 * n + i]);
        double s = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
        hit = !(s <= trig);
    }
    // one store per warp that saw a crossing; nothing at all in the common case
    if (__any_sync(0xffffffffu, hit) && (threadIdx.x & 31) == 0) *flag = stamp;
}

// Domain._pbc_kernel / _pbc_vremap_kernel (domain.py:560-571), orthogonal.
__global__ void __launch_bounds__(kBlock) k_pbc(tmps_atoms a, const tmps_box* __restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double4 x = ld4(a.xr, i);
    double xx[3] = {x.x, x.y, x.z};
    if (b->vremap) {
        double c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            c[k] = b->per[k] == 1 ? floor(__ddiv_rn(__dsub_rn(xx[k], b->lo[k]), b->prd[k])) : 0.0;
        if (c[0] != 0.0 || c[1] != 0.0 || c[2] != 0.0) {
            const double* h = b->h_rate;
            double4 v = ld4(a.vm, i);
            v.x += -__dadd_rn(__dadd_rn(__dmul_rn(c[0], h[0]), __dmul_rn(c[1], h[5])), __dmul_rn(c[2], h[4]));
            v.y += -__dadd_rn(__dmul_rn(c[1], h[1]), __dmul_rn(c[2], h[3]));
            v.z += -__dmul_rn(c[2], h[2]);
            st4(a.vm, i, v);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (b->per[k] == 1) {
            double s = __ddiv_rn(__dsub_rn(xx[k], b->lo[k]), b->prd[k]);
            xx[k] = __dadd_rn(b->lo[k], __dmul_rn(__dsub_rn(s, floor(s)), b->prd[k]));
        }
    }
    x.x = xx[0]; x.y = xx[1]; x.z = xx[2];
    st4(a.xr, i, x);
}

// ----------------------------------------------------------- virial

// Computes.compute_virial_kernel (thermo.py:89-109): per-atom virial plus,
// with keflag, m v_a v_b.  Two passes with a grid of fixed width, so the
// summation order depends only on n: deterministic run to run.
constexpr int kVirBlocks = 512;

__global__ void __launch_bounds__(kBlock) k_virial_partial(tmps_atoms a, int keflag, double* part) {
    __shared__ double smem[6 * (kBlock / 32)];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (a.virial) {
#pragma unroll
            for (int k = 0; k < 6; ++k) acc[k] += a.virial[k * n + i];
        }
        if (keflag) {
            double4 v = ld4(a.vm, i);
            double m = v.w;
            acc[0] += (m * v.x) * v.x;
            acc[1] += (m * v.y) * v.y;
            acc[2] += (m * v.z) * v.z;
            acc[3] += (m * v.x) * v.y;
            acc[4] += (m * v.x) * v.z;
            acc[5] += (m * v.y) * v.z;
        }
    }
    block_sum<6, kBlock>(acc, smem);
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) part[blockIdx.x * 6 + k] = acc[k];
}

__global__ void k_virial_final(const double* part, int nparts, double* out) {
    __shared__ double smem[6 * (kBlock / 32)];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < nparts; p += blockDim.x)
        for (int k = 0; k < 6; ++k) acc[k] += part[p * 6 + k];
    block_sum<6, kBlock>(acc, smem);
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) out[k] = acc[k];
}

// ------------------------------------------------------------ servo

// FixDeformPressure._limit_rate (deform_pressure.py:737-752)
__device__ double limit_rate(double rate, double ptarget, int normalize, double max_rate) {
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

// One deformation update on the device: FixDeformPressure._servo_kernel
// (deform_pressure.py:598-702) for x/y/z, covering the strain styles of
// _apply_strain (:770-805) and the pressure styles of _apply_pressure
// (:833-847).  Serial: three axes.
__global__ void k_servo(tmps_box* b, tmps_servo* s, const double* vir, double elapsed, double frac,
                        double dt, int32_t* status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double lo[3], hi[3], prd[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = b->lo[d];
        hi[d] = b->hi[d];
        prd[d] = b->prd[d];
    }
    const double vol = prd[0] * prd[1] * prd[2];
    double t[6];
    for (int k = 0; k < 6; ++k) t[k] = vol > 0.0 ? vir[k] / vol : 0.0;
    for (int k = 0; k < 6; ++k) s->pressure[k] = t[k];
    const double scalar = ((t[0] + t[1]) + t[2]) / 3.0;
    double p[3] = {t[0], t[1], t[2]};
    if (s->couple == 1) {
        p[0] = p[1] = p[2] = scalar;
    } else if (s->couple == 2) {
        double m = (t[0] + t[1]) / 2.0;
        p[0] = m; p[1] = m;
    } else if (s->couple == 3) {
        double m = (t[1] + t[2]) / 2.0;
        p[1] = m; p[2] = m;
    } else if (s->couple == 4) {
        double m = (t[0] + t[2]) / 2.0;
        p[0] = m; p[2] = m;
    }
    double nlo[3], nhi[3];
    for (int d = 0; d < 3; ++d) {
        const int st = s->style[d];
        const double ls = s->lo_start[d], hs = s->hi_start[d];
        nlo[d] = lo[d];
        nhi[d] = hi[d];
        if (st == 1) {  // erate
            double shift = ((0.5 * elapsed) * s->rate[d]) * (hs - ls);
            nlo[d] = ls - shift; nhi[d] = hs + shift;
        } else if (st == 2) {  // trate
            double mid = 0.5 * (ls + hs);
            double half = (0.5 * (hs - ls)) * exp(s->rate[d] * elapsed);
            nlo[d] = mid - half; nhi[d] = mid + half;
        } else if (st == 3) {  // vel
            double shift = (0.5 * elapsed) * s->vel[d];
            nlo[d] = ls - shift; nhi[d] = hs + shift;
        } else if (st == 4) {  // wiggle
            double shift = (0.5 * s->amp[d]) * sin(((2.0 * 3.14159265358979323846) * elapsed) / s->tper[d]);
            nlo[d] = ls - shift; nhi[d] = hs + shift;
        } else if (st == 5) {  // final
            nlo[d] = ls + frac * (s->flo[d] - ls);
            nhi[d] = hs + frac * (s->fhi[d] - hs);
        } else if (st == 6) {  // delta
            double lo_stop = ls + s->dlo[d], hi_stop = hs + s->dhi[d];
            nlo[d] = ls + frac * (lo_stop - ls);
            nhi[d] = hs + frac * (hi_stop - hs);
        } else if (st == 7) {  // scale
            double mid = 0.5 * (ls + hs);
            double half = (0.5 * s->scale[d]) * (hs - ls);
            nlo[d] = ls + frac * ((mid - half) - ls);
            nhi[d] = hs + frac * ((mid + half) - hs);
        } else if (st == 8 || st == 9) {  // pressure, pressure/mean
            // _current_pressure (deform_pressure.py:717-731): with a couple
            // the coupled mean (or the raw component) wins over pressure/mean
            double pd = (s->couple == 0 && st == 9) ? scalar : p[d];
            double tgt = s->ptarget[d];
            double rate = limit_rate(s->pgain[d] * (pd - tgt), tgt, s->normalize, s->max_rate);
            s->cum[d] += (dt * rate) * prd[d];
            nlo[d] = ls - 0.5 * s->cum[d];
            nhi[d] = hs + 0.5 * s->cum[d];
        }
    }
    // volume and box styles (cross-axis, after the per-axis targets)
    if (s->post) servo_post(*s, prd, t, dt, nlo, nhi);
    double nprd[3];
    bool bad = false;
    for (int d = 0; d < 3; ++d) {
        nprd[d] = nhi[d] - nlo[d];
        bad = bad || !(nprd[d] > 0.0);
    }
    if (bad) {
        *status |= TMPS_STATUS_BOX_NONPOSITIVE;
        return;  // keep the old box; the host raises
    }
    for (int d = 0; d < 3; ++d) {
        b->old_lo[d] = lo[d];
        b->old_prd[d] = prd[d];
        b->lo[d] = nlo[d];
        b->hi[d] = nhi[d];
        b->prd[d] = nprd[d];
        b->inv_prd[d] = 1.0 / nprd[d];
        b->hcell[d] = nprd[d] / (double)b->g[d];
        b->h_rate[d] = (nprd[d] - prd[d]) / dt;
        b->h_rate[3 + d] = 0.0;
    }
    b->vremap = s->remap == 2 ? 1 : 0;
    b->remap_pending = s->remap == 1 ? 1 : 0;
}

// FixDeformPressure.remap_positions (deform_pressure.py:512-530), orthogonal:
// lamda with the old box, back with the new one, anchored on the new lo.
__global__ void __launch_bounds__(kBlock) k_remap_x(tmps_atoms a, const tmps_box* __restrict__ b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !b->remap_pending) return;
    double4 x = ld4(a.xr, i);
    double xx[3] = {x.x, x.y, x.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double d = __dsub_rn(xx[k], b->old_lo[k]);
        double lam = __ddiv_rn(d, b->old_prd[k]);
        xx[k] = __dadd_rn(__dmul_rn(b->prd[k], lam), b->lo[k]);
    }
    x.x = xx[0]; x.y = xx[1]; x.z = xx[2];
    st4(a.xr, i, x);
}

__global__ void k_clear_remap_pending(tmps_box* b) { b->remap_pending = 0; }

bool launch_ok() { return cudaPeekAtLastError() == cudaSuccess; }

}  // namespace

namespace tmps {
static std::atomic<long long> g_launches{0};
void note_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
}  // namespace tmps

// =================================================================== C ABI

extern "C" {

const char* tmps_version(void) { return "taichimps_gb300 0.1 (sm_103a)"; }

long long tmps_launch_count(void) { return tmps::g_launches.load(std::memory_order_relaxed); }

const char* tmps_last_cuda_error(void) {
    static thread_local char buf[256];
    const cudaError_t e = cudaPeekAtLastError();
    snprintf(buf, sizeof(buf), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return buf;
}

int tmps_box_set(tmps_box* d_box, const tmps_box* h_box, void* stream) {
    if (!d_box || !h_box) return TMPS_ERR_BAD_ARG;
    cudaError_t e = cudaMemcpyAsync(d_box, h_box, sizeof(tmps_box), cudaMemcpyHostToDevice,
                                    (cudaStream_t)stream);
    return e == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_verlet_initial(const tmps_atoms* a, double dt, void* stream) {
    if (!a || a->n < 0) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_verlet_initial<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, dt);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_verlet_final(const tmps_atoms* a, double dt, void* stream) {
    if (!a || a->n < 0) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_verlet_final<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, dt);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_clear_forces(const tmps_atoms* a, void* stream) {
    if (!a || a->n < 0) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    size_t n = (size_t)a->n;
    cudaError_t e = cudaMemsetAsync(a->f, 0, 3 * n * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->torque, 0, 3 * n * sizeof(double), s);
    if (e == cudaSuccess && a->virial) e = cudaMemsetAsync(a->virial, 0, 6 * n * sizeof(double), s);
    return e == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_damping_cundall(const tmps_atoms* a, double gamma_lin, double gamma_ang, void* stream) {
    if (!a || a->n < 0) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_cundall<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, gamma_lin, gamma_ang);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_skin_check(const tmps_atoms* a, double trigger_sq, int32_t stamp, int32_t* d_flag,
                    void* stream) {
    if (!a || a->n < 0 || !d_flag || !a->x0) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_skin_check<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, trigger_sq, stamp,
                                                                              d_flag);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_pbc(const tmps_atoms* a, const tmps_box* d_box, void* stream) {
    if (!a || a->n < 0 || !d_box) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_pbc<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, d_box);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int64_t tmps_virial_workspace_bytes(int32_t n) {
    (void)n;
    return (int64_t)kVirBlocks * 6 * sizeof(double);
}

int tmps_virial_reduce(const tmps_atoms* a, int32_t keflag, double* d_out, void* workspace,
                       int64_t workspace_bytes, void* stream) {
    if (!a || a->n < 0 || !d_out || !workspace) return TMPS_ERR_BAD_ARG;
    if (workspace_bytes < tmps_virial_workspace_bytes(a->n)) return TMPS_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int blocks = grid_for(a->n, kBlock);
    if (blocks > kVirBlocks) blocks = kVirBlocks;
    double* part = (double*)workspace;
    k_virial_partial<<<blocks, kBlock, 0, s>>>(*a, keflag, part);
    k_virial_final<<<1, kBlock, 0, s>>>(part, blocks, d_out);
    note_launches(2);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_servo_step(tmps_box* d_box, tmps_servo* d_servo, const double* d_virial, double elapsed,
                    double frac, double dt, int32_t* d_status, void* stream) {
    if (!d_box || !d_servo || !d_virial || !d_status || !(dt > 0.0)) return TMPS_ERR_BAD_ARG;
    k_servo<<<1, 32, 0, (cudaStream_t)stream>>>(d_box, d_servo, d_virial, elapsed, frac, dt, d_status);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_remap_x(const tmps_atoms* a, tmps_box* d_box, void* stream) {
    if (!a || a->n < 0 || !d_box) return TMPS_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (a->n > 0) {
        k_remap_x<<<grid_for(a->n, kBlock), kBlock, 0, s>>>(*a, d_box);
        note_launches(1);
    }
    k_clear_remap_pending<<<1, 1, 0, s>>>(d_box);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

}  // extern "C"
