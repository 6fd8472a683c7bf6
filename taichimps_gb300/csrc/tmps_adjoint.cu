// Differentiable run: forward steps that record a tape, and the hand-written
// reverse of each step (contact law, both half-kicks of nve/sphere, pressure,
// servo and remap x).  FP64 throughout; atoms in the caller's order; the
// contacts are a half pair list (i < j) sorted by (i, j), and every per-atom
// sum gathers over the pairs in a fixed order (pairs as i, then as j), so
// results are bit-reproducible and the reverse sees exactly the forward's
// values.
//
// Forward of step s (Simulation._sub_step_inner, simulation.py:205-247):
//   k_initial   v += dtf f / m; x += dt v; w += dtf t / I     (nve_sphere.py:56-80)
//   k_pairs     contacts on the tape's xh, vh, wh (hertz_history.py:92-157)
//   k_gather    f, t per atom; v += dtf f / m; w += dtf t / I; kinetic partials
//   k_servo     virial total, pressure, servo, new box        (deform_pressure.py:598-702)
//   k_remap     x from the old box into the new one           (deform_pressure.py:493-530)
// Reverse of step s runs these backwards: k_b_remap, k_b_servo, k_b_final,
// k_b_pairs, k_b_reduce, k_b_gather, k_b_initial.
#include "tmps_adjoint.cuh"
#include "tmps_common.cuh"

using namespace tmps;
using namespace tmps_adj;

namespace {

constexpr int kBlk = 256;
constexpr int kNG = 16;  // doubles per pair in the reverse's per-pair record

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct Work {
    double* fp;     // [3][P] pair force on a
    double* tp;     // [3][P] pair torque term (d x fs) / r
    double* gp;     // [16][P] per-pair adjoints for the gather
    double* partw;  // [6][nbP] pair virial partials
    double* partk;  // [6][nbA] kinetic / remap partials
    double* partg;  // [8][nbP] parameter and image partials of the reverse
    double* wbar;   // [6] dL/d(virial total) of the current reverse step
};

Work carve(void* base, int n, int npairs) {
    const int nbA = grid_for(n, kBlk), nbP = grid_for(npairs, kBlk);
    char* p = static_cast<char*>(base);
    Work w;
    w.fp = reinterpret_cast<double*>(p); p += align256(sizeof(double) * 3 * (size_t)npairs);
    w.tp = reinterpret_cast<double*>(p); p += align256(sizeof(double) * 3 * (size_t)npairs);
    w.gp = reinterpret_cast<double*>(p); p += align256(sizeof(double) * kNG * (size_t)npairs);
    w.partw = reinterpret_cast<double*>(p); p += align256(sizeof(double) * 6 * (size_t)nbP);
    w.partk = reinterpret_cast<double*>(p); p += align256(sizeof(double) * 6 * (size_t)nbA);
    w.partg = reinterpret_cast<double*>(p); p += align256(sizeof(double) * 8 * (size_t)nbP);
    w.wbar = reinterpret_cast<double*>(p);
    return w;
}

size_t work_bytes(int n, int npairs) {
    const int nbA = grid_for(n, kBlk), nbP = grid_for(npairs, kBlk);
    return align256(sizeof(double) * 3 * (size_t)npairs) * 2 + align256(sizeof(double) * kNG * (size_t)npairs) +
           align256(sizeof(double) * 6 * (size_t)nbP) + align256(sizeof(double) * 6 * (size_t)nbA) +
           align256(sizeof(double) * 8 * (size_t)nbP) + align256(sizeof(double) * 8);
}

Params to_params(const tmps_adj_params& p) {
    Params q;
    q.kn = p.kn;
    q.kt = p.kt;
    q.gamman = p.gamman;
    q.gammat = p.gammat;
    q.xmu = p.xmu;
    q.dt = p.dt;
    q.limit_damping = p.limit_damping;
    return q;
}

// Minimum image on a fully periodic orthogonal box (domain.py:389-500 with
// round(d / prd) taken as rint(d * (1 / prd)); they differ only within an ulp
// of half a box, which no listed pair is).
__device__ __forceinline__ void min_image(const double* prd, const double* iprd, double* d, double* nimg) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        nimg[c] = rint(d[c] * iprd[c]);
        d[c] -= nimg[c] * prd[c];
    }
}

__device__ __forceinline__ double inertia(double m, double r) { return ((0.4 * m) * r) * r; }

// Sum over the blocks' partials [NV][nb] into out[NV]: warp c sums component
// c with lane-strided partial sums and a shuffle tree (fixed order).
template <int NV>
__device__ void sum_partials(const double* part, int nb, double* out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < NV) {
        double s = 0.0;
        for (int k = lane; k < nb; k += 32) s += part[(size_t)warp * nb + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) out[warp] = s;
    }
}

// ------------------------------------------------------------------ pairs

__global__ void __launch_bounds__(128) k_pairs_build(int n, const double* __restrict__ x, const double* __restrict__ rad,
                                                     const tmps_adj_rec* __restrict__ box, double skin,
                                                     int32_t* __restrict__ count, const int32_t* __restrict__ ibeg,
                                                     int32_t* __restrict__ pi, int32_t* __restrict__ pj) {
    // All pairs by tiles of 128 candidates in shared memory; an FP32 screen
    // with a wide margin, then the exact FP64 test (neighbor.py:348-356).
    __shared__ float4 tile[128];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double prd[3], iprd[3];
    float prd32[3], iprd32[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        prd[c] = box->prd[c];
        iprd[c] = 1.0 / prd[c];
        prd32[c] = (float)prd[c];
        iprd32[c] = (float)iprd[c];
    }
    const bool act = i < n;
    double xi[3] = {0, 0, 0}, ri = 0.0;
    if (act) {
        xi[0] = x[i];
        xi[1] = x[n + i];
        xi[2] = x[2 * n + i];
        ri = rad[i];
    }
    const float xi32[3] = {(float)xi[0], (float)xi[1], (float)xi[2]};
    int cnt = 0;
    int out = (act && pj) ? ibeg[i] : 0;
    const int j0 = blockIdx.x * blockDim.x;  // no candidate below the block's first atom can be above i
    for (int base = j0; base < n; base += 128) {
        __syncthreads();
        const int jl = base + threadIdx.x;
        if (jl < n) tile[threadIdx.x] = make_float4((float)x[jl], (float)x[n + jl], (float)x[2 * n + jl], (float)rad[jl]);
        __syncthreads();
        if (!act) continue;
        const int m = min(128, n - base);
        for (int k = 0; k < m; ++k) {
            const int j = base + k;
            if (j <= i) continue;
            const float4 q = tile[k];
            float d0 = xi32[0] - q.x, d1 = xi32[1] - q.y, d2 = xi32[2] - q.z;
            d0 -= prd32[0] * rintf(d0 * iprd32[0]);
            d1 -= prd32[1] * rintf(d1 * iprd32[1]);
            d2 -= prd32[2] * rintf(d2 * iprd32[2]);
            const float cut32 = ((float)ri + q.w + (float)skin) * 1.0001f + 1e-3f;
            if (d0 * d0 + d1 * d1 + d2 * d2 >= cut32 * cut32) continue;
            double d[3] = {xi[0] - x[j], xi[1] - x[n + j], xi[2] - x[2 * n + j]}, nimg[3];
            min_image(prd, iprd, d, nimg);
            const double rsq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
            const double cut = (ri + rad[j]) + skin;
            if (rsq < cut * cut) {
                if (pj) {
                    pi[out] = i;
                    pj[out] = j;
                    ++out;
                }
                ++cnt;
            }
        }
    }
    if (act && !pj) count[i] = cnt;
}

__global__ void k_pair_map(int nold, const int32_t* __restrict__ opi, const int32_t* __restrict__ opj,
                           const int32_t* __restrict__ nibeg, const int32_t* __restrict__ npj, int32_t* __restrict__ map) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nold) return;
    const int i = opi[p], j = opj[p];
    int lo = nibeg[i], hi = nibeg[i + 1] - 1, r = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int v = npj[mid];
        if (v == j) {
            r = mid;
            break;
        }
        if (v < j) lo = mid + 1;
        else hi = mid - 1;
    }
    map[p] = r;
}

__global__ void k_carry(int nold, int nnew, const int32_t* __restrict__ map, double* __restrict__ old_,
                        double* __restrict__ new_, int reverse) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nold) return;
    const int q = map[p];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (reverse) old_[(size_t)c * nold + p] = q >= 0 ? new_[(size_t)c * nnew + q] : 0.0;
        else if (q >= 0) new_[(size_t)c * nnew + q] = old_[(size_t)c * nold + p];
    }
}

// ---------------------------------------------------------------- forward

__global__ void __launch_bounds__(kBlk) k_initial(tmps_adj_sys S, double dt, tmps_adj_tape T,
                                                  const double* __restrict__ xbuild, unsigned long long* disp) {
    const int n = S.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dd = 0.0;
    if (i < n) {
        const double dtf = 0.5 * dt;
        const double m = S.mass[i], r = S.radius[i], I = inertia(m, r);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const size_t k = (size_t)c * n + i;
            const double v = S.v[k] + dtf * (S.f[k] / m);
            const double x = S.x[k] + dt * v;
            T.vh[k] = v;
            T.xh[k] = x;
            T.wh[k] = S.w[k] + dtf * (S.t[k] / I);
            const double e = x - xbuild[k];
            dd += e * e;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dd = fmax(dd, __shfl_down_sync(0xffffffffu, dd, o));
    // non-negative doubles order as their bit patterns
    if ((threadIdx.x & 31) == 0 && dd > 0.0) atomicMax(disp, (unsigned long long)__double_as_longlong(dd));
}

__device__ __forceinline__ void load_pair(const tmps_adj_sys& S, const double* xs, const double* vs, const double* ws,
                                          const double* prd, const double* iprd, int p, int i, int j, PairIn& in,
                                          double* nimg) {
    const int n = S.n;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        in.d[c] = xs[(size_t)c * n + i] - xs[(size_t)c * n + j];
        in.va[c] = vs[(size_t)c * n + i];
        in.vb[c] = vs[(size_t)c * n + j];
        in.wa[c] = ws[(size_t)c * n + i];
        in.wb[c] = ws[(size_t)c * n + j];
    }
    min_image(prd, iprd, in.d, nimg);
    in.ra = S.radius[i];
    in.rb = S.radius[j];
    in.ma = S.mass[i];
    in.mb = S.mass[j];
    (void)p;
}

// Contacts of one pass: pair forces and torque terms into the workspace,
// history updated in place (the entering history recorded), virial partials.
__global__ void __launch_bounds__(kBlk) k_pairs(tmps_adj_sys S, Params P, int shearupdate, const double* xs,
                                                const double* vs, const double* ws, const tmps_adj_rec* __restrict__ box,
                                                double* __restrict__ sh_rec, uint8_t* __restrict__ mask_rec, Work W) {
    __shared__ double smem[6 * (kBlk / 32)];
    const int np = S.npairs;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double vir[6] = {0, 0, 0, 0, 0, 0};
    if (p < np) {
        double prd[3], iprd[3], nimg[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            prd[c] = box->prd[c];
            iprd[c] = 1.0 / prd[c];
        }
        PairIn in;
        load_pair(S, xs, vs, ws, prd, iprd, p, S.pi[p], S.pj[p], in, nimg);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            in.sh[c] = S.shear[(size_t)c * np + p];
            sh_rec[(size_t)c * np + p] = in.sh[c];
        }
        PairOut o;
        PairTape t;
        int mask;
        pair_forward(P, shearupdate, in, -1, o, t, &mask);
        mask_rec[p] = (uint8_t)mask;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            S.shear[(size_t)c * np + p] = o.sh[c];
            W.fp[(size_t)c * np + p] = o.F[c];
            W.tp[(size_t)c * np + p] = o.tor[c];
        }
        vir[0] = in.d[0] * o.F[0];
        vir[1] = in.d[1] * o.F[1];
        vir[2] = in.d[2] * o.F[2];
        vir[3] = in.d[0] * o.F[1];
        vir[4] = in.d[0] * o.F[2];
        vir[5] = in.d[1] * o.F[2];
    }
    block_sum<6, kBlk>(vir, smem);
    if (threadIdx.x == 0) {
        const int nb = gridDim.x;
#pragma unroll
        for (int c = 0; c < 6; ++c) W.partw[(size_t)c * nb + blockIdx.x] = vir[c];
    }
}

// Per-atom force and torque from the pairs (as i: +F, then as j: -F; the
// torque term times -r either way), then the second half-kick (final = 1)
// and the kinetic partials m v v.
__global__ void __launch_bounds__(kBlk) k_gather(tmps_adj_sys S, double dt, int final_, const double* __restrict__ vh,
                                                 const double* __restrict__ wh, double* __restrict__ ft,
                                                 double* __restrict__ tt, Work W) {
    __shared__ double smem[6 * (kBlk / 32)];
    const int n = S.n, np = S.npairs;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double kin[6] = {0, 0, 0, 0, 0, 0};
    if (a < n) {
        double F[3] = {0, 0, 0}, Tq[3] = {0, 0, 0};
        const double ra = S.radius[a];
        for (int q = S.ibeg[a]; q < S.ibeg[a + 1]; ++q)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                F[c] += W.fp[(size_t)c * np + q];
                Tq[c] += -ra * W.tp[(size_t)c * np + q];
            }
        for (int k = S.jbeg[a]; k < S.jbeg[a + 1]; ++k) {
            const int q = S.jlist[k];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                F[c] -= W.fp[(size_t)c * np + q];
                Tq[c] += -ra * W.tp[(size_t)c * np + q];
            }
        }
        const double m = S.mass[a], I = inertia(m, ra), dtf = 0.5 * dt;
        double v[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const size_t k = (size_t)c * n + a;
            S.f[k] = F[c];
            S.t[k] = Tq[c];
            if (ft) {
                ft[k] = F[c];
                tt[k] = Tq[c];
            }
            if (final_) {
                v[c] = vh[k] + dtf * (F[c] / m);
                S.v[k] = v[c];
                S.w[k] = wh[k] + dtf * (Tq[c] / I);
            }
        }
        if (final_) {
            kin[0] = (m * v[0]) * v[0];
            kin[1] = (m * v[1]) * v[1];
            kin[2] = (m * v[2]) * v[2];
            kin[3] = (m * v[0]) * v[1];
            kin[4] = (m * v[0]) * v[2];
            kin[5] = (m * v[1]) * v[2];
        }
    }
    if (!final_) return;
    block_sum<6, kBlk>(kin, smem);
    if (threadIdx.x == 0) {
        const int nb = gridDim.x;
#pragma unroll
        for (int c = 0; c < 6; ++c) W.partk[(size_t)c * nb + blockIdx.x] = kin[c];
    }
}

// The servo rate of a pressure axis: gain, normalize/pressure, max/rate
// (_limit_rate_device, deform_pressure.py:583-596).  Sets *clamped when
// max/rate (or a zero target under normalize) fixed the value.
__device__ double servo_rate(const tmps_adj_servo& sv, int d, double pd, bool* clamped) {
    double out = sv.pgain[d] * (pd - sv.ptarget[d]);
    *clamped = false;
    if (sv.normalize == 1) {
        if (sv.ptarget[d] == 0.0) {
            if (out != 0.0) {
                out = sv.max_rate * (out > 0.0 ? 1.0 : -1.0);
                *clamped = true;
            }
        } else {
            out = out / fabs(sv.ptarget[d]);
        }
    }
    if (sv.max_rate != 0.0 && fabs(out) > sv.max_rate) {
        out = sv.max_rate * (out > 0.0 ? 1.0 : -1.0);
        *clamped = true;
    }
    return out;
}

__device__ void coupled(int couple, const double* P, double* p) {
    p[0] = P[0];
    p[1] = P[1];
    p[2] = P[2];
    if (couple == 1) {
        const double s = (P[0] + P[1] + P[2]) / 3.0;
        p[0] = p[1] = p[2] = s;
    } else if (couple == 2) {
        const double m = 0.5 * (P[0] + P[1]);
        p[0] = p[1] = m;
    } else if (couple == 3) {
        const double m = 0.5 * (P[1] + P[2]);
        p[1] = p[2] = m;
    } else if (couple == 4) {
        const double m = 0.5 * (P[0] + P[2]);
        p[0] = p[2] = m;
    }
}

// Virial total, pressure tensor, deviatoric stress, the servo's new box.
__global__ void __launch_bounds__(256) k_servo(tmps_adj_servo sv, double dt, int64_t step, const tmps_adj_rec* prev,
                                               tmps_adj_rec* next, int nbP, int nbA, Work W) {
    __shared__ double sw[6], sk[6];
    sum_partials<6>(W.partw, nbP, sw);
    sum_partials<6>(W.partk, nbA, sk);
    __syncthreads();
    if (threadIdx.x != 0) return;
    tmps_adj_rec r = *prev;
    const double vol = (r.prd[0] * r.prd[1]) * r.prd[2];
    double Pt[6];
    for (int c = 0; c < 6; ++c) {
        r.w[c] = sw[c] + sk[c];
        Pt[c] = r.w[c] / vol;
    }
    r.q = Pt[2] - 0.5 * (Pt[0] + Pt[1]);
    r.elapsed = (double)step * dt;
    double p[3];
    coupled(sv.couple, Pt, p);
    r.clamp = 0;
    for (int d = 0; d < 3; ++d) {
        const double lo_s = sv.lo_start[d], hi_s = sv.hi_start[d];
        double lo, hi;
        if (sv.style[d] == 1) {
            const double shift = ((0.5 * r.elapsed) * sv.rate[d]) * (hi_s - lo_s);
            lo = lo_s - shift;
            hi = hi_s + shift;
        } else if (sv.style[d] == 8) {
            bool cl;
            const double rate = servo_rate(sv, d, p[d], &cl);
            if (cl) r.clamp |= 1 << d;
            r.cum[d] += (dt * rate) * r.prd[d];
            lo = lo_s - 0.5 * r.cum[d];
            hi = hi_s + 0.5 * r.cum[d];
        } else {
            continue;  // style none: the box stays as it is
        }
        r.lo[d] = lo;
        r.prd[d] = hi - lo;
    }
    *next = r;
}

__global__ void __launch_bounds__(kBlk) k_remap(int n, const double* __restrict__ xh, const tmps_adj_rec* prev,
                                                const tmps_adj_rec* next, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * n + i;
        const double lam = (xh[k] - prev->lo[c]) / prev->prd[c];
        x[k] = next->prd[c] * lam + next->lo[c];
    }
}

// ---------------------------------------------------------------- reverse

// x' = prd' (xh - lo) / prd + lo': the adjoint of xh in place, and the
// partial sums of x'bar and x'bar lam per dimension for the box adjoints.
__global__ void __launch_bounds__(kBlk) k_b_remap(int n, const double* __restrict__ xh, const tmps_adj_rec* prev,
                                                  const tmps_adj_rec* next, double* __restrict__ xb, Work W) {
    __shared__ double smem[6 * (kBlk / 32)];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s[6] = {0, 0, 0, 0, 0, 0};
    if (i < n) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const size_t k = (size_t)c * n + i;
            const double lam = (xh[k] - prev->lo[c]) / prev->prd[c];
            const double g = xb[k];
            s[c] = g;
            s[3 + c] = g * lam;
            xb[k] = g * (next->prd[c] / prev->prd[c]);
        }
    }
    block_sum<6, kBlk>(s, smem);
    if (threadIdx.x == 0) {
        const int nb = gridDim.x;
#pragma unroll
        for (int c = 0; c < 6; ++c) W.partk[(size_t)c * nb + blockIdx.x] = s[c];
    }
}

// Reverse of the servo and the pressure: box adjoints (slot of record n =
// step - 1 and of record n + 1 by parity), dL/d(virial total) into W.wbar.
__global__ void __launch_bounds__(256) k_b_servo(tmps_adj_servo sv, double dt, int64_t step, const tmps_adj_rec* prev,
                                                 const tmps_adj_rec* next, double qbar, int nbA, double* box_bar, Work W) {
    __shared__ double s[6];
    sum_partials<6>(W.partk, nbA, s);
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int n = (int)(step - 1);
    double* bn = box_bar + 9 * (n & 1);          // record n: lo 0..2, prd 3..5, cum 6..8
    double* bn1 = box_bar + 9 * ((n + 1) & 1);   // record n + 1
    double Pt[6], p[3], pb[3] = {0, 0, 0}, Pb[6] = {0, 0, 0, 0, 0, 0};
    const double vol = (prev->prd[0] * prev->prd[1]) * prev->prd[2];
    for (int c = 0; c < 6; ++c) Pt[c] = next->w[c] / vol;
    coupled(sv.couple, Pt, p);
    for (int d = 0; d < 3; ++d) {
        const double ratio = next->prd[d] / prev->prd[d];
        // remap
        bn1[d] += s[d];
        bn1[3 + d] += s[3 + d];
        bn[d] -= s[d] * ratio;
        bn[3 + d] -= s[3 + d] * ratio;
        if (sv.style[d] != 8) continue;
        // record n + 1's box from its cumulative shift: lo = lo_s - cum / 2, prd = L + cum
        const double cumb = bn1[6 + d] + bn1[3 + d] - 0.5 * bn1[d];
        // cum' = cum + (dt rate) prd
        bool cl;
        const double rate = servo_rate(sv, d, p[d], &cl);
        bn[6 + d] += cumb;
        bn[3 + d] += cumb * dt * rate;
        if (!((next->clamp >> d) & 1)) {
            double rb = cumb * dt * prev->prd[d] * sv.pgain[d];
            if (sv.normalize == 1) rb = rb / fabs(sv.ptarget[d]);
            pb[d] += rb;
        }
    }
    for (int c = 0; c < 9; ++c) bn1[c] = 0.0;
    // couple
    if (sv.couple == 1) {
        const double g = (pb[0] + pb[1] + pb[2]) / 3.0;
        Pb[0] = Pb[1] = Pb[2] = g;
    } else if (sv.couple == 2) {
        Pb[0] = Pb[1] = 0.5 * (pb[0] + pb[1]);
        Pb[2] = pb[2];
    } else if (sv.couple == 3) {
        Pb[1] = Pb[2] = 0.5 * (pb[1] + pb[2]);
        Pb[0] = pb[0];
    } else if (sv.couple == 4) {
        Pb[0] = Pb[2] = 0.5 * (pb[0] + pb[2]);
        Pb[1] = pb[1];
    } else {
        Pb[0] = pb[0];
        Pb[1] = pb[1];
        Pb[2] = pb[2];
    }
    // deviatoric stress q = Pzz - (Pxx + Pyy) / 2
    Pb[2] += qbar;
    Pb[0] -= 0.5 * qbar;
    Pb[1] -= 0.5 * qbar;
    // P = W / vol
    double volb = 0.0;
    for (int c = 0; c < 6; ++c) {
        W.wbar[c] = Pb[c] / vol;
        volb -= Pb[c] * Pt[c] / vol;
    }
    bn[3] += volb * prev->prd[1] * prev->prd[2];
    bn[4] += volb * prev->prd[0] * prev->prd[2];
    bn[5] += volb * prev->prd[0] * prev->prd[1];
}

// Reverse of the second half-kick and of the kinetic virial term.
__global__ void __launch_bounds__(kBlk) k_b_final(tmps_adj_sys S, double dt, tmps_adj_tape T, tmps_adj_bar B, Work W) {
    const int n = S.n;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double m = S.mass[a], r = S.radius[a], I = inertia(m, r), dtf = 0.5 * dt;
    double wb[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) wb[c] = W.wbar[c];
    double v[3], vb[3], f[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * n + a;
        f[c] = T.f[k];
        v[c] = T.vh[k] + dtf * (f[c] / m);
        vb[c] = B.v[k];
    }
    // kinetic m v_a v_b
    vb[0] += m * (2.0 * wb[0] * v[0] + wb[3] * v[1] + wb[4] * v[2]);
    vb[1] += m * (2.0 * wb[1] * v[1] + wb[3] * v[0] + wb[5] * v[2]);
    vb[2] += m * (2.0 * wb[2] * v[2] + wb[4] * v[0] + wb[5] * v[1]);
    double mb = wb[0] * v[0] * v[0] + wb[1] * v[1] * v[1] + wb[2] * v[2] * v[2] + wb[3] * v[0] * v[1] +
                wb[4] * v[0] * v[2] + wb[5] * v[1] * v[2];
    double Ib = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * n + a;
        // v = vh + dtf f / m
        B.v[k] = vb[c];
        B.f[k] += dtf * vb[c] / m;
        mb -= dtf * vb[c] * f[c] / (m * m);
        // w = wh + dtf t / I
        const double wbar = B.w[k];
        B.t[k] += dtf * wbar / I;
        Ib -= dtf * wbar * T.t[k] / (I * I);
    }
    B.mass[a] += mb + Ib * 0.4 * r * r;
    B.radius[a] += Ib * 0.8 * m * r;
}

// Reverse of the contact pass: per pair, recompute under the recorded mask,
// then the reverse; per-pair adjoints for the gather, the entering history's
// adjoint in place, parameter and image partials.
__global__ void __launch_bounds__(kBlk) k_b_pairs(tmps_adj_sys S, Params P, int shearupdate, const double* xs,
                                                  const double* vs, const double* ws, const double* __restrict__ sh_rec,
                                                  const uint8_t* __restrict__ mask_rec,
                                                  const tmps_adj_rec* __restrict__ box, const double* __restrict__ wbar,
                                                  tmps_adj_bar B, Work W) {
    __shared__ double smem[8 * (kBlk / 32)];
    const int n = S.n, np = S.npairs;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double part[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (p < np) {
        double prd[3], iprd[3], nimg[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            prd[c] = box->prd[c];
            iprd[c] = 1.0 / prd[c];
        }
        const int i = S.pi[p], j = S.pj[p];
        PairIn in;
        load_pair(S, xs, vs, ws, prd, iprd, p, i, j, in, nimg);
#pragma unroll
        for (int c = 0; c < 3; ++c) in.sh[c] = sh_rec[(size_t)c * np + p];
        PairOut o;
        PairTape t;
        int mask;
        const int rec = mask_rec[p];
        pair_forward(P, shearupdate, in, rec, o, t, &mask);
        PairBar b;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            b.fa[c] = B.f[(size_t)c * n + i];
            b.fb[c] = B.f[(size_t)c * n + j];
            b.ta[c] = B.t[(size_t)c * n + i];
            b.tb[c] = B.t[(size_t)c * n + j];
            b.sh[c] = B.shear[(size_t)c * np + p];
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) b.w[c] = wbar ? wbar[c] : 0.0;
        PairGrad g;
        pair_reverse(P, shearupdate, rec, in, o, t, b, g);
        double* G = W.gp;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            B.shear[(size_t)c * np + p] = g.sh[c];
            G[(size_t)c * np + p] = g.d[c];
            G[(size_t)(3 + c) * np + p] = g.vrel[c];
            G[(size_t)(6 + c) * np + p] = g.wa[c];
            G[(size_t)(9 + c) * np + p] = g.wb[c];
        }
        G[(size_t)12 * np + p] = g.ra;
        G[(size_t)13 * np + p] = g.rb;
        G[(size_t)14 * np + p] = g.ma;
        G[(size_t)15 * np + p] = g.mb;
        part[0] = g.kn;
        part[1] = g.kt;
        part[2] = g.gamman;
        part[3] = g.gammat;
        part[4] = g.xmu;
        // d = xa - xb - nimg prd
#pragma unroll
        for (int c = 0; c < 3; ++c) part[5 + c] = -nimg[c] * g.d[c];
    }
    block_sum<8, kBlk>(part, smem);
    if (threadIdx.x == 0) {
        const int nb = gridDim.x;
#pragma unroll
        for (int c = 0; c < 8; ++c) W.partg[(size_t)c * nb + blockIdx.x] = part[c];
    }
}

__global__ void __launch_bounds__(256) k_b_reduce(int nbP, int slot, tmps_adj_bar B, Work W) {
    __shared__ double s[8];
    sum_partials<8>(W.partg, nbP, s);
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int c = 0; c < 5; ++c) B.params[c] += s[c];
    for (int c = 0; c < 3; ++c) B.box[9 * slot + 3 + c] += s[5 + c];
}

// Per-atom sums of the pairs' adjoints (as i, then as j).
__global__ void __launch_bounds__(kBlk) k_b_gather(tmps_adj_sys S, tmps_adj_bar B, Work W) {
    const int n = S.n, np = S.npairs;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double* G = W.gp;
    double xb[3] = {0, 0, 0}, vb[3] = {0, 0, 0}, wb[3] = {0, 0, 0}, rb = 0.0, mb = 0.0;
    for (int q = S.ibeg[a]; q < S.ibeg[a + 1]; ++q) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            xb[c] += G[(size_t)c * np + q];
            vb[c] += G[(size_t)(3 + c) * np + q];
            wb[c] += G[(size_t)(6 + c) * np + q];
        }
        rb += G[(size_t)12 * np + q];
        mb += G[(size_t)14 * np + q];
    }
    for (int k = S.jbeg[a]; k < S.jbeg[a + 1]; ++k) {
        const int q = S.jlist[k];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            xb[c] -= G[(size_t)c * np + q];
            vb[c] -= G[(size_t)(3 + c) * np + q];
            wb[c] += G[(size_t)(9 + c) * np + q];
        }
        rb += G[(size_t)13 * np + q];
        mb += G[(size_t)15 * np + q];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * n + a;
        B.x[k] += xb[c];
        B.v[k] += vb[c];
        B.w[k] += wb[c];
    }
    B.radius[a] += rb;
    B.mass[a] += mb;
}

// Reverse of the first half-kick and the drift: leaves the adjoint of the
// state before the step, and the adjoint of the forces it started from.
__global__ void __launch_bounds__(kBlk) k_b_initial(tmps_adj_sys S, double dt, const double* __restrict__ fprev,
                                                    const double* __restrict__ tprev, tmps_adj_bar B) {
    const int n = S.n;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double m = S.mass[a], r = S.radius[a], I = inertia(m, r), dtf = 0.5 * dt;
    double mb = 0.0, Ib = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * n + a;
        // x = x0 + dt vh; vh = v0 + dtf f / m
        const double vhb = B.v[k] + dt * B.x[k];
        B.v[k] = vhb;
        B.f[k] = dtf * vhb / m;
        mb -= dtf * vhb * fprev[k] / (m * m);
        // wh = w0 + dtf t / I
        const double whb = B.w[k];
        B.t[k] = dtf * whb / I;
        Ib -= dtf * whb * tprev[k] / (I * I);
    }
    B.mass[a] += mb + Ib * 0.4 * r * r;
    B.radius[a] += Ib * 0.8 * m * r;
}

bool ok() { return cudaPeekAtLastError() == cudaSuccess; }

bool sys_ok(const tmps_adj_sys* s) {
    return s && s->n >= 0 && s->npairs >= 0 && s->x && s->v && s->w && s->f && s->t && s->radius && s->mass &&
           (s->npairs == 0 || (s->shear && s->pi && s->pj)) && s->ibeg && s->jbeg && (s->npairs == 0 || s->jlist);
}

}  // namespace

extern "C" {

int64_t tmps_adj_workspace_bytes(int32_t n, int32_t npairs) {
    if (n < 0 || npairs < 0) return -1;
    return (int64_t)work_bytes(n, npairs);
}

int tmps_adj_pairs(int32_t n, const double* d_x, const double* d_radius, const tmps_adj_rec* d_box, double skin,
                   int32_t* d_count, const int32_t* d_ibeg, int32_t* d_pi, int32_t* d_pj, void* stream) {
    if (n < 0 || !d_x || !d_radius || !d_box || !(skin >= 0.0)) return TMPS_ERR_BAD_ARG;
    if (!d_pj && !d_count) return TMPS_ERR_BAD_ARG;
    if (d_pj && (!d_ibeg || !d_pi)) return TMPS_ERR_BAD_ARG;
    if (n == 0) return TMPS_OK;
    k_pairs_build<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(n, d_x, d_radius, d_box, skin, d_count, d_ibeg,
                                                                      d_pi, d_pj);
    note_launches(1);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_pair_map(int32_t nold, const int32_t* d_old_pi, const int32_t* d_old_pj, const int32_t* d_new_ibeg,
                      const int32_t* d_new_pj, int32_t* d_map, void* stream) {
    if (nold < 0 || (nold > 0 && (!d_old_pi || !d_old_pj || !d_new_ibeg || !d_new_pj || !d_map)))
        return TMPS_ERR_BAD_ARG;
    if (nold == 0) return TMPS_OK;
    k_pair_map<<<grid_for(nold, kBlk), kBlk, 0, (cudaStream_t)stream>>>(nold, d_old_pi, d_old_pj, d_new_ibeg, d_new_pj,
                                                                        d_map);
    note_launches(1);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_carry(int32_t nold, int32_t nnew, const int32_t* d_map, double* d_old, double* d_new, int32_t reverse,
                   void* stream) {
    if (nold < 0 || nnew < 0 || (nold > 0 && (!d_map || !d_old || (nnew > 0 && !d_new)))) return TMPS_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (!reverse && nnew > 0 && cudaMemsetAsync(d_new, 0, sizeof(double) * 3 * (size_t)nnew, st) != cudaSuccess)
        return TMPS_ERR_CUDA;
    if (nold == 0) return TMPS_OK;
    k_carry<<<grid_for(nold, kBlk), kBlk, 0, st>>>(nold, nnew, d_map, d_old, d_new, reverse);
    note_launches(1);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_setup(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_rec* d_box,
                   const tmps_adj_tape* tape, void* work, void* stream) {
    if (!sys_ok(s) || !p || !d_box || !tape || !work || !tape->shear || !tape->mask) return TMPS_ERR_BAD_ARG;
    if (s->n == 0) return TMPS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    Work W = carve(work, s->n, s->npairs);
    if (s->npairs > 0) {
        k_pairs<<<grid_for(s->npairs, kBlk), kBlk, 0, st>>>(*s, to_params(*p), 0, s->x, s->v, s->w, d_box,
                                                             tape->shear, tape->mask, W);
        note_launches(1);
    }
    k_gather<<<grid_for(s->n, kBlk), kBlk, 0, st>>>(*s, p->dt, 0, nullptr, nullptr, tape->f, tape->t, W);
    note_launches(1);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_initial(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_tape* tape,
                     const double* d_xbuild, uint64_t* d_disp, void* stream) {
    if (!sys_ok(s) || !p || !tape || !tape->xh || !tape->vh || !tape->wh || !d_xbuild || !d_disp)
        return TMPS_ERR_BAD_ARG;
    if (s->n == 0) return TMPS_OK;
    k_initial<<<grid_for(s->n, kBlk), kBlk, 0, (cudaStream_t)stream>>>(*s, p->dt, *tape, d_xbuild,
                                                                        (unsigned long long*)d_disp);
    note_launches(1);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_finish(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_servo* sv,
                    const tmps_adj_tape* tape, tmps_adj_rec* d_rec, int64_t step, void* work, void* stream) {
    if (!sys_ok(s) || !p || !sv || !tape || !d_rec || step < 1 || !work || !tape->xh || !tape->shear || !tape->mask ||
        !tape->f || !tape->t)
        return TMPS_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    Work W = carve(work, s->n, s->npairs);
    const int nbA = grid_for(s->n, kBlk), nbP = grid_for(s->npairs, kBlk);
    tmps_adj_rec* prev = d_rec + (step - 1);
    tmps_adj_rec* next = d_rec + step;
    if (s->npairs > 0) {
        k_pairs<<<nbP, kBlk, 0, st>>>(*s, to_params(*p), 1, tape->xh, tape->vh, tape->wh, prev, tape->shear,
                                      tape->mask, W);
        note_launches(1);
    } else if (cudaMemsetAsync(W.partw, 0, sizeof(double) * 6 * nbP, st) != cudaSuccess) {
        return TMPS_ERR_CUDA;
    }
    if (s->n > 0) {
        k_gather<<<nbA, kBlk, 0, st>>>(*s, p->dt, 1, tape->vh, tape->wh, tape->f, tape->t, W);
        note_launches(1);
    } else if (cudaMemsetAsync(W.partk, 0, sizeof(double) * 6 * nbA, st) != cudaSuccess) {
        return TMPS_ERR_CUDA;
    }
    k_servo<<<1, 256, 0, st>>>(*sv, p->dt, step, prev, next, nbP, nbA, W);
    note_launches(1);
    if (s->n > 0) {
        k_remap<<<nbA, kBlk, 0, st>>>(s->n, tape->xh, prev, next, s->x);
        note_launches(1);
    }
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_step_back(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_servo* sv,
                       const tmps_adj_tape* tape, const tmps_adj_rec* d_rec, int64_t step, const double* d_fprev,
                       const double* d_tprev, double qbar, const tmps_adj_bar* b, void* work, void* stream) {
    if (!sys_ok(s) || !p || !sv || !tape || !d_rec || step < 1 || !d_fprev || !d_tprev || !b || !work)
        return TMPS_ERR_BAD_ARG;
    if (!b->x || !b->v || !b->w || !b->f || !b->t || !b->radius || !b->mass || !b->params || !b->box ||
        (s->npairs > 0 && !b->shear))
        return TMPS_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    Work W = carve(work, s->n, s->npairs);
    const int nbA = grid_for(s->n, kBlk), nbP = grid_for(s->npairs, kBlk);
    const tmps_adj_rec* prev = d_rec + (step - 1);
    const tmps_adj_rec* next = d_rec + step;
    if (s->n > 0) {
        k_b_remap<<<nbA, kBlk, 0, st>>>(s->n, tape->xh, prev, next, b->x, W);
        note_launches(1);
    } else if (cudaMemsetAsync(W.partk, 0, sizeof(double) * 6 * nbA, st) != cudaSuccess) {
        return TMPS_ERR_CUDA;
    }
    k_b_servo<<<1, 256, 0, st>>>(*sv, p->dt, step, prev, next, qbar, nbA, b->box, W);
    note_launches(1);
    if (s->n == 0) return ok() ? TMPS_OK : TMPS_ERR_CUDA;
    k_b_final<<<nbA, kBlk, 0, st>>>(*s, p->dt, *tape, *b, W);
    note_launches(1);
    if (s->npairs > 0) {
        k_b_pairs<<<nbP, kBlk, 0, st>>>(*s, to_params(*p), 1, tape->xh, tape->vh, tape->wh, tape->shear, tape->mask,
                                        prev, W.wbar, *b, W);
        k_b_reduce<<<1, 256, 0, st>>>(nbP, (int)((step - 1) & 1), *b, W);
        k_b_gather<<<nbA, kBlk, 0, st>>>(*s, *b, W);
        note_launches(3);
    }
    k_b_initial<<<nbA, kBlk, 0, st>>>(*s, p->dt, d_fprev, d_tprev, *b);
    note_launches(1);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_adj_setup_back(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_rec* d_box,
                        const tmps_adj_tape* tape, const tmps_adj_bar* b, void* work, void* stream) {
    if (!sys_ok(s) || !p || !d_box || !tape || !b || !work || !b->x || !b->v || !b->w || !b->f || !b->t ||
        !b->radius || !b->mass || !b->params || !b->box || (s->npairs > 0 && (!b->shear || !tape->shear || !tape->mask)))
        return TMPS_ERR_BAD_ARG;
    if (s->n == 0 || s->npairs == 0) return TMPS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    Work W = carve(work, s->n, s->npairs);
    const int nbA = grid_for(s->n, kBlk), nbP = grid_for(s->npairs, kBlk);
    k_b_pairs<<<nbP, kBlk, 0, st>>>(*s, to_params(*p), 0, s->x, s->v, s->w, tape->shear, tape->mask, d_box, nullptr,
                                    *b, W);
    k_b_reduce<<<1, 256, 0, st>>>(nbP, 0, *b, W);
    k_b_gather<<<nbA, kBlk, 0, st>>>(*s, *b, W);
    note_launches(3);
    return ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

}  // extern "C"
