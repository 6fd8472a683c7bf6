// Granular walls: a flat axis-aligned plane (fix wall/gran) and the curved
// side of a cylinder region (fix wall/gran/region), one thread per atom, FP64,
// in the reference kernels' evaluation order.  The wall is a partner of zero
// radius and infinite mass (radsum = Reff = r_i, meff = m_i, arm = r_i).
#include "tmps_common.cuh"

using namespace tmps;

namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// The tangential part shared by both walls (linear_history_classic with the
// contact-radius factor `poly`, or the history-free viscous dashpot with the
// Coulomb cap): returns fs; updates the slot's history.
__device__ __forceinline__ void tangential(const tmps_wall_params& P, double dt, int upd, const double* n,
                                           const double* vtr, double vrel, double fscrit, double damp_t,
                                           double poly, double* sh, int* touch, double* fs) {
    if (P.history) {
        double hist[3] = {sh[0], sh[1], sh[2]};
        if (*touch == 0) {
            hist[0] = hist[1] = hist[2] = 0.0;
            *touch = 1;
        }
        if (upd)
            for (int k = 0; k < 3; ++k) hist[k] = hist[k] + vtr[k] * dt;
        const double shrmag = sqrt(dot3(hist, hist));
        if (upd) {
            const double hn = dot3(hist, n);
            for (int k = 0; k < 3; ++k) hist[k] = hist[k] - hn * n[k];
        }
        double fdamp[3];
        for (int k = 0; k < 3; ++k) {
            fdamp[k] = -damp_t * vtr[k];
            // plane: -kt hist + fdamp (poly == 1); cylinder: -kt poly hist + fdamp
            fs[k] = P.kind == 0 ? -P.kt * hist[k] + fdamp[k] : (-P.kt * poly) * hist[k] + fdamp[k];
        }
        const double magfs = sqrt(dot3(fs, fs));
        if (magfs > fscrit) {
            if (shrmag != 0.0) {
                const double s = fscrit / magfs;
                const double kk = P.kind == 0 ? P.kt : P.kt * poly;
                for (int k = 0; k < 3; ++k) {
                    fs[k] = fs[k] * s;
                    hist[k] = -(fs[k] - fdamp[k]) / kk;
                }
            } else {
                fs[0] = fs[1] = fs[2] = 0.0;
            }
        }
        sh[0] = hist[0];
        sh[1] = hist[1];
        sh[2] = hist[2];
    } else {
        double ft = 0.0;
        if (vrel != 0.0) ft = fmin(fscrit, damp_t * vrel) / vrel;
        for (int k = 0; k < 3; ++k) fs[k] = -ft * vtr[k];
    }
}

__global__ void __launch_bounds__(kBlock) k_wall(tmps_atoms a, tmps_wall_params P, double dt, int upd,
                                                 double* __restrict__ shear, int32_t* __restrict__ touch_,
                                                 int nslots) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    if (i >= n) return;
    const int u = a.uid ? a.uid[i] : i;
    double sh[3] = {0.0, 0.0, 0.0};
    int touch = 0;
    if (P.history) {
        sh[0] = shear[u];
        sh[1] = shear[(size_t)nslots + u];
        sh[2] = shear[2 * (size_t)nslots + u];
        touch = touch_[u];
    }
    const double4 xr = ld4(a.xr, i), vm = ld4(a.vm, i), om = ld4(a.om, i);
    const double x[3] = {xr.x, xr.y, xr.z}, v[3] = {vm.x, vm.y, vm.z}, w[3] = {om.x, om.y, om.z};
    const double ri = xr.w, mi = vm.w;
    bool contact = false;
    double F[3] = {0, 0, 0}, T[3] = {0, 0, 0};
    if (P.kind == 0) {
        // FixWallGran.post_force_kernel (wall_gran.py:143-228)
        double nrm[3] = {0, 0, 0}, vwall[3] = {0, 0, 0};
        nrm[P.axis] = P.side == 1 ? -1.0 : 1.0;
        vwall[P.axis] = P.vwall_n;
        if (P.shear_axis >= 0) vwall[P.shear_axis] = P.vwall_s;
        const double dist = P.side == -1 ? x[P.axis] - P.coord : P.coord - x[P.axis];
        const double delta = ri - dist;
        if (delta > 0.0) {
            contact = true;
            const double meff = mi;
            double vr[3], vt[3], wr[3], c[3], vtr[3];
            for (int k = 0; k < 3; ++k) vr[k] = v[k] - vwall[k];
            const double vnnr = dot3(vr, nrm);
            for (int k = 0; k < 3; ++k) {
                vt[k] = vr[k] - vnnr * nrm[k];
                wr[k] = ri * w[k];
            }
            cross3(wr, nrm, c);
            for (int k = 0; k < 3; ++k) vtr[k] = vt[k] - c[k];
            const double vrel = sqrt(dot3(vtr, vtr));
            const double damp_prefactor = meff * P.gamman;
            double fntot = P.kn * delta - damp_prefactor * vnnr;
            if (P.limit_damping == 1) fntot = fmax(fntot, 0.0);
            const double fscrit = P.xmu * fabs(fntot);
            const double damp_t = meff * P.gammat;
            double fs[3];
            tangential(P, dt, upd, nrm, vtr, vrel, fscrit, damp_t, 1.0, sh, &touch, fs);
            double nf[3];
            cross3(nrm, fs, nf);
            for (int k = 0; k < 3; ++k) {
                F[k] = fntot * nrm[k] + fs[k];
                T[k] = -ri * nf[k];
            }
        }
    } else {
        // FixWallGranRegion.post_force_kernel (wall_gran_region.py:134-276)
        const double pa = x[P.axis];
        const bool inside = !(P.has_axis_bounds == 1 && (pa < P.axis_lo || pa > P.axis_hi));
        if (inside) {
            const int a1 = P.axis == 0 ? 1 : 0, a2 = P.axis == 2 ? 1 : 2;
            const double d1 = x[a1] - P.c1, d2 = x[a2] - P.c2;
            const double r_perp = sqrt(d1 * d1 + d2 * d2);
            if (r_perp > 1e-14) {
                const double inv = 1.0 / r_perp;
                const double u1 = d1 * inv, u2 = d2 * inv;
                const double sg = P.side == -1 ? -1.0 : 1.0;
                double nrm[3] = {0, 0, 0};
                nrm[a1] = sg * u1;
                nrm[a2] = sg * u2;
                const double delta = P.side == -1 ? ri - (P.radius - r_perp) : ri - (r_perp - P.radius);
                if (delta > 0.0) {
                    contact = true;
                    double c[3], vr[3], vrt[3];
                    cross3(w, nrm, c);
                    for (int k = 0; k < 3; ++k) vr[k] = v[k] - ri * c[k];
                    const double vn = dot3(vr, nrm);
                    for (int k = 0; k < 3; ++k) vrt[k] = vr[k] - vn * nrm[k];
                    const double vrel = sqrt(dot3(vrt, vrt));
                    const double poly = P.hertz ? sqrt(ri * delta) : 1.0;
                    const double fn_elastic = P.kn * delta * poly;
                    const double damp_prefactor = mi * P.gamman * poly;
                    double fntot = fn_elastic - damp_prefactor * vn;
                    if (P.limit_damping == 1) fntot = fmax(fntot, 0.0);
                    const double fscrit = P.xmu * fabs(fntot);
                    const double damp_t = mi * P.gammat * poly;
                    double fs[3];
                    tangential(P, dt, upd, nrm, vrt, vrel, fscrit, damp_t, poly, sh, &touch, fs);
                    double nf[3];
                    cross3(nrm, fs, nf);
                    for (int k = 0; k < 3; ++k) {
                        F[k] = fntot * nrm[k] + fs[k];
                        T[k] = -ri * nf[k];
                    }
                }
            }
        }
    }
    if (contact) {
        for (int k = 0; k < 3; ++k) {
            a.f[(size_t)k * n + i] += F[k];
            a.torque[(size_t)k * n + i] += T[k];
        }
    } else {
        touch = 0;
        sh[0] = sh[1] = sh[2] = 0.0;
    }
    if (P.history) {
        shear[u] = sh[0];
        shear[(size_t)nslots + u] = sh[1];
        shear[2 * (size_t)nslots + u] = sh[2];
        touch_[u] = touch;
    }
}

}  // namespace

extern "C" int tmps_wall_gran(const tmps_atoms* a, const tmps_wall_params* p, double dt, int32_t history_update,
                              double* d_shear, int32_t* d_touch, int32_t nslots, void* stream) {
    if (!a || !p || a->n < 0) return TMPS_ERR_BAD_ARG;
    if (p->kind < 0 || p->kind > 1 || p->axis < 0 || p->axis > 2 || (p->side != -1 && p->side != 1))
        return TMPS_ERR_BAD_ARG;
    if (p->kind == 0 && (p->shear_axis < -1 || p->shear_axis > 2 || p->shear_axis == p->axis)) return TMPS_ERR_BAD_ARG;
    if (p->history && (!d_shear || !d_touch || nslots < a->n)) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_wall<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, *p, dt, history_update, d_shear,
                                                                          d_touch, nslots);
    note_launches(1);
    return cudaPeekAtLastError() == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}
