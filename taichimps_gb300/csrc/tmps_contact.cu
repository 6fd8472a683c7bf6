// Contact force kernel, FP64 form: one thread per atom over its full
// neighbor row (slot-major, so a warp's loads of slot k are one coalesced
// line).  Forces, torques and the virial of the row atom are accumulated in
// registers and stored once: no atomics.  Each contact is evaluated by both
// of its atoms in the same orientation (lower internal index first), with
// bit-identical inputs, so both atoms see the same force and the two stored
// copies of the shear stay exact negatives of one another.
#include "tmps_contact.cuh"

using namespace tmps;

namespace {

constexpr int kBlock = 128;

template <int STYLE>
__global__ void __launch_bounds__(kBlock)
    k_contact64(tmps_atoms A, tmps_nlist L, tmps_pair_params P, const tmps_box* __restrict__ B,
                double dt, int shearupdate, int accumulate) {
    constexpr bool kHist = STYLE == STYLE_HOOKE_HISTORY || STYLE == STYLE_HERTZ_HISTORY ||
                           STYLE == STYLE_GRANULAR;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = A.n;
    if (i >= n) return;
    const bool hist = kHist && (STYLE != STYLE_GRANULAR || P.tangential_id >= 2 || P.rolling_id != 0);
    const bool roll = STYLE == STYLE_GRANULAR && P.rolling_id != 0;
    double prd[3], iprd[3];
    int per[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        prd[k] = B->prd[k];
        iprd[k] = B->inv_prd[k];
        per[k] = B->per[k];
    }
    const int vremap = B->vremap;
    const double4 xi = ld4(A.xr, i), vi = ld4(A.vm, i), wi = ld4(A.om, i);
    double F[3] = {0, 0, 0}, Tq[3] = {0, 0, 0}, V[6] = {0, 0, 0, 0, 0, 0};
    const int nn = L.nnb[i];
    const uint64_t touch = hist ? L.touch[i] : 0ull;
    uint64_t newtouch = 0ull;
    const size_t ss = (size_t)L.slots * n;
    // the separation of i and partner j in the canonical orientation (lower
    // internal index first) and the contact test, as the reference makes it
    auto geom = [&](const int j, const double4 xj, PairIn<double>& in, double (&nimg)[3]) -> bool {
        const bool lo = i < j;  // this atom is `a` of the canonical pair
        const double4 xa = lo ? xi : xj, xb = lo ? xj : xi;
        in.d[0] = xa.x - xb.x;
        in.d[1] = xa.y - xb.y;
        in.d[2] = xa.z - xb.z;
        // Image count.  rint(d / prd) and rint(d * (1/prd)) differ only for a
        // separation within an ulp of half a box, which a listed neighbor
        // (|d| < cut <= prd / 3 after the image) never is.
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            nimg[c] = 0.0;
            if (per[c] == 1) {
                nimg[c] = rint(in.d[c] * iprd[c]);
                in.d[c] = image_sub64(in.d[c], nimg[c], prd[c]);
            }
        }
        in.rsq = rsq64(in.d);
        in.ra = xa.w;
        in.rb = xb.w;
        const double radsum = in.ra + in.rb;
        return in.rsq < __dmul_rn(radsum, radsum) && in.rsq > 1e-28;
    };
    // The contact test of every row entry, four at a time (all loads in
    // flight together), then the law over the slots in contact, in slot order.
    // An FP32 screen from the positions' truncated copies (approx_f32) first
    // rules out the entries that cannot touch, by a margin of 1e-5 of the
    // magnitudes involved, far above its error (2^-20 of each value plus
    // FP32 rounding); only the rest take the exact FP64 test, whose cost on
    // this part's narrow FP64 pipe is per warp, however few lanes are active.
    const float xi32[3] = {approx_f32(xi.x), approx_f32(xi.y), approx_f32(xi.z)}, ri32 = approx_f32(xi.w);
    float prd32[3], iprd32[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        prd32[c] = approx_f32(prd[c]);
        iprd32[c] = approx_f32(iprd[c]);
    }
    const float base32 = l1f(xi32[0], xi32[1], xi32[2]) + l1f(prd32[0], prd32[1], prd32[2]);
    uint64_t cmask = 0ull;
    for (int k0 = 0; k0 < nn; k0 += 4) {
        int jj[4];
        double4 xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) jj[u] = k0 + u < nn ? L.nbr[(size_t)(k0 + u) * n + i] & kNbrIndexMask : 0;
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k0 + u < nn) xj[u] = ld4(A.xr, jj[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (k0 + u >= nn) continue;
            const float xj32[3] = {approx_f32(xj[u].x), approx_f32(xj[u].y), approx_f32(xj[u].z)};
            float d[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                d[c] = xi32[c] - xj32[c];
                if (per[c] == 1) d[c] -= rintf(d[c] * iprd32[c]) * prd32[c];
            }
            const float rq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
            const float rs = ri32 + approx_f32(xj[u].w);
            const float lim = rs + 1e-5f * ((base32 + l1f(xj32[0], xj32[1], xj32[2])) + rs);
            if (rq > lim * lim) continue;  // out of reach beyond doubt (a NaN goes on to the exact test)
            PairIn<double> t;
            double ni[3];
            if (geom(jj[u], xj[u], t, ni)) cmask |= 1ull << (k0 + u);
        }
    }
    for (uint64_t m = cmask; m; m &= m - 1ull) {
        const int k = __ffsll((long long)m) - 1;
        const int j = L.nbr[(size_t)k * n + i] & kNbrIndexMask;
        const bool lo = i < j;
        PairIn<double> in;
        double nimg[3];
        geom(j, ld4(A.xr, j), in, nimg);
        const double radsum = in.ra + in.rb;
        in.r = sqrt(in.rsq);
        in.delta = radsum - in.r;
        const double4 vj = ld4(A.vm, j), wj = ld4(A.om, j);
        const double4 va = lo ? vi : vj, vb = lo ? vj : vi, wa = lo ? wi : wj, wb = lo ? wj : wi;
        double dv[3] = {0, 0, 0};
        if (vremap) {
            const double* h = B->h_rate;
            dv[0] = (nimg[0] * h[0] + nimg[1] * h[5]) + nimg[2] * h[4];
            dv[1] = nimg[1] * h[1] + nimg[2] * h[3];
            dv[2] = nimg[2] * h[2];
        }
        in.ma = va.w;
        in.mb = vb.w;
        in.va[0] = va.x; in.va[1] = va.y; in.va[2] = va.z;
        in.vb[0] = vb.x + dv[0]; in.vb[1] = vb.y + dv[1]; in.vb[2] = vb.z + dv[2];
        in.wa[0] = wa.x; in.wa[1] = wa.y; in.wa[2] = wa.z;
        in.wb[0] = wb.x; in.wb[1] = wb.y; in.wb[2] = wb.z;
        double sh[3] = {0, 0, 0}, rl[3] = {0, 0, 0};
        const size_t so = (size_t)k * n + i;
        if (hist && ((touch >> k) & 1ull)) {
            const double sg = lo ? 1.0 : -1.0;
            sh[0] = sg * L.shear[so];
            sh[1] = sg * L.shear[ss + so];
            sh[2] = sg * L.shear[2 * ss + so];
            if (roll) {
                rl[0] = sg * L.rolling[so];
                rl[1] = sg * L.rolling[ss + so];
                rl[2] = sg * L.rolling[2 * ss + so];
            }
        }
        PairOut<double> out;
        contact_law<double, STYLE>(P, dt, shearupdate, in, sh, rl, out);
        if (hist) {
            const double sg = lo ? 1.0 : -1.0;
            L.shear[so] = sg * sh[0];
            L.shear[ss + so] = sg * sh[1];
            L.shear[2 * ss + so] = sg * sh[2];
            if (roll) {
                L.rolling[so] = sg * rl[0];
                L.rolling[ss + so] = sg * rl[1];
                L.rolling[2 * ss + so] = sg * rl[2];
            }
            newtouch |= 1ull << k;
        }
        const double sgn = lo ? 1.0 : -1.0;
        const double arm = lo ? out.arm_a : out.arm_b;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            F[c] += sgn * out.f[c];
            Tq[c] += arm * out.tor[c];
            Tq[c] += sgn * out.troll[c];
        }
        V[0] += 0.5 * (in.d[0] * out.f[0]);
        V[1] += 0.5 * (in.d[1] * out.f[1]);
        V[2] += 0.5 * (in.d[2] * out.f[2]);
        V[3] += 0.5 * (in.d[0] * out.f[1]);
        V[4] += 0.5 * (in.d[0] * out.f[2]);
        V[5] += 0.5 * (in.d[1] * out.f[2]);
    }
    if (hist) L.touch[i] = newtouch;
    if (accumulate) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            A.f[c * n + i] += F[c];
            A.torque[c * n + i] += Tq[c];
        }
        if (A.virial)
#pragma unroll
            for (int c = 0; c < 6; ++c) A.virial[c * n + i] += V[c];
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            A.f[c * n + i] = F[c];
            A.torque[c * n + i] = Tq[c];
        }
        if (A.virial)
#pragma unroll
            for (int c = 0; c < 6; ++c) A.virial[c * n + i] = V[c];
    }
}

bool launch_ok() { return cudaPeekAtLastError() == cudaSuccess; }

bool params_ok(const tmps_pair_params* p) {
    if (p->style < 0 || p->style > 4) return false;
    if (p->style == 4) {
        if (p->normal_id < 0 || p->normal_id > 2 || p->damping_id < 0 || p->damping_id > 5 ||
            p->tangential_id < 0 || p->tangential_id > 3 || p->rolling_id < 0 || p->rolling_id > 1)
            return false;
    }
    return true;
}

// ComputeContactAtom.compute_kernel (computes/contact_atom.py:21-52): the
// number of neighbors in geometric contact, rsq < (ri + rj)^2 and rsq > 1e-18,
// each contact counted for both partners.  On the full list every atom counts
// its own row; d = x_i - x_j is the exact negation of the partner's, so both
// sides see the same rsq.
__global__ void __launch_bounds__(kBlock) k_contact_count(tmps_atoms A, tmps_nlist L, const tmps_box* __restrict__ B,
                                                          int32_t* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = A.n;
    if (i >= n) return;
    double prd[3];
    int per[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        prd[k] = B->prd[k];
        per[k] = B->per[k];
    }
    const double4 xi = ld4(A.xr, i);
    const int nn = L.nnb[i];
    int c = 0;
    for (int k = 0; k < nn; ++k) {
        const double4 xj = ld4(A.xr, L.nbr[(size_t)k * n + i] & kNbrIndexMask);
        // Domain.minimum_image (domain.py:481-486) and the dot product, with
        // explicit round-to-nearest operations: an integer result admits no
        // contraction that could move a pair across the threshold
        double d[3] = {__dsub_rn(xi.x, xj.x), __dsub_rn(xi.y, xj.y), __dsub_rn(xi.z, xj.z)};
#pragma unroll
        for (int q = 0; q < 3; ++q)
            if (per[q] == 1) d[q] = __dsub_rn(d[q], __dmul_rn(prd[q], round(__ddiv_rn(d[q], prd[q]))));
        const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
        const double radsum = __dadd_rn(xi.w, xj.w);
        if (rsq < __dmul_rn(radsum, radsum) && rsq > 1e-18) ++c;
    }
    count[i] = c;
}

}  // namespace

extern "C" {

int tmps_contact_count(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box, int32_t* d_count,
                       void* stream) {
    if (!a || !nl || !d_box || !d_count || a->n < 0 || nl->n != a->n) return TMPS_ERR_BAD_ARG;
    if (nl->slots < 1 || nl->slots > kMaxSlots) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    k_contact_count<<<grid_for(a->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*a, *nl, d_box, d_count);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_contact(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box,
                 const tmps_pair_params* p, double dt, int32_t shearupdate, int32_t accumulate,
                 void* stream) {
    if (!a || !nl || !d_box || !p || a->n < 0 || nl->n != a->n || !params_ok(p)) return TMPS_ERR_BAD_ARG;
    if (nl->slots < 1 || nl->slots > kMaxSlots) return TMPS_ERR_BAD_ARG;
    if (p->style == 4 && p->rolling_id != 0 && !nl->rolling) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    const int g = grid_for(a->n, kBlock);
    cudaStream_t s = (cudaStream_t)stream;
    switch (p->style) {
        case 0: k_contact64<0><<<g, kBlock, 0, s>>>(*a, *nl, *p, d_box, dt, shearupdate, accumulate); break;
        case 1: k_contact64<1><<<g, kBlock, 0, s>>>(*a, *nl, *p, d_box, dt, shearupdate, accumulate); break;
        case 2: k_contact64<2><<<g, kBlock, 0, s>>>(*a, *nl, *p, d_box, dt, shearupdate, accumulate); break;
        case 3: k_contact64<3><<<g, kBlock, 0, s>>>(*a, *nl, *p, d_box, dt, shearupdate, accumulate); break;
        default: k_contact64<4><<<g, kBlock, 0, s>>>(*a, *nl, *p, d_box, dt, shearupdate, accumulate); break;
    }
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

}  // extern "C"
