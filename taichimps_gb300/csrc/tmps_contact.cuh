// The contact laws, written once over the arithmetic type T.
//
// T = double gives the plain FP64 form; T = float gives the mixed form, where
// the per-contact shear history stays double (the many tiny vtr*dt
// increments are added in FP64) and everything else runs in FP32.
//
// Every law is evaluated for one canonical orientation a -> b of the pair
// (d = x_a - x_b after the minimum image).  The expressions follow the
// reference kernels term for term:
//   gran/hooke            GRANULAR/hooke.py:83-143
//   gran/hooke/history    GRANULAR/hooke_history.py:144-217
//   gran/hertz            GRANULAR/hertz.py:77-118
//   gran/hertz/history    GRANULAR/hertz_history.py:92-157
//   granular              GRANULAR/granular.py:316-414 (+ rotate_rescale :271-280)
#pragma once

#include "tmps_common.cuh"

namespace tmps {

enum { STYLE_HOOKE = 0, STYLE_HOOKE_HISTORY = 1, STYLE_HERTZ = 2, STYLE_HERTZ_HISTORY = 3, STYLE_GRANULAR = 4 };

template <int STYLE>
struct StyleTraits {
    static constexpr bool legacy = STYLE != STYLE_GRANULAR;
    static constexpr bool hertz = STYLE == STYLE_HERTZ || STYLE == STYLE_HERTZ_HISTORY;
    static constexpr bool legacy_history = STYLE == STYLE_HOOKE_HISTORY || STYLE == STYLE_HERTZ_HISTORY;
};

// Division and square root of the law.  The FP64 form keeps IEEE-rounded
// operations (its results follow the reference to 1e-12).  The mixed form's
// law is FP32 arithmetic whose every operation already rounds at 2^-24, so
// it uses the hardware's approximate reciprocal and reciprocal square root
// (errors of a few ulp, the same order): a tenth of the instructions of the
// IEEE sequences.
template <typename T>
TMPS_DEV T ldiv(T a, T b) { return a / b; }
template <>
TMPS_DEV float ldiv<float>(float a, float b) { return __fdividef(a, b); }
template <typename T>
TMPS_DEV T lsqrt(T a) { return sqrt(a); }
template <>
TMPS_DEV float lsqrt<float>(float a) {
    // a * rsqrt(a); IEEE sqrtf for zero and for tiny arguments, whose reciprocal
    // square root would overflow
    return a >= 1e-30f ? a * rsqrtf(a) : sqrtf(a);
}

// The FP64 form's separation component and |d|^2, every operation rounded as
// the reference writes it (d - n prd, d0 d0 + d1 d1 + d2 d2), with no
// multiply-add contraction: the overlap radsum - |d| of a near contact cancels
// about three digits, so a contracted |d|^2 or image shift would move a force
// by ~1e-13 relative.
TMPS_DEV double image_sub64(double d, double nimg, double prd) { return __dsub_rn(d, __dmul_rn(nimg, prd)); }
TMPS_DEV double rsq64(const double* d) {
    return __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
}

// a * b and a + b rounded as written (no multiply-add contraction), for sums
// whose rounding must not depend on where the compiler inlines them
TMPS_DEV float mul_rn(float a, float b) { return __fmul_rn(a, b); }
TMPS_DEV double mul_rn(double a, double b) { return __dmul_rn(a, b); }
TMPS_DEV float add_rn(float a, float b) { return __fadd_rn(a, b); }
TMPS_DEV double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
TMPS_DEV T dot3(const T* a, const T* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
template <typename T>
TMPS_DEV T norm3(const T* a) { return lsqrt(dot3(a, a)); }
template <typename T>
TMPS_DEV void cross3(const T* a, const T* b, T* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// Storage of a per-contact history component.  The FP64 form keeps it in a
// double; the mixed form keeps it as an FP32 double word (hi + lo, ~48 bits)
// so that its contact pass, which is otherwise all FP32, issues no FP64
// instruction for it: increments are added with an error-free two-sum,
// values the law computes in FP32 replace it outright (as a double would get
// the same FP32 value), and a read gives hi (hi + lo rounded to FP32).
struct DW {
    float hi, lo;
};

template <typename H>
struct Hist;

template <>
struct Hist<double> {
    template <typename T>
    TMPS_DEV static T get(double h) { return (T)h; }
    template <typename T>
    TMPS_DEV static void add(double& h, T v) { h = h + (double)v; }
    template <typename T>
    TMPS_DEV static void set(double& h, T v) { h = (double)v; }
    // h = ratio (h + dc) - dc, the legacy Coulomb rescale (hooke_history.py:183-187)
    template <typename T>
    TMPS_DEV static void rescale(double& h, T ratio, T dc) { h = (double)ratio * (h + (double)dc) - (double)dc; }
};

template <>
struct Hist<DW> {
    template <typename T>
    TMPS_DEV static T get(DW h) { return (T)h.hi; }
    template <typename T>
    TMPS_DEV static void add(DW& h, T v) {
        // two-sum of hi and v, the error and lo folded back (fast two-sum)
        const float a = h.hi, b = (float)v;
        const float s = a + b;
        const float bb = s - a;
        const float e = (a - (s - bb)) + (b - bb);
        const float t = e + h.lo;
        const float hi = s + t;
        h.lo = t - (hi - s);
        h.hi = hi;
    }
    template <typename T>
    TMPS_DEV static void set(DW& h, T v) {
        h.hi = (float)v;
        h.lo = 0.0f;
    }
    template <typename T>
    TMPS_DEV static void rescale(DW& h, T ratio, T dc) { set(h, (float)(ratio * (h.hi + dc) - dc)); }
};

template <typename T>
struct PairIn {
    T d[3];      // x_a - x_b, minimum image
    T rsq;
    T r;         // |d|
    T delta;     // overlap ra + rb - r (the caller may form it more accurately than T allows)
    T ra, rb, ma, mb;
    T va[3], vb[3];  // vb already shifted by the remap-v image velocity
    T wa[3], wb[3];
};

template <typename T>
struct PairOut {
    T f[3];      // force on a (b gets -f)
    T tor[3];    // torque term; a gets arm_a * tor, b gets arm_b * tor
    T arm_a, arm_b;
    T troll[3];  // rolling-resistance torque: a gets +troll, b gets -troll
};

// One contact (the caller has established rsq < (ra + rb)^2 and supplies r and
// the overlap).  `sh` and `rl` (canonical sense) are read and written only by
// history styles and by the rolling model; the caller passes zeros when the
// slot held no live contact (the reference's partner != jtag reset).
// The pair coefficients in FP32, for the mixed form's law: read from double
// fields, every coefficient of every contact would be an FP64 -> FP32
// conversion, which this part runs on its narrow FP64 pipe.  Same field names
// as tmps_pair_params, so the law reads either.
struct PairParams32 {
    int32_t style, normal_id, damping_id, tangential_id, limit_damping, rolling_id;
    float kn, kt, gamman, gammat, xmu, damp, xt, mu, k_roll, gamma_roll, mu_roll;
};

TMPS_DEV void params32(const tmps_pair_params& P, PairParams32& q) {
    q.style = P.style;
    q.normal_id = P.normal_id;
    q.damping_id = P.damping_id;
    q.tangential_id = P.tangential_id;
    q.limit_damping = P.limit_damping;
    q.rolling_id = P.rolling_id;
    q.kn = (float)P.kn; q.kt = (float)P.kt; q.gamman = (float)P.gamman; q.gammat = (float)P.gammat;
    q.xmu = (float)P.xmu; q.damp = (float)P.damp; q.xt = (float)P.xt; q.mu = (float)P.mu;
    q.k_roll = (float)P.k_roll; q.gamma_roll = (float)P.gamma_roll; q.mu_roll = (float)P.mu_roll;
}

template <typename T, int STYLE, typename H = double, typename PP = tmps_pair_params>
TMPS_DEV void contact_law(const PP& P, T dt, int shearupdate, const PairIn<T>& in,
                          H* sh, H* rl, PairOut<T>& out) {
    using HS = Hist<H>;
    using S = StyleTraits<STYLE>;
    out.troll[0] = out.troll[1] = out.troll[2] = T(0);
    if constexpr (S::legacy) {
        const T r = in.r;
        const T delta = in.delta;
        T polyhertz = T(1);
        if constexpr (S::hertz) {
            const T reff = ldiv(in.ra * in.rb, in.ra + in.rb);
            polyhertz = lsqrt(reff * delta);
        }
        const T meff = ldiv(in.ma * in.mb, in.ma + in.mb);
        const T rsqinv = ldiv(T(1), in.rsq);
        const T rinv = ldiv(T(1), r);
        T vrel_t[3], vt[3], wr[3], cr[3], vtr[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) vrel_t[k] = in.va[k] - in.vb[k];
        const T vnnr = dot3(vrel_t, in.d);
        const T s = vnnr * rsqinv;
#pragma unroll
        for (int k = 0; k < 3; ++k) vt[k] = vrel_t[k] - in.d[k] * s;
#pragma unroll
        for (int k = 0; k < 3; ++k) wr[k] = (in.ra * in.wa[k] + in.rb * in.wb[k]) * rinv;
        cross3(in.d, wr, cr);
#pragma unroll
        for (int k = 0; k < 3; ++k) vtr[k] = vt[k] + cr[k];
        const T damp = ((meff * T(P.gamman)) * vnnr) * rsqinv;
        T ccel = (T(P.kn) * delta) * rinv - damp;
        if constexpr (S::hertz) ccel = ccel * polyhertz;
        if (P.limit_damping == 1 && ccel < T(0)) ccel = T(0);
        T fs[3];
        if constexpr (!S::legacy_history) {
            const T vrel = norm3(vtr);
            const T fn = T(P.xmu) * fabs(ccel * r);
            const T fsd = (meff * T(P.gammat)) * vrel;
            T ft = T(0);
            if (vrel > T(1e-16)) ft = ldiv(fn < fsd ? fn : fsd, vrel);
#pragma unroll
            for (int k = 0; k < 3; ++k) fs[k] = (-ft) * vtr[k];
        } else {
            const T geff = meff * T(P.gammat);
            T shf[3];
            if (shearupdate) {
#pragma unroll
                for (int k = 0; k < 3; ++k) HS::add(sh[k], vtr[k] * dt);
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) shf[k] = HS::template get<T>(sh[k]);
            const T shrmag = norm3(shf);
            if (shearupdate) {
                const T rsht = dot3(shf, in.d) * rsqinv;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    HS::add(sh[k], -(rsht * in.d[k]));
                    shf[k] = HS::template get<T>(sh[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T t = T(P.kt) * shf[k] + geff * vtr[k];
                if constexpr (S::hertz) fs[k] = (-polyhertz) * t;
                else fs[k] = -t;
            }
            const T fsmag = norm3(fs);
            const T fn = T(P.xmu) * fabs(ccel * r);
            if (fsmag > fn) {
                if (shrmag != T(0)) {
                    const T ratio = ldiv(fn, fsmag);
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const T dc = ldiv(geff * vtr[k], T(P.kt));
                        HS::rescale(sh[k], ratio, dc);
                        fs[k] = ratio * fs[k];
                    }
                } else {
                    fs[0] = fs[1] = fs[2] = T(0);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) out.f[k] = in.d[k] * ccel + fs[k];
        T c[3];
        cross3(in.d, fs, c);
#pragma unroll
        for (int k = 0; k < 3; ++k) out.tor[k] = rinv * c[k];
        out.arm_a = -in.ra;
        out.arm_b = -in.rb;
    } else {
        const T r = in.r;
        const T rinv = ldiv(T(1), r);
        T nv[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) nv[k] = in.d[k] * rinv;
        const T delta = in.delta;
        const T reff = ldiv(in.ra * in.rb, in.ra + in.rb);
        const T meff = ldiv(in.ma * in.mb, in.ma + in.mb);
        const T a = lsqrt(delta * reff);
        T vr[3], vt[3], wr[3], cr[3], vtr[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) vr[k] = in.va[k] - in.vb[k];
        const T vnnr = dot3(vr, nv);
#pragma unroll
        for (int k = 0; k < 3; ++k) vt[k] = vr[k] - vnnr * nv[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) wr[k] = in.ra * in.wa[k] + in.rb * in.wb[k];
        cross3(wr, nv, cr);
#pragma unroll
        for (int k = 0; k < 3; ++k) vtr[k] = vt[k] - cr[k];
        const T vrel = norm3(vtr);
        const T fne = P.normal_id != 0 ? (T(P.kn) * a) * delta : T(P.kn) * delta;
        T dpf = T(0);
        switch (P.damping_id) {
            case 1: dpf = T(P.damp); break;
            case 2: dpf = T(P.damp) * meff; break;
            case 3: dpf = (T(P.damp) * meff) * a; break;
            case 4:
            case 5: {
                T arg = T(0);
                if (delta > T(0)) {
                    const T q = ldiv(meff * fne, delta);
                    arg = q > T(0) ? q : T(0);
                }
                dpf = T(P.damp) * lsqrt(arg);
                break;
            }
            default: break;
        }
        T fntot = fne - dpf * vnnr;
        if (P.limit_damping == 1 && fntot < T(0)) fntot = T(0);
        const T fscrit = T(P.mu) * fabs(fntot);
        T fs[3] = {T(0), T(0), T(0)};
        if (P.tangential_id == 1) {
            const T damp_t = T(P.xt) * dpf;
            T ft = T(0);
            if (vrel != T(0)) {
                const T q = damp_t * vrel;
                ft = ldiv(fscrit < q ? fscrit : q, vrel);
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) fs[k] = (-ft) * vtr[k];
        } else if (P.tangential_id == 2 || P.tangential_id == 3) {
            T keff = T(P.kt);
            if (P.tangential_id == 3) keff = T(P.kt) * a;
            const T damp_t = T(P.xt) * dpf;
            T hf[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) hf[k] = HS::template get<T>(sh[k]);
            if (shearupdate) {
                const T rsht = dot3(hf, nv);
                if (fabs(rsht) * keff > T(1e-10) * fscrit) {
                    // rotate_rescale: project onto the tangent plane, keep |h|
                    const T shrmag = norm3(hf);
                    T o[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) o[k] = hf[k] - rsht * nv[k];
                    const T prjmag = norm3(o);
                    T scale = T(0);
                    if (prjmag > T(0)) scale = ldiv(shrmag, prjmag);
#pragma unroll
                    for (int k = 0; k < 3; ++k) HS::set(sh[k], o[k] * scale);
                }
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    HS::add(sh[k], vtr[k] * dt);
                    hf[k] = HS::template get<T>(sh[k]);
                }
            }
            T fdamp[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) fdamp[k] = (-damp_t) * vtr[k];
#pragma unroll
            for (int k = 0; k < 3; ++k) fs[k] = (-keff) * hf[k] + fdamp[k];
            const T magfs = norm3(fs);
            if (magfs > fscrit) {
                if (norm3(hf) != T(0)) {
                    const T sc = ldiv(fscrit, magfs);
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        fs[k] = fs[k] * sc;
                        HS::set(sh[k], ldiv(-(fs[k] - fdamp[k]), keff));
                    }
                } else {
                    fs[0] = fs[1] = fs[2] = T(0);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) out.f[k] = fntot * nv[k] + fs[k];
        T c[3];
        cross3(nv, fs, c);
#pragma unroll
        for (int k = 0; k < 3; ++k) out.tor[k] = -c[k];
        out.arm_a = in.ra - T(0.5) * delta;
        out.arm_b = in.rb - T(0.5) * delta;
        if (P.rolling_id == 1) {
            // RollingResistance.compute_torque (rolling.py:30-50), as the reference writes
            // it: omega_rel = omega_a - omega_b, r_eff, fn = |fntot|; the history (FP64,
            // like the shear) advances only on a history update
            T wrel[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) wrel[k] = in.wa[k] - in.wb[k];
            if (shearupdate) {
#pragma unroll
                for (int k = 0; k < 3; ++k) HS::add(rl[k], wrel[k] * dt);
            }
            T h[3] = {HS::template get<T>(rl[0]), HS::template get<T>(rl[1]), HS::template get<T>(rl[2])};
            const T tr_mag = T(P.k_roll) * norm3(h);
            const T tr_max = (T(P.mu_roll) * reff) * fabs(fntot);
#pragma unroll
            for (int k = 0; k < 3; ++k) out.troll[k] = (-T(P.k_roll)) * h[k] - T(P.gamma_roll) * wrel[k];
            if (tr_mag > tr_max && tr_mag > T(1e-12)) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    out.troll[k] = (-tr_max) * ldiv(h[k], tr_mag);
                    HS::set(rl[k], ldiv(tr_max, T(P.k_roll)) * ldiv(h[k], tr_mag));
                }
            }
        }
    }
}

}  // namespace tmps
