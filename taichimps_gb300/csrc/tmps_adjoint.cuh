// One contact of gran/hertz/history in FP64 and its hand-written reverse
// (vector-Jacobian product), for the differentiable run.
//
// The forward is GranHertzHistory.compute_kernel (GRANULAR/hertz_history.py:92-157)
// term for term, in the evaluation order of the fused step's contact law:
//
//   r = |d|, delta = ra + rb - r, reff = ra rb / (ra + rb), meff = ma mb / (ma + mb)
//   ph = sqrt(reff delta)
//   vrel = va - vb, vnnr = vrel . d, vt = vrel - d (vnnr / r^2)
//   wr = (ra wa + rb wb) / r, vtr = vt + d x wr
//   ccel = (kn delta / r - meff gamman vnnr / r^2) ph        (0 if clamped by limit_damping)
//   sh1 = sh + vtr dt; sh2 = sh1 - ((sh1 . d) / r^2) d      (shearupdate only)
//   fs0 = -ph (kt sh2 + meff gammat vtr)
//   Coulomb: |fs0| > xmu |ccel r|: fs = ratio fs0, sh3 = ratio (sh2 + dc) - dc
//            (dc = meff gammat vtr / kt); fs = 0 when |sh1| == 0
//   F = d ccel + fs (on a; b gets -F), tor = (d x fs) / r (a gets -ra tor, b -rb tor)
//   virial d (x) F over [xx, yy, zz, xy, xz, yz]
//
// The reverse follows the recorded branch mask, so a replay takes the
// forward's branches exactly (no smoothing of the Coulomb cap or of the
// contact switch).  Everything here is plain scalar code: it compiles for the
// device and for the host (the CPU unit test checks it against autograd).
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define TMPS_HD __host__ __device__ __forceinline__
#else
#define TMPS_HD inline
#endif

namespace tmps_adj {

enum { M_CONTACT = 1, M_SLIP = 2, M_SHRMAG = 4, M_CLAMP = 8 };

struct Params {
    double kn, kt, gamman, gammat, xmu, dt;
    int limit_damping;
};

struct PairIn {
    double d[3];  // x_a - x_b after the minimum image
    double ra, rb, ma, mb;
    double va[3], vb[3], wa[3], wb[3];
    double sh[3];  // history entering the pass (a -> b sense)
};

struct PairOut {
    double F[3];    // force on a
    double tor[3];  // (d x fs) / r
    double sh[3];   // history leaving the pass
};

// Forward intermediates the reverse reads.
struct PairTape {
    double rsq, r, delta, reff, ph, meff, rsqinv, rinv;
    double vrel[3], vnnr, s, g[3], wr[3], vtr[3];
    double ccel0, ccel, geff;
    double sh1[3], rsht, sh2[3], t[3], fs0[3], fsmag, u, fn, ratio, dc[3];
    double fs[3], c[3];
};

// Adjoints arriving at one contact.
struct PairBar {
    double fa[3], fb[3];  // dL/d(force of a), dL/d(force of b)
    double ta[3], tb[3];  // dL/d(torque of a), dL/d(torque of b)
    double w[6];          // dL/d(virial total)
    double sh[3];         // dL/d(history leaving the pass)
};

// Adjoints leaving it.
struct PairGrad {
    double d[3], vrel[3], wa[3], wb[3];
    double ra, rb, ma, mb;
    double sh[3];
    double kn, kt, gamman, gammat, xmu;
};

TMPS_HD double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
TMPS_HD void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// `forced` < 0: branches from the values (and returned in *mask); otherwise
// the branches of that recorded mask.
TMPS_HD void pair_forward(const Params& P, int shearupdate, const PairIn& in, int forced, PairOut& o, PairTape& t,
                          int* mask) {
    const double* d = in.d;
    int m = 0;
    t.rsq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
    const double radsum = in.ra + in.rb;
    const bool contact = forced >= 0 ? (forced & M_CONTACT) != 0 : (t.rsq < radsum * radsum && t.rsq > 1e-28);
    if (!contact) {
        for (int k = 0; k < 3; ++k) o.F[k] = o.tor[k] = o.sh[k] = 0.0;
        *mask = 0;
        return;
    }
    m |= M_CONTACT;
    t.r = sqrt(t.rsq);
    t.delta = radsum - t.r;
    t.reff = (in.ra * in.rb) / (in.ra + in.rb);
    t.ph = sqrt(t.reff * t.delta);
    t.meff = (in.ma * in.mb) / (in.ma + in.mb);
    t.rsqinv = 1.0 / t.rsq;
    t.rinv = 1.0 / t.r;
    for (int k = 0; k < 3; ++k) t.vrel[k] = in.va[k] - in.vb[k];
    t.vnnr = dot3(t.vrel, d);
    t.s = t.vnnr * t.rsqinv;
    double cr[3];
    for (int k = 0; k < 3; ++k) {
        t.g[k] = in.ra * in.wa[k] + in.rb * in.wb[k];
        t.wr[k] = t.g[k] * t.rinv;
    }
    cross3(d, t.wr, cr);
    for (int k = 0; k < 3; ++k) t.vtr[k] = (t.vrel[k] - d[k] * t.s) + cr[k];
    const double damp = ((t.meff * P.gamman) * t.vnnr) * t.rsqinv;
    t.ccel0 = (P.kn * t.delta) * t.rinv - damp;
    t.ccel = t.ccel0 * t.ph;
    const bool clamp = forced >= 0 ? (forced & M_CLAMP) != 0 : (P.limit_damping == 1 && t.ccel < 0.0);
    if (clamp) {
        m |= M_CLAMP;
        t.ccel = 0.0;
    }
    t.geff = t.meff * P.gammat;
    for (int k = 0; k < 3; ++k) t.sh1[k] = shearupdate ? in.sh[k] + t.vtr[k] * P.dt : in.sh[k];
    const double shrmag = sqrt(dot3(t.sh1, t.sh1));
    const bool shnz = forced >= 0 ? (forced & M_SHRMAG) != 0 : shrmag != 0.0;
    if (shnz) m |= M_SHRMAG;
    if (shearupdate) {
        t.rsht = dot3(t.sh1, d) * t.rsqinv;
        for (int k = 0; k < 3; ++k) t.sh2[k] = t.sh1[k] - t.rsht * d[k];
    } else {
        t.rsht = 0.0;
        for (int k = 0; k < 3; ++k) t.sh2[k] = t.sh1[k];
    }
    for (int k = 0; k < 3; ++k) {
        t.t[k] = P.kt * t.sh2[k] + t.geff * t.vtr[k];
        t.fs0[k] = (-t.ph) * t.t[k];
    }
    t.fsmag = sqrt(dot3(t.fs0, t.fs0));
    t.u = t.ccel * t.r;
    t.fn = P.xmu * fabs(t.u);
    t.ratio = 1.0;
    for (int k = 0; k < 3; ++k) t.dc[k] = 0.0;
    const bool slip = forced >= 0 ? (forced & M_SLIP) != 0 : t.fsmag > t.fn;
    if (slip) {
        m |= M_SLIP;
        if (shnz) {
            t.ratio = t.fn / t.fsmag;
            for (int k = 0; k < 3; ++k) {
                t.dc[k] = (t.geff * t.vtr[k]) / P.kt;
                o.sh[k] = t.ratio * (t.sh2[k] + t.dc[k]) - t.dc[k];
                t.fs[k] = t.ratio * t.fs0[k];
            }
        } else {
            for (int k = 0; k < 3; ++k) {
                o.sh[k] = t.sh2[k];
                t.fs[k] = 0.0;
            }
        }
    } else {
        for (int k = 0; k < 3; ++k) {
            o.sh[k] = t.sh2[k];
            t.fs[k] = t.fs0[k];
        }
    }
    for (int k = 0; k < 3; ++k) o.F[k] = d[k] * t.ccel + t.fs[k];
    cross3(d, t.fs, t.c);
    for (int k = 0; k < 3; ++k) o.tor[k] = t.rinv * t.c[k];
    *mask = m;
}

// Reverse of pair_forward under `mask` (the forward's own), from its tape.
TMPS_HD void pair_reverse(const Params& P, int shearupdate, int mask, const PairIn& in, const PairOut& o,
                          const PairTape& t, const PairBar& b, PairGrad& g) {
    for (int k = 0; k < 3; ++k) g.d[k] = g.vrel[k] = g.wa[k] = g.wb[k] = g.sh[k] = 0.0;
    g.ra = g.rb = g.ma = g.mb = 0.0;
    g.kn = g.kt = g.gamman = g.gammat = g.xmu = 0.0;
    if (!(mask & M_CONTACT)) return;  // F = 0, tor = 0, history reset: nothing depends on the inputs
    const double* d = in.d;
    double Fb[3], db[3], fsb[3], torb[3], cb[3], tmp[3];
    double rinvb = 0.0, rsqinvb = 0.0, rbar = 0.0, rsqb = 0.0, ccelb = 0.0, phb = 0.0, deltab = 0.0;
    double meffb = 0.0, geffb = 0.0, reffb = 0.0;
    double vtrb[3] = {0.0, 0.0, 0.0}, sh2b[3], fs0b[3], vrelb[3];
    for (int k = 0; k < 3; ++k) Fb[k] = b.fa[k] - b.fb[k];
    // virial total d (x) F
    Fb[0] += b.w[0] * d[0];
    Fb[1] += b.w[1] * d[1] + b.w[3] * d[0];
    Fb[2] += b.w[2] * d[2] + b.w[4] * d[0] + b.w[5] * d[1];
    db[0] = b.w[0] * o.F[0] + b.w[3] * o.F[1] + b.w[4] * o.F[2];
    db[1] = b.w[1] * o.F[1] + b.w[5] * o.F[2];
    db[2] = b.w[2] * o.F[2];
    // torques -ra tor, -rb tor
    for (int k = 0; k < 3; ++k) torb[k] = -in.ra * b.ta[k] - in.rb * b.tb[k];
    g.ra -= dot3(b.ta, o.tor);
    g.rb -= dot3(b.tb, o.tor);
    // tor = rinv c, c = d x fs
    for (int k = 0; k < 3; ++k) cb[k] = t.rinv * torb[k];
    rinvb += dot3(torb, t.c);
    cross3(t.fs, cb, tmp);
    for (int k = 0; k < 3; ++k) db[k] += tmp[k];
    cross3(cb, d, fsb);
    // F = d ccel + fs
    for (int k = 0; k < 3; ++k) {
        db[k] += t.ccel * Fb[k];
        fsb[k] += Fb[k];
    }
    ccelb += dot3(Fb, d);
    // Coulomb cap
    double fnb = 0.0, fsmagb = 0.0;
    if (mask & M_SLIP) {
        if (mask & M_SHRMAG) {
            double ratiob = dot3(fsb, t.fs0);
            double dcb[3];
            for (int k = 0; k < 3; ++k) {
                ratiob += b.sh[k] * (t.sh2[k] + t.dc[k]);
                fs0b[k] = t.ratio * fsb[k];
                sh2b[k] = t.ratio * b.sh[k];
                dcb[k] = (t.ratio - 1.0) * b.sh[k];
            }
            // dc = geff vtr / kt
            for (int k = 0; k < 3; ++k) {
                geffb += dcb[k] * t.vtr[k] / P.kt;
                vtrb[k] += t.geff * dcb[k] / P.kt;
            }
            g.kt -= dot3(dcb, t.dc) / P.kt;
            // ratio = fn / fsmag
            fnb += ratiob / t.fsmag;
            fsmagb -= ratiob * t.ratio / t.fsmag;
        } else {
            for (int k = 0; k < 3; ++k) {
                fs0b[k] = 0.0;
                sh2b[k] = b.sh[k];
            }
        }
    } else {
        for (int k = 0; k < 3; ++k) {
            fs0b[k] = fsb[k];
            sh2b[k] = b.sh[k];
        }
    }
    // fn = xmu |u|, u = ccel r
    g.xmu += fnb * fabs(t.u);
    const double ub = fnb * P.xmu * (t.u > 0.0 ? 1.0 : (t.u < 0.0 ? -1.0 : 0.0));
    ccelb += ub * t.r;
    rbar += ub * t.ccel;
    // fsmag = |fs0|
    if (t.fsmag > 0.0)
        for (int k = 0; k < 3; ++k) fs0b[k] += fsmagb * t.fs0[k] / t.fsmag;
    // fs0 = -ph t, t = kt sh2 + geff vtr
    for (int k = 0; k < 3; ++k) {
        phb -= fs0b[k] * t.t[k];
        const double tb = -t.ph * fs0b[k];
        g.kt += tb * t.sh2[k];
        sh2b[k] += P.kt * tb;
        geffb += tb * t.vtr[k];
        vtrb[k] += t.geff * tb;
    }
    // history: sh2 = sh1 - rsht d, rsht = (sh1 . d) rsqinv, sh1 = sh + vtr dt
    if (shearupdate) {
        const double rshtb = -dot3(sh2b, d);
        const double sd = dot3(t.sh1, d);
        for (int k = 0; k < 3; ++k) {
            db[k] -= t.rsht * sh2b[k];
            const double sh1b = sh2b[k] + rshtb * t.rsqinv * d[k];
            db[k] += rshtb * t.rsqinv * t.sh1[k];
            g.sh[k] = sh1b;
            vtrb[k] += P.dt * sh1b;
        }
        rsqinvb += rshtb * sd;
    } else {
        for (int k = 0; k < 3; ++k) g.sh[k] = sh2b[k];
    }
    // geff = meff gammat
    meffb += geffb * P.gammat;
    g.gammat += geffb * t.meff;
    // ccel = ccel0 ph (0 when clamped)
    if (mask & M_CLAMP) ccelb = 0.0;
    const double ccel0b = ccelb * t.ph;
    phb += ccelb * t.ccel0;
    // ccel0 = kn delta rinv - damp, damp = meff gamman vnnr rsqinv
    g.kn += ccel0b * t.delta * t.rinv;
    deltab += ccel0b * P.kn * t.rinv;
    rinvb += ccel0b * P.kn * t.delta;
    const double dampb = -ccel0b;
    meffb += dampb * P.gamman * t.vnnr * t.rsqinv;
    g.gamman += dampb * t.meff * t.vnnr * t.rsqinv;
    double vnnrb = dampb * t.meff * P.gamman * t.rsqinv;
    rsqinvb += dampb * t.meff * P.gamman * t.vnnr;
    // vtr = (vrel - d s) + d x wr
    double wrb[3];
    cross3(t.wr, vtrb, tmp);
    for (int k = 0; k < 3; ++k) db[k] += tmp[k];
    cross3(vtrb, d, wrb);
    // wr = g rinv, g = ra wa + rb wb
    rinvb += dot3(wrb, t.g);
    for (int k = 0; k < 3; ++k) {
        const double gb = wrb[k] * t.rinv;
        g.ra += gb * in.wa[k];
        g.rb += gb * in.wb[k];
        g.wa[k] = in.ra * gb;
        g.wb[k] = in.rb * gb;
    }
    const double sb = -dot3(vtrb, d);
    for (int k = 0; k < 3; ++k) {
        vrelb[k] = vtrb[k];
        db[k] -= t.s * vtrb[k];
    }
    // s = vnnr rsqinv, vnnr = vrel . d
    vnnrb += sb * t.rsqinv;
    rsqinvb += sb * t.vnnr;
    for (int k = 0; k < 3; ++k) {
        vrelb[k] += vnnrb * d[k];
        db[k] += vnnrb * t.vrel[k];
        g.vrel[k] = vrelb[k];
    }
    // rinv = 1 / r, rsqinv = 1 / rsq
    rbar -= rinvb * t.rinv * t.rinv;
    rsqb -= rsqinvb * t.rsqinv * t.rsqinv;
    // meff = ma mb / (ma + mb)
    const double ms = in.ma + in.mb;
    g.ma += meffb * in.mb * in.mb / (ms * ms);
    g.mb += meffb * in.ma * in.ma / (ms * ms);
    // ph = sqrt(reff delta)
    if (t.ph > 0.0) {
        const double u2 = phb / (2.0 * t.ph);
        reffb += u2 * t.delta;
        deltab += u2 * t.reff;
    }
    // reff = ra rb / (ra + rb)
    const double rs = in.ra + in.rb;
    g.ra += reffb * in.rb * in.rb / (rs * rs);
    g.rb += reffb * in.ra * in.ra / (rs * rs);
    // delta = ra + rb - r
    g.ra += deltab;
    g.rb += deltab;
    rbar -= deltab;
    // r = sqrt(rsq), rsq = d . d
    rsqb += rbar / (2.0 * t.r);
    for (int k = 0; k < 3; ++k) g.d[k] = db[k] + 2.0 * rsqb * d[k];
}

}  // namespace tmps_adj
