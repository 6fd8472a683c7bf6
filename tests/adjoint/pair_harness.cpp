// Test harness: the differentiable run's per-contact forward and reverse
// (taichimps_gb300/csrc/tmps_adjoint.cuh) compiled for the host, so the CPU
// tests can check the hand-written reverse against autograd.  Not part of the
// library.
#include "../../taichimps_gb300/csrc/tmps_adjoint.cuh"

using namespace tmps_adj;

namespace {
Params params_of(const double* p) {
    Params q;
    q.kn = p[0];
    q.kt = p[1];
    q.gamman = p[2];
    q.gammat = p[3];
    q.xmu = p[4];
    q.dt = p[5];
    q.limit_damping = (int)p[6];
    return q;
}
// in: d[3] ra rb ma mb va[3] vb[3] wa[3] wb[3] sh[3]  (22)
PairIn in_of(const double* a) {
    PairIn in;
    for (int k = 0; k < 3; ++k) in.d[k] = a[k];
    in.ra = a[3];
    in.rb = a[4];
    in.ma = a[5];
    in.mb = a[6];
    for (int k = 0; k < 3; ++k) {
        in.va[k] = a[7 + k];
        in.vb[k] = a[10 + k];
        in.wa[k] = a[13 + k];
        in.wb[k] = a[16 + k];
        in.sh[k] = a[19 + k];
    }
    return in;
}
}  // namespace

extern "C" {

// out: F[3] tor[3] sh[3]
int harness_pair_forward(const double* p, int shearupdate, const double* a, double* out) {
    PairIn in = in_of(a);
    PairOut o;
    PairTape t;
    int mask;
    pair_forward(params_of(p), shearupdate, in, -1, o, t, &mask);
    for (int k = 0; k < 3; ++k) {
        out[k] = o.F[k];
        out[3 + k] = o.tor[k];
        out[6 + k] = o.sh[k];
    }
    return mask;
}

// bar: fa[3] fb[3] ta[3] tb[3] w[6] sh[3]  (21)
// grad: d[3] vrel[3] wa[3] wb[3] ra rb ma mb sh[3] kn kt gamman gammat xmu  (24)
int harness_pair_reverse(const double* p, int shearupdate, const double* a, const double* bar, double* grad) {
    const Params P = params_of(p);
    PairIn in = in_of(a);
    PairOut o;
    PairTape t;
    int mask;
    pair_forward(P, shearupdate, in, -1, o, t, &mask);
    PairBar b;
    for (int k = 0; k < 3; ++k) {
        b.fa[k] = bar[k];
        b.fb[k] = bar[3 + k];
        b.ta[k] = bar[6 + k];
        b.tb[k] = bar[9 + k];
        b.sh[k] = bar[18 + k];
    }
    for (int k = 0; k < 6; ++k) b.w[k] = bar[12 + k];
    PairGrad g;
    pair_reverse(P, shearupdate, mask, in, o, t, b, g);
    for (int k = 0; k < 3; ++k) {
        grad[k] = g.d[k];
        grad[3 + k] = g.vrel[k];
        grad[6 + k] = g.wa[k];
        grad[9 + k] = g.wb[k];
        grad[16 + k] = g.sh[k];
    }
    grad[12] = g.ra;
    grad[13] = g.rb;
    grad[14] = g.ma;
    grad[15] = g.mb;
    grad[19] = g.kn;
    grad[20] = g.kt;
    grad[21] = g.gamman;
    grad[22] = g.gammat;
    grad[23] = g.xmu;
    return mask;
}

}  // extern "C"
