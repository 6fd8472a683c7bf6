// The cross-axis part of the deform/pressure update, shared by the per-hook
// servo kernel and the fused step's S: the volume style, the box style and
// the bookkeeping vol/balance/p reads on the next step.  One thread runs it,
// after the per-axis strain and pressure targets are known, and only when
// tmps_servo.post is set.  FixDeformPressure.end_of_step host path
// (deform_pressure.py:1113-1219): _apply_volume (:872-903),
// _balanced_volume_half (:905-956), _adjust_linked_rates (:858-870),
// _apply_box (:958-991), every expression in the reference's order.
#pragma once

#include "../../include/taichimps_gb300.h"

namespace tmps {

// _limit_rate (deform_pressure.py:737-752) without the host-side error (the
// zero-target + normalize case without max/rate is rejected at setup)
__device__ __forceinline__ double servo_limit(const tmps_servo& sv, double rate, double ptarget) {
    double out = rate;
    if (sv.normalize) {
        if (ptarget == 0.0) {
            if (out != 0.0) out = copysign(sv.max_rate, out);
        } else {
            out = out / fabs(ptarget);
        }
    }
    if (sv.max_rate != 0.0 && fabs(out) > sv.max_rate) out = copysign(sv.max_rate, out);
    return out;
}

// _adjust_linked_rates: a volume-preserving pair of strain rates rescaled to
// honour max/rate; returns (first, second) in *a, *b.
__device__ __forceinline__ void servo_adjust_linked(double m, double e_larger, double e3, double vi, double v,
                                                     double dt, double* a, double* b) {
    const double e_lim_pos = (vi - v * (1 + m * dt)) / (v * (1 + m * dt) * dt);
    const double e_lim_neg = (vi - v * (1 - m * dt)) / (v * (1 - m * dt) * dt);
    if (e_larger * e3 >= 0) {
        if (e_larger > 0.0) {
            *a = e_lim_neg;
            *b = -m;
        } else {
            *a = e_lim_pos;
            *b = m;
        }
    } else if (e_larger > 0.0) {
        *a = m;
        *b = e_lim_pos;
    } else {
        *a = -m;
        *b = e_lim_neg;
    }
}

// nlo/nhi: targets after the per-axis updates (in and out); prd: the box
// before this update; t: this step's pressure tensor.
__device__ inline void servo_post(tmps_servo& sv, const double* prd, const double* t, double dt, double* nlo,
                                  double* nhi) {
    bool needs_p = sv.box_style == 2 || sv.vol_balance_p;
    for (int d = 0; d < 3; ++d) needs_p = needs_p || sv.style[d] == 8 || sv.style[d] == 9;
    if (needs_p && !sv.saved) {
        for (int d = 0; d < 3; ++d) {
            sv.prior_rate[d] = 0.0;
            sv.prior_pressure[d] = t[d];
        }
        sv.saved = 1;
    }
    // _apply_volume
    bool linked_done = false;
    double e2_linked = 0.0;
    for (int i = 0; i < 3; ++i) {
        if (sv.style[i] != 10) continue;
        const double v0 = sv.vol_start;
        const int d1 = sv.vdyn1[i], fx = sv.vfixed[i], d2 = sv.vdyn2[i];
        double half;
        if (sv.vsub[i] == 0) {
            half = 0.5 * (v0 / (nhi[d1] - nlo[d1]) / (sv.hi_start[fx] - sv.lo_start[fx]));
        } else if (sv.vsub[i] == 1) {
            half = 0.5 * (v0 / (nhi[d1] - nlo[d1]) / (nhi[d2] - nlo[d2]));
        } else if (!sv.vol_balance_p) {
            half = 0.5 * sqrt(v0 * (sv.hi_start[i] - sv.lo_start[i]) / (nhi[d1] - nlo[d1]) /
                              (sv.hi_start[fx] - sv.lo_start[fx]));
        } else {
            // _balanced_volume_half
            const double l1i = prd[i], l2i = prd[fx], l3i = prd[d1];
            const double l3 = nhi[d1] - nlo[d1];
            const double vi = l1i * l2i * l3i;
            const double v = l3 * l1i * l2i;
            const double e3 = (l3 / l3i - 1.0) / dt;
            const double e1i = sv.prior_rate[i], e2i = sv.prior_rate[fx];
            const double p1 = t[i], p2 = t[fx];
            const double p1i = sv.prior_pressure[i], p2i = sv.prior_pressure[fx];
            if (e3 == 0.0) {
                half = 0.5 * l1i;
            } else if (e1i == 0.0 || e2i == 0.0 || (p2 == p2i && p1 == p1i)) {
                half = 0.5 * sqrt(sv.vol_start * l1i / l3 / l2i);
            } else if (linked_done) {
                half = 0.5 * l1i * (1.0 + e2_linked * dt);
            } else {
                const double denominator = p2 - p2i + e2i * ((p1 - p1i) / e1i);
                double e1 = denominator != 0.0
                                ? (((p2 - p2i) * (vi - v) / (v * dt)) - e2i * (p1 - p2)) / denominator
                                : e2i;
                double e2 = (vi - v * (1 + e1 * dt)) / (v * (1 + e1 * dt) * dt);
                if (sv.max_rate != 0.0 && (fabs(e1) > sv.max_rate || fabs(e2) > sv.max_rate)) {
                    if (fabs(e1) > fabs(e2)) servo_adjust_linked(sv.max_rate, e1, e3, vi, v, dt, &e1, &e2);
                    else servo_adjust_linked(sv.max_rate, e2, e3, vi, v, dt, &e2, &e1);
                }
                half = 0.5 * l1i * (1.0 + e1 * dt);
                linked_done = true;
                e2_linked = e2;
            }
        }
        const double mid = 0.5 * (sv.lo_start[i] + sv.hi_start[i]);
        nlo[i] = mid - half;
        nhi[i] = mid + half;
    }
    // _apply_box
    if (sv.box_style == 1) {
        double v = 1.0;
        for (int i = 0; i < 3; ++i) v *= nhi[i] - nlo[i];
        const double scale = pow(sv.vol_start / v, 1.0 / 3.0);
        for (int i = 0; i < 3; ++i) {
            const double half = 0.5 * (nhi[i] - nlo[i]) * scale;
            const double mid = 0.5 * (sv.lo_start[i] + sv.hi_start[i]);
            nlo[i] = mid - half;
            nhi[i] = mid + half;
        }
    } else if (sv.box_style == 2) {
        const double mean = ((t[0] + t[1]) + t[2]) / 3.0;
        const double v_rate = servo_limit(sv, sv.box_pgain * (mean - sv.box_ptarget), sv.box_ptarget);
        for (int i = 0; i < 3; ++i) {
            const double shift = (nhi[i] - nlo[i]) * dt * v_rate;
            sv.box_vshift[i] += shift;
            if (sv.style[i] == 0) {
                nlo[i] = sv.lo_start[i];
                nhi[i] = sv.hi_start[i];
            }
            nlo[i] -= 0.5 * sv.box_vshift[i];
            nhi[i] += 0.5 * sv.box_vshift[i];
        }
    }
    // this step's response for the next vol/balance/p update
    if (needs_p)
        for (int i = 0; i < 3; ++i) {
            sv.prior_pressure[i] = t[i];
            sv.prior_rate[i] = ((nhi[i] - nlo[i]) / prd[i] - 1.0) / dt;
        }
}

}  // namespace tmps
