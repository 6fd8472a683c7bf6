"""
Plain PyTorch (autograd) restatement of the differentiable run, FP64, for the
tests: the reference the hand-written adjoint is compared with.

torch_pair: one gran/hertz/history contact per row (GRANULAR/hertz_history.py:92-157),
            branches from the values, every branch's unused side kept finite so
            that autograd sees no NaN.
torch_run:  the whole run on a fixed pair list -- setup force evaluation, then
            per step nve/sphere (nve_sphere.py:56-80), contacts, second half-kick,
            pressure, servo and remap x (deform_pressure.py:493-530, 583-702) --
            returning the deviatoric stress of every step.
"""

from __future__ import annotations

import math

import torch


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def torch_pair(P: dict, shearupdate: bool, d, ra, rb, ma, mb, va, vb, wa, wb, sh):
    """Rows of contacts; returns (F, tor, sh_out, mask)."""
    rsq = _dot(d, d)
    radsum = ra + rb
    c = (rsq < radsum * radsum) & (rsq > 1e-28)
    one = torch.ones_like(rsq)
    rsq_s = torch.where(c, rsq, one)
    r = torch.sqrt(rsq_s)
    delta = torch.where(c, radsum - r, one)
    reff = (ra * rb) / (ra + rb)
    ph = torch.sqrt(reff * delta)
    meff = (ma * mb) / (ma + mb)
    rsqinv = 1.0 / rsq_s
    rinv = 1.0 / r
    vrel = va - vb
    vnnr = _dot(vrel, d)
    s = vnnr * rsqinv
    wr = (ra[:, None] * wa + rb[:, None] * wb) * rinv[:, None]
    vtr = (vrel - d * s[:, None]) + torch.cross(d, wr, dim=-1)
    damp = ((meff * P["gamman"]) * vnnr) * rsqinv
    ccel = ((P["kn"] * delta) * rinv - damp) * ph
    clamp = torch.zeros_like(c)
    if P.get("limit_damping", 0) == 1:
        clamp = ccel < 0
        ccel = torch.where(clamp, torch.zeros_like(ccel), ccel)
    geff = meff * P["gammat"]
    sh1 = sh + vtr * P["dt"] if shearupdate else sh
    shrmag = torch.sqrt(_dot(sh1, sh1)).detach()
    if shearupdate:
        rsht = _dot(sh1, d) * rsqinv
        sh2 = sh1 - rsht[:, None] * d
    else:
        sh2 = sh1
    t = P["kt"] * sh2 + geff[:, None] * vtr
    fs0 = (-ph)[:, None] * t
    q = _dot(fs0, fs0)
    qpos = q > 0
    fsmag = torch.where(qpos, torch.sqrt(torch.where(qpos, q, one)), torch.zeros_like(q))
    u = ccel * r
    fn = P["xmu"] * torch.abs(u)
    slip = fsmag > fn
    shnz = shrmag != 0
    ratio = fn / torch.where(slip & shnz, fsmag, one)
    dc = (geff[:, None] * vtr) / P["kt"]
    sh_slip = ratio[:, None] * (sh2 + dc) - dc
    fs = torch.where((slip & shnz)[:, None], ratio[:, None] * fs0,
                     torch.where(slip[:, None], torch.zeros_like(fs0), fs0))
    sh_out = torch.where((slip & shnz)[:, None], sh_slip, sh2)
    F = d * ccel[:, None] + fs
    tor = rinv[:, None] * torch.cross(d, fs, dim=-1)
    z = torch.zeros_like(F)
    cc = c[:, None]
    mask = (c.int() | ((c & slip).int() << 1) | ((c & shnz).int() << 2) | ((c & clamp).int() << 3))
    return torch.where(cc, F, z), torch.where(cc, tor, z), torch.where(cc, sh_out, z), mask


def _min_image(d, prd):
    return d - torch.round(d / prd) * prd


def torch_run(P: dict, servo: dict, x0, v0, w0, radius, density, pi, pj, lo0, prd0, steps: int):
    """Deviatoric stress q of steps 1..steps (tensor [steps]).  `servo`: per-axis
    style ('none' | 'erate' | 'pressure'), rate, ptarget, pgain, couple ('none' |
    'xy' | 'xyz'), max_rate.  Every tensor may require grad (radius, and the
    scalars in P)."""
    dt = P["dt"]
    dtf = 0.5 * dt
    m = ((4.0 / 3.0) * math.pi * radius ** 3) * density
    inertia = ((0.4 * m) * radius) * radius
    lo = lo0.clone()
    prd = prd0.clone()
    lo_s, hi_s = lo0.clone(), lo0 + prd0
    cum = torch.zeros(3, dtype=torch.float64, device=x0.device)
    npair = pi.numel()
    sh = torch.zeros((npair, 3), dtype=torch.float64, device=x0.device)

    def forces(x, v, w, sh, prd, shearupdate):
        d = _min_image(x[pi] - x[pj], prd)
        F, tor, sh_out, _ = torch_pair(P, shearupdate, d, radius[pi], radius[pj], m[pi], m[pj], v[pi], v[pj],
                                       w[pi], w[pj], sh)
        f = torch.zeros_like(x).index_add(0, pi, F).index_add(0, pj, -F)
        t = (torch.zeros_like(x).index_add(0, pi, -radius[pi][:, None] * tor)
             .index_add(0, pj, -radius[pj][:, None] * tor))
        vir = torch.stack([(d[:, 0] * F[:, 0]).sum(), (d[:, 1] * F[:, 1]).sum(), (d[:, 2] * F[:, 2]).sum(),
                           (d[:, 0] * F[:, 1]).sum(), (d[:, 0] * F[:, 2]).sum(), (d[:, 1] * F[:, 2]).sum()])
        return f, t, sh_out, vir

    x, v, w = x0, v0, w0
    f, t, sh, _ = forces(x, v, w, sh, prd, False)
    qs = []
    for s in range(1, steps + 1):
        v = v + dtf * (f / m[:, None])
        x = x + dt * v
        w = w + dtf * (t / inertia[:, None])
        f, t, sh, vir = forces(x, v, w, sh, prd, True)
        v = v + dtf * (f / m[:, None])
        w = w + dtf * (t / inertia[:, None])
        kin = torch.stack([(m * v[:, 0] * v[:, 0]).sum(), (m * v[:, 1] * v[:, 1]).sum(), (m * v[:, 2] * v[:, 2]).sum(),
                           (m * v[:, 0] * v[:, 1]).sum(), (m * v[:, 0] * v[:, 2]).sum(),
                           (m * v[:, 1] * v[:, 2]).sum()])
        vol = (prd[0] * prd[1]) * prd[2]
        Pt = (vir + kin) / vol
        qs.append(Pt[2] - 0.5 * (Pt[0] + Pt[1]))
        p = Pt[:3]
        if servo["couple"] == "xy":
            mxy = 0.5 * (Pt[0] + Pt[1])
            p = torch.stack([mxy, mxy, Pt[2]])
        elif servo["couple"] == "xyz":
            p = (Pt[0] + Pt[1] + Pt[2]).repeat(3) / 3.0
        new_lo, new_prd = [], []
        for d in range(3):
            st = servo["style"][d]
            if st == "erate":
                shift = ((0.5 * (s * dt)) * servo["rate"][d]) * (hi_s[d] - lo_s[d])
                nlo, nhi = lo_s[d] - shift, hi_s[d] + shift
            elif st == "pressure":
                rate = servo["pgain"][d] * (p[d] - servo["ptarget"][d])
                mr = servo.get("max_rate", 0.0)
                if mr != 0.0 and abs(float(rate)) > mr:
                    rate = torch.full_like(rate, mr if float(rate) > 0 else -mr).detach()
                cum = cum.clone()
                cum[d] = cum[d] + (dt * rate) * prd[d]
                nlo, nhi = lo_s[d] - 0.5 * cum[d], hi_s[d] + 0.5 * cum[d]
            else:
                nlo, nhi = lo[d], lo[d] + prd[d]
                new_lo.append(nlo)
                new_prd.append(prd[d])
                continue
            new_lo.append(nlo)
            new_prd.append(nhi - nlo)
        nlo_t, nprd_t = torch.stack(new_lo), torch.stack(new_prd)
        x = nprd_t * ((x - lo) / prd) + nlo_t
        lo, prd = nlo_t, nprd_t
    return torch.stack(qs)
