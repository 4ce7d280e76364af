"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: FP64 torch reference of the soft
transmission, differentiated by torch autograd.

Only tests/ import this module, as the checker of the GPU discrete adjoint
(ctraj_soft_transmission).  It restates the soft model independently, in
float64 torch operations vectorised over molecules:

* initial conditions from unit normals: v = mu + sigma n, x = sigma_x n_x, y =
  sigma_y n_y (sigma_vx, sigma_vy are parameters);
* ballistic flights to each aperture plane in closed form with a = (0, -g)
  (molecule.py:26-68: x + v t + a t^2 / 2, v + a t);
* every hard test of a circular aperture (apertures.py:101-115, alive iff
  sqrt(x^2 + y^2) <= d/2), of the lens entrance and of the bore after each RK4
  step (electrostatic_lens.py:60-66, 112-118) replaced by the log weight
  log sigmoid((R - r) / width);
* behind the lens, circular apertures reached by a flight with a = (0, -g)
  from the state after the last RK4 step at z0 + N dz (t = (z - z0 - N dz) /
  vz), each plane with its soft test;
* the lens interior as the reference's RK4 (electrostatic_lens.py:91-111:
  k1 = v, stage-2 point x + dt k1, stage-3 point x + dt/2 k2, stage-4 point
  x + dt k3; x' = x + dt/6 (k1 + 2 k2 + 2 k3 + k4), v' likewise) with
  N = rint(L/dz), dt = dz/vz and dz = vz dt_fixed (electrostatic_lens.py:87-88),
  for the hexapole force a = -W'(E) grad|E| / m, |E| = 3 V r^2 / R^3, W' the
  derivative of the cubic Stark spline (scipy PPoly nu = 1 polynomial);
* molecules whose log weight falls below log_floor are frozen and count zero.

The loss is sum(exp(log weight)) / n.
"""
from __future__ import annotations

import math

import numpy as np

G = 9.80665
CIRCULAR_APERTURE = 1
ELECTROSTATIC_LENS = 4
STEP_DT = 1
RK4_CLASSIC = 1


def _logsig(z):
    import torch

    return torch.nn.functional.logsigmoid(z)


def soft_loss(cb, normals, xdist, vdist, params, aperture: int = -1, width: float = 0.2e-3,
              log_floor: float = -30.0, g: float = G):
    """Soft transmission (torch float64 scalar) for params = (V, lens z0,
    aperture radius, bore radius, sigma_vx, sigma_vy), a torch float64 tensor.

    cb: a compiled beamline (element structs and force tables, the inputs the
    CUDA library receives); normals: (5, n) unit normals; xdist / vdist:
    Gaussian position / velocity descriptors (p arrays as in ctraj.h).
    """
    import torch

    f64 = torch.float64
    V, z0, r_ap, bore, s_vx, s_vy = params.unbind()
    els = list(cb.elements)
    li = [i for i, e in enumerate(els) if e.type == ELECTROSTATIC_LENS][0]
    L = els[li]
    tab = cb.tables[L.table]
    nrm = torch.as_tensor(np.asarray(normals), dtype=f64)
    n = nrm.shape[1]
    vx = vdist.p[0] + s_vx * nrm[0]
    vy = vdist.p[2] + s_vy * nrm[1]
    vz = vdist.p[4] + vdist.p[5] * nrm[2]
    x = xdist.p[0] * nrm[3]
    y = xdist.p[1] * nrm[4]
    lw = torch.zeros(n, dtype=f64)
    zprev = torch.tensor(xdist.p[2], dtype=f64)

    def fly(zp, x, y, vy, zprev):
        t = (zp - zprev) / vz
        return x + vx * t, y + vy * t - 0.5 * g * t * t, vy - g * t

    inv_w = 1.0 / width
    for i in range(li):
        e = els[i]
        R = r_ap if i == aperture else torch.tensor(e.p[0] / 2, dtype=f64)
        for zp in (e.z0, e.z1):
            zp = torch.tensor(zp, dtype=f64)
            x, y, vy = fly(zp, x, y, vy, zprev)
            zprev = zp
            if math.isfinite(float(R.detach())):
                lw = lw + _logsig((R - torch.sqrt(x * x + y * y)) * inv_w)
    x, y, vy = fly(z0, x, y, vy, zprev)
    lw = lw + _logsig((bore - torch.sqrt(x * x + y * y)) * inv_w)

    keep = (lw.detach() >= log_floor).nonzero().flatten()
    x, y, vx, vy, vz, lw = x[keep], y[keep], vx[keep], vy[keep], vz[keep], lw[keep]
    # step count and size in float64 exactly as electrostatic_lens.py:87-88
    vz_np = vz.detach().numpy()
    dz = vz_np * L.p[2] if L.step_mode == STEP_DT else np.full_like(vz_np, L.p[1])
    N = np.rint(L.p[7] / dz)
    ok = np.isfinite(N) & (np.abs(N) <= 1e7)
    N = np.where(ok, np.maximum(N, 0), 0).astype(np.int64)
    dt = torch.as_tensor(np.where(ok, dz / vz_np, 0.0), dtype=f64)
    alive = torch.as_tensor(ok)
    hdt = 0.5 * dt
    c2 = hdt if L.scheme == RK4_CLASSIC else dt

    knots = np.asarray(tab.knots, dtype=np.float64)
    coef = np.asarray(tab.coef, dtype=np.float64)
    h = (knots[-1] - knots[0]) / (knots.size - 1)
    q0 = torch.as_tensor(coef[:, 2], dtype=f64)
    q1 = torch.as_tensor(2.0 * coef[:, 1] * h, dtype=f64)
    q2 = torch.as_tensor(3.0 * coef[:, 0] * h * h, dtype=f64)
    n_int = knots.size - 1
    Rf, mass = L.p[4], L.p[5]
    alpha = 3.0 * V / Rf ** 3
    beta = alpha / h
    s0 = knots[0] / h
    kappa = -2.0 * alpha / mass

    def accel(px, py):
        s = beta * (px * px + py * py) - s0
        i = torch.clamp(torch.floor(s.detach()), 0, n_int - 1).long()
        u = s - i.to(f64)
        w = kappa * (q0[i] + u * (q1[i] + u * q2[i]))
        return w * px, w * py - g

    Nt = torch.as_tensor(N)
    for k in range(int(N.max()) if N.size else 0):
        act = (k < Nt) & alive
        if not bool(act.any()):
            break
        l1x, l1y = accel(x, y)
        k2x, k2y = vx + hdt * l1x, vy + hdt * l1y
        l2x, l2y = accel(x + c2 * vx, y + c2 * vy)
        k3x, k3y = vx + hdt * l2x, vy + hdt * l2y
        l3x, l3y = accel(x + hdt * k2x, y + hdt * k2y)
        k4x, k4y = vx + dt * l3x, vy + dt * l3y
        l4x, l4y = accel(x + dt * k3x, y + dt * k3y)
        xn = x + dt / 6 * (vx + 2 * k2x + 2 * k3x + k4x)
        yn = y + dt / 6 * (vy + 2 * k2y + 2 * k3y + k4y)
        vxn = vx + dt / 6 * (l1x + 2 * l2x + 2 * l3x + l4x)
        vyn = vy + dt / 6 * (l1y + 2 * l2y + 2 * l3y + l4y)
        x, y = torch.where(act, xn, x), torch.where(act, yn, y)
        vx, vy = torch.where(act, vxn, vx), torch.where(act, vyn, vy)
        ls = _logsig((bore - torch.sqrt(x * x + y * y)) * inv_w)
        lw = lw + torch.where(act, ls, torch.zeros_like(ls))
        alive = alive & ~(act & (lw.detach() < log_floor))
    # circular apertures behind the lens, from the state after the last step
    zrel = torch.as_tensor(N * dz, dtype=f64)
    for i in range(li + 1, len(els)):
        e = els[i]
        R = r_ap if i == aperture else torch.tensor(e.p[0] / 2, dtype=f64)
        if not math.isfinite(float(R.detach())):
            continue
        for zp in (e.z0, e.z1):
            t = (zp - z0 - zrel) / vz
            xp = x + vx * t
            yp = y + vy * t - 0.5 * g * t * t
            ls = _logsig((R - torch.sqrt(xp * xp + yp * yp)) * inv_w)
            lw = lw + torch.where(alive, ls, torch.zeros_like(ls))
    alive = alive & (lw.detach() >= log_floor)
    return torch.where(alive, torch.exp(lw), torch.zeros_like(lw)).sum() / n


def soft_grad(cb, normals, xdist, vdist, params, **kw):
    """(loss, d loss / d params) by torch autograd, float64."""
    import torch

    p = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
    loss = soft_loss(cb, normals, xdist, vdist, p, **kw)
    loss.backward()
    return float(loss.item()), p.grad.numpy().copy()


def soft_fd(cb, normals, xdist, vdist, params, rel: float = 1e-4, **kw):
    """Central finite differences with step rel * |param| (float64, no autograd)."""
    import torch

    p0 = np.asarray(params, dtype=np.float64)
    out = np.zeros_like(p0)
    with torch.no_grad():
        for k in range(p0.size):
            hk = rel * abs(p0[k])
            pp, pm = p0.copy(), p0.copy()
            pp[k] += hk
            pm[k] -= hk
            lp = float(soft_loss(cb, normals, xdist, vdist, torch.tensor(pp), **kw))
            lm = float(soft_loss(cb, normals, xdist, vdist, torch.tensor(pm), **kw))
            out[k] = (lp - lm) / (2 * hk)
    return out
