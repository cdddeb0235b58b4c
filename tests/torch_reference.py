"""FP64 torch restatement of the std chain on a frozen edge list — the reference gradient.

Test infrastructure only.  Written with plain tensor ops so that torch.autograd gives an
independent gradient of exactly the function the hand-written adjoint differentiates: the table
interpolant (its slope is the derivative), the viscosity branch as a where(), the IAD inverse as
a batched 3x3 inverse.  Reference formulas: sph/include/sph/hydro_std/density.hpp:41-60,
hydro_std/eos.hpp:54-80, hydro_std/iad_kern.hpp:12-77, hydro_std/momentum_energy_kern.hpp:12-134.
"""

from __future__ import annotations

import torch


def hermite_tables(n: float, intervals: int = 19999):
    """W = sinc^n and dW/dv as cubic Hermite pieces on `intervals` equal intervals of [0, 2], rows
    {c0 c1 c2 c3} of c0 + f (c1 + f (c2 + f c3)): the smooth kernel form of the FP64 passes
    (sphgb_set_kernel_form), node values and derivatives from the closed form of
    sph/include/sph/kernels.hpp:35-61 (series below pi v / 2 = 1e-2)."""
    import numpy as np
    a = np.pi / 2
    v = np.arange(intervals + 1) * (2.0 / intervals)
    x = a * v
    small = x < 1e-2
    xs = np.where(small, 1.0, x)
    sn, cs = np.sin(xs), np.cos(xs)
    x2 = x * x
    s0 = np.where(small, 1 - x2 / 6 + x2 * x2 / 120 - x2 ** 3 / 5040, sn / xs)
    s1 = np.where(small, a * x * (-1 / 3 + x2 / 30 - x2 * x2 / 840), a * (xs * cs - sn) / (xs * xs))
    s2 = np.where(small, a * a * (-1 / 3 + x2 / 10 - x2 * x2 / 168),
                  a * a * (-xs * xs * sn - 2 * xs * cs + 2 * sn) / xs ** 3)
    s0 = np.maximum(s0, 0.0)
    w = s0 ** n
    w1 = n * s0 ** (n - 1) * s1
    w2 = np.where(s0 > 0, n * (n - 1) * s0 ** (n - 2) * s1 * s1 + n * s0 ** (n - 1) * s2, 0.0)
    dv = 2.0 / intervals

    def pieces(f, d):
        f0, f1, d0, d1 = f[:-1], f[1:], dv * d[:-1], dv * d[1:]
        return np.stack([f0, d0, 3 * (f1 - f0) - 2 * d0 - d1, 2 * (f0 - f1) + d0 + d1], 1)

    return pieces(w, w1), pieces(w1, w2)


def lookup(tab: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """kernel function at v: the linear interpolant of a 1-D table, or the cubic pieces of a
    (intervals, 4) coefficient table (the smooth form)"""
    if tab.dim() == 2:
        n_int = tab.shape[0]
        inv_dx = n_int / 2.0
        xv = v * inv_dx
        idx = torch.clamp(xv.detach().to(torch.int64), max=n_int)
        c = tab[torch.clamp(idx, max=n_int - 1)]
        f = xv - idx.to(v.dtype)
        val = c[:, 0] + f * (c[:, 1] + f * (c[:, 2] + f * c[:, 3]))
        return torch.where(idx >= n_int, torch.zeros_like(v), val)
    n_int = tab.numel() - 1
    dx = 2.0 / n_int
    inv_dx = 1.0 / dx
    idx = torch.clamp((v.detach() * inv_dx).to(torch.int64), max=n_int)
    a = tab[torch.clamp(idx, max=n_int - 1)]
    b = tab[torch.clamp(idx + 1, max=n_int)]
    slope = (b - a) * inv_dx
    val = a + slope * (v - idx.to(v.dtype) * dx)
    return torch.where(idx >= n_int, torch.zeros_like(v), val)


def std_chain(x, y, z, vx, vy, vz, h, u, m, edges_i, edges_j, tab, K, gamma, box_len, pbc):
    """returns rho, ax, ay, az, du of the std sweep for the given inputs and frozen edges (i owns)."""
    i, j = edges_i, edges_j
    two_h = 2.0 * h[i]

    def fold(d, k):
        if not pbc[k]:
            return d
        d = torch.where(d > two_h, d - box_len[k], d)
        return torch.where(d < -two_h, d + box_len[k], d)

    rx = fold(x[i] - x[j], 0)
    ry = fold(y[i] - y[j], 1)
    rz = fold(z[i] - z[j], 2)
    dist = torch.sqrt(rx * rx + ry * ry + rz * rz)
    n = x.shape[0]
    zeros = torch.zeros(n, dtype=x.dtype, device=x.device)

    hinv = 1.0 / h
    # density
    w_i = lookup(tab, dist * hinv[i])
    rho0 = m + zeros.index_add(0, i, w_i * m[j])
    rho = K * hinv ** 3 * rho0
    # EOS
    p = (gamma - 1.0) * rho * u
    c = torch.sqrt(gamma * (gamma - 1.0) * u)
    # IAD
    vol = (m / rho)[j] * w_i
    tau = torch.zeros(n, 3, 3, dtype=x.dtype, device=x.device)
    r = torch.stack([rx, ry, rz], 1)
    outer = r[:, :, None] * r[:, None, :] * vol[:, None, None]
    tau = tau.index_add(0, i, outer)
    C = torch.linalg.inv(tau) * (h ** 3 / K)[:, None, None]
    # momentum and energy
    vxij, vyij, vzij = vx[i] - vx[j], vy[i] - vy[j], vz[i] - vz[j]
    v = torch.stack([vxij, vyij, vzij], 1)
    Wi = hinv[i] ** 3 * w_i
    Wj = hinv[j] ** 3 * lookup(tab, dist * hinv[j])
    Ai = torch.einsum("pab,pb->pa", C[i], r)
    Aj = torch.einsum("pab,pb->pa", C[j], r)
    rv = (r * v).sum(1)
    wij = rv / dist
    cs = c[i] + c[j]
    visc = 0.5 * torch.where(wij < 0, -(0.5 * cs - 2.0 * wij) * wij, torch.zeros_like(wij))
    qi = m[j] * p[i] / (rho[i] * rho[i])
    si = (m / rho)[i]
    tj = (m / rho)[j]
    uj = (p / rho)[j]
    alpha = Wi * (qi + visc * si)
    beta = tj * Wj * (uj + visc)
    alphaP = Wi * (2.0 * qi + visc * si)
    betaP = visc * tj * Wj
    mom = alpha[:, None] * Ai + beta[:, None] * Aj
    en = (v * (alphaP[:, None] * Ai + betaP[:, None] * Aj)).sum(1)
    acc = torch.zeros(n, 3, dtype=x.dtype, device=x.device).index_add(0, i, mom) * K
    du = -0.5 * K * zeros.index_add(0, i, en)
    return rho, acc[:, 0], acc[:, 1], acc[:, 2], du


def ve_chain(x, y, z, vx, vy, vz, h, u, m, alpha0, edges_i, edges_j, tab, tabd, K, gamma, box_len, pbc,
             dt, alphamin, alphamax, decay_constant, av_clean):
    """returns rho, ax, ay, az, du of the VE sweep (xmass, gradh, EOS, IAD + divv/curlv, AV switches,
    momentum-energy) for the given inputs, the alpha before the AV switch and frozen edges (i owns).

    Reference formulas: hydro_ve/xmass_kern.hpp:50-79, ve_def_gradh_kern.hpp:43-90, eos.hpp:52-94,
    iad_kern.hpp:43-109, divv_curlv_kern.hpp:43-123, av_switches_kern.hpp:43-137,
    momentum_energy_kern.hpp:43-222.  Branches of the reference are where()s with the reference's
    tie rules: min(v1, v2) takes v1 unless v2 < v1; the signal-velocity maximum of the AV switch
    keeps the first pair of a tie (torch spreads a tie's gradient; seeded sets have none)."""
    i, j = edges_i, edges_j
    n = x.shape[0]
    two_h = 2.0 * h[i]

    def fold(d, k):
        if not pbc[k]:
            return d
        d = torch.where(d > two_h, d - box_len[k], d)
        return torch.where(d < -two_h, d + box_len[k], d)

    rx = fold(x[i] - x[j], 0)
    ry = fold(y[i] - y[j], 1)
    rz = fold(z[i] - z[j], 2)
    r = torch.stack([rx, ry, rz], 1)
    dist = torch.sqrt(rx * rx + ry * ry + rz * rz)
    zeros = torch.zeros(n, dtype=x.dtype, device=x.device)

    def seg(vals):
        return zeros.index_add(0, i, vals)

    hinv = 1.0 / h
    v1 = dist * hinv[i]
    w1 = lookup(tab, v1)
    # xmass
    xm = m / (K * hinv ** 3 * (m + seg(w1 * m[j])))
    # kx and gradh
    wd1 = lookup(tabd, v1)
    dterh = -(3.0 * w1 + v1 * wd1)
    kx = K * hinv ** 3 * (xm + seg(w1 * xm[j]))
    whomega0 = K * hinv ** 4 * (-3.0 * xm + seg(dterh * xm[j]))
    wrho0 = K * hinv ** 4 * (-3.0 * m + seg(dterh * m[j]))
    whomega = whomega0 * m / xm + (kx - K * xm * hinv ** 3) * wrho0
    rho = kx * m / xm
    dhdrho = -h / (rho * 3.0)
    gradh = 1.0 - dhdrho * whomega
    # EOS
    p = (gamma - 1.0) * rho * u
    c = torch.sqrt(gamma * (gamma - 1.0) * u)
    prho = p / (kx * m * m * gradh)
    # IAD with volumes xm / kx
    vol = xm / kx
    outer = r[:, :, None] * r[:, None, :] * (vol[j] * w1)[:, None, None]
    tau = torch.zeros(n, 3, 3, dtype=x.dtype, device=x.device).index_add(0, i, outer)
    C = torch.linalg.inv(tau) * (h ** 3 / K)[:, None, None]
    # divv, velocity gradient
    Cr_i = torch.einsum("pab,pb->pa", C[i], r)
    tA = -Cr_i * w1[:, None]
    v = torch.stack([vx, vy, vz], 1)
    vij = v[i] - v[j]
    dV = torch.zeros(n, 3, 3, dtype=x.dtype, device=x.device).index_add(
        0, i, (-vij * xm[j][:, None])[:, :, None] * tA[:, None, :])
    nk = K * hinv ** 3 / kx
    divv = nk * (dV[:, 0, 0] + dV[:, 1, 1] + dV[:, 2, 2])
    gsym = torch.stack([dV[:, 0, 0], dV[:, 0, 1] + dV[:, 1, 0], dV[:, 0, 2] + dV[:, 2, 0], dV[:, 1, 1],
                        dV[:, 1, 2] + dV[:, 2, 1], dV[:, 2, 2]], 1) * nk[:, None]
    # AV switches
    rv = (r * vij).sum(1)
    vsig_pair = torch.where(rv < 0, c[i] + c[j] - 3.0 * rv / dist, torch.zeros_like(rv))
    vsig = torch.maximum(1e-40 * c, zeros.scatter_reduce(0, i, vsig_pair, "amax", include_self=True))
    t = -Cr_i * (K * hinv[i] ** 3 * w1)[:, None]
    fac = vol[j] * (divv[i] - divv[j])
    g = torch.zeros(n, 3, dtype=x.dtype, device=x.device).index_add(0, i, fac[:, None] * t)
    gdv = torch.sqrt((g * g).sum(1))
    ac = h * h * gdv
    aloc = torch.where(divv < 0, alphamax * ac / (ac + h * divv.abs() + 0.05 * c), zeros)
    decay = h / (decay_constant * vsig)
    target = torch.where(aloc >= alphamin, aloc, torch.full_like(aloc, alphamin))
    alpha = torch.where(aloc >= alpha0, aloc, alpha0 + (target - alpha0) / decay * dt)
    # momentum and energy
    v2 = dist * hinv[j]
    Wi = hinv[i] ** 3 * w1
    Wj = hinv[j] ** 3 * lookup(tab, v2)
    Ai = -Cr_i * Wi[:, None]
    Aj = -torch.einsum("pab,pb->pa", C[j], r) * Wj[:, None]
    rv_me = rv
    if av_clean:
        cnt = zeros.index_add(0, i, torch.ones_like(rv))
        eta_crit = torch.pow(32.0 * torch.pi / 3.0 / (cnt + 1.0), 1.0 / 3.0)[i]

        def quad(gs):
            return (gs[:, 0] * rx * rx + gs[:, 1] * rx * ry + gs[:, 2] * rx * rz + gs[:, 3] * ry * ry
                    + gs[:, 4] * ry * rz + gs[:, 5] * rz * rz)

        d1, d2 = quad(gsym[i]), quad(gsym[j])
        eta = torch.where(v2 < v1, v2, v1)
        e = 5.0 * (eta - eta_crit)
        d3 = torch.where(eta < eta_crit, torch.exp(-e * e), torch.ones_like(eta))
        nz = d2 != 0
        A = torch.where(nz, d1 / torch.where(nz, d2, torch.ones_like(d2)), torch.zeros_like(d2))
        phi = 0.5 * d3 * torch.clamp(4.0 * A / ((1.0 + A) * (1.0 + A)), 0.0, 1.0)
        rv_me = rv - phi * (d1 + d2)
    wij = rv_me / dist
    visc = torch.where(wij < 0, -((alpha[i] + alpha[j]) / 4.0 * (c[i] + c[j]) - 2.0 * wij) * wij,
                       torch.zeros_like(wij))
    rhoi, rhoj = rho[i], rho[j]
    At = (rhoi - rhoj).abs() / (rhoi + rhoj)
    s = (At - 0.1) / (0.2 - 0.1)
    xmi, xmj = xm[i], xm[j]
    mid_a = xmi ** (2.0 - s) * xmj ** s
    mid_b = xmj ** (2.0 - s) * xmi ** s
    am = torch.where(At < 0.1, xmi * xmi, torch.where(At > 0.2, xmi * xmj, mid_a))
    bm = torch.where(At < 0.1, xmj * xmj, torch.where(At > 0.2, xmi * xmj, mid_b))
    mj = m[j]
    av = mj / rhoi * visc
    bv = mj / rhoj * visc
    avv = 0.5 * (av[:, None] * Ai + bv[:, None] * Aj)
    avE = torch.clamp(seg((avv * vij).sum(1)), min=0.0)
    en = seg(mj * am * (vij * Ai).sum(1))
    mom = (mj * prho[i] * am)[:, None] * Ai + (mj * prho[j] * bm)[:, None] * Aj + avv
    acc = -K * torch.zeros(n, 3, dtype=x.dtype, device=x.device).index_add(0, i, mom)
    du = K * (prho * en + 0.5 * avE)
    return rho, acc[:, 0], acc[:, 1], acc[:, 2], du
