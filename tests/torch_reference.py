"""FP64 torch restatement of the std chain on a frozen edge list — the reference gradient.

Test infrastructure only.  Written with plain tensor ops so that torch.autograd gives an
independent gradient of exactly the function the hand-written adjoint differentiates: the table
interpolant (its slope is the derivative), the viscosity branch as a where(), the IAD inverse as
a batched 3x3 inverse.  Reference formulas: sph/include/sph/hydro_std/density.hpp:41-60,
hydro_std/eos.hpp:54-80, hydro_std/iad_kern.hpp:12-77, hydro_std/momentum_energy_kern.hpp:12-134.
"""

from __future__ import annotations

import torch


def lookup(tab: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
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
