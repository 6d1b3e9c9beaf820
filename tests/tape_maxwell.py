"""FP64 torch restatement of the oracle's time step, for tape (reverse-mode)
automatic differentiation with respect to the permittivity at every node.

Test infrastructure: it follows the oracle routines (oracle/refcpu.c) on the
oracle's own mesh arrays, with eps as a differentiable input --
set_materials (src/cem_maxwell.F:262-325: impedances, gs sum, PEC doubling,
ebm1), wght_curl (src/cem_maxwell.F:1428-1497), restrict_to_face,
flux3d (src/cem_maxwell.F:922-1002, gs pair sums, PEC, upwind combination),
add_flux_to_res, usersrc, invqmass and the RK45 low-storage update
(src/cem_common.F:18-104).  Summation orders differ from the oracle, so it
agrees with it to rounding, not bit for bit.
"""
from __future__ import annotations

import numpy as np
import torch

from oracle import refcpu as R


class TapeMaxwell:
    def __init__(self, ref: R.RefBox, C0: float = 1.0):
        f64 = torch.float64
        self.n, self.nelt, self.npts, self.nxzf = ref.n, ref.nelt, ref.npts, ref.nxzf
        n = self.n
        T = lambda name: torch.tensor(ref.d(name).copy(), dtype=f64)
        self.D = torch.tensor(ref.d("dxm1").copy().reshape(n, n).T.copy(), dtype=f64)  # D[i, l]
        self.w3 = T("w3m1")
        self.bm1 = T("bm1")
        self.geo = {k: T(k) for k in ("rxm1", "rym1", "rzm1", "sxm1", "sym1", "szm1", "txm1",
                                      "tym1", "tzm1")}
        self.unx, self.uny, self.unz, self.area = T("unx"), T("uny"), T("unz"), T("area")
        self.cemface = torch.tensor(ref.i("cemface").astype(np.int64))
        pec = ref.i("cempec").astype(np.int64)
        self.cempec = torch.tensor(pec)
        ids = ref.l("glo_face").copy()
        _, inv = np.unique(ids, return_inverse=True)
        self.group = torch.tensor(inv.astype(np.int64))
        self.ngroups = int(inv.max()) + 1
        cbc = ref.i("cbc").copy()
        dbl = np.zeros(ref.nxzfl)
        for e in range(self.nelt):
            for f in range(6):
                if cbc[6 * e + f] == 1:
                    dbl[ref.nxzf * (f + 6 * e):ref.nxzf * (f + 6 * e + 1)] = 1.0
        self.pec_face = torch.tensor(dbl, dtype=f64)
        self.mu = T("permeability")
        self.C0 = C0
        self.rk_a, self.rk_b, self.rk_c = R.rk_coeffs()
        self.src_w = None

    # ---- pieces ------------------------------------------------------------------
    def gs(self, v):
        s = torch.zeros(self.ngroups, dtype=v.dtype).index_add(0, self.group, v)
        return s[self.group]

    def materials(self, eps):
        impede = torch.sqrt(self.mu / eps)
        conduc = torch.sqrt(eps / self.mu)
        zi, yc = impede[self.cemface], conduc[self.cemface]
        Z0 = self.gs(zi) * (1.0 + self.pec_face)
        Y0 = self.gs(yc) * (1.0 + self.pec_face)
        Z1, Y1 = Z0 - zi, Y0 - yc
        return 0.5 * Z0, Z1, 0.5 * Y0, Y1

    def grad3(self, u):
        n = self.n
        v = u.reshape(self.nelt, n, n, n)  # [e, k, j, i]
        ur = torch.einsum("il,ekjl->ekji", self.D, v).reshape(-1)
        us = torch.einsum("jl,ekli->ekji", self.D, v).reshape(-1)
        ut = torch.einsum("kl,elji->ekji", self.D, v).reshape(-1)
        return ur, us, ut

    def curl(self, u1, u2, u3):
        w = self.w3.repeat(self.nelt)
        g = self.geo
        r1, s1, t1 = (x * w for x in self.grad3(u1))
        r2, s2, t2 = (x * w for x in self.grad3(u2))
        r3, s3, t3 = (x * w for x in self.grad3(u3))
        w1 = r3 * g["rym1"] + s3 * g["sym1"] + t3 * g["tym1"] - r2 * g["rzm1"] - s2 * g["szm1"] - t2 * g["tzm1"]
        w2 = r1 * g["rzm1"] + s1 * g["szm1"] + t1 * g["tzm1"] - r3 * g["rxm1"] - s3 * g["sxm1"] - t3 * g["txm1"]
        w3 = r2 * g["rxm1"] + s2 * g["sxm1"] + t2 * g["txm1"] - r1 * g["rym1"] - s1 * g["sym1"] - t1 * g["tym1"]
        return w1, w2, w3

    def operator(self, H, E, eps, mats, rktime):
        """cem_maxwell_op: the residuals (reshn, resen) after invqmass."""
        Z0, Z1, Y0, Y1 = mats
        resE = torch.stack(self.curl(H[0], H[1], H[2]))
        resH = -torch.stack(self.curl(E[0], E[1], E[2]))
        fh, fe = H[:, self.cemface], E[:, self.cemface]
        nx, ny, nz = self.unx, self.uny, self.unz
        s = torch.stack([-ny * fe[2] + nz * fe[1], -nz * fe[0] + nx * fe[2], -nx * fe[1] + ny * fe[0],
                         -ny * fh[2] + nz * fh[1], -nz * fh[0] + nx * fh[2], -nx * fh[1] + ny * fh[0]])
        s = torch.stack([self.gs(s[q]) for q in range(6)])
        if self.cempec.numel():
            m = torch.ones(6, s.shape[1], dtype=s.dtype)
            m[:3, self.cempec] = 2.0
            m[3:, self.cempec] = 0.0
            s = s * m
        Y02, Z02 = -0.5 / Y0 * Y1, 0.5 / Z0 * Z1
        C02Y, C02Z = 0.5 / Y0 * self.C0, 0.5 / Z0 * self.C0
        fu = [ny * s[5] - nz * s[4], nz * s[3] - nx * s[5], nx * s[4] - ny * s[3]]
        fw = [ny * s[2] - nz * s[1], nz * s[0] - nx * s[2], nx * s[1] - ny * s[0]]
        sh = torch.stack([Y02 * s[q] - C02Y * fu[q] for q in range(3)])
        se = torch.stack([Z02 * s[3 + q] - C02Z * fw[q] for q in range(3)])
        resH = resH.index_add(1, self.cemface, self.area * sh)
        resE = resE.index_add(1, self.cemface, self.area * se)
        if self.src_w is not None:
            a = np.pi * self.src_f0 * (rktime - self.src_t0)
            ft = self.src_amp * (1.0 - 2.0 * a * a) * np.exp(-a * a)
            resE = resE + torch.stack([0 * self.src_w, 0 * self.src_w, self.src_w * ft])
        hbm1 = 1.0 / (self.mu * self.bm1)
        ebm1 = 1.0 / (eps * self.bm1)
        return resH * hbm1, resE * ebm1

    def set_source(self, x, y, z, xc, sigma, amp, f0, t0):
        r2 = (x - xc[0]) ** 2 + (y - xc[1]) ** 2 + (z - xc[2]) ** 2
        self.src_w = self.bm1 * torch.tensor(np.exp(-r2 / (2.0 * sigma * sigma)))
        self.src_amp, self.src_f0, self.src_t0 = amp, f0, t0

    def run(self, H, E, eps, nsteps, t0, dt):
        """time_advancing_pde: nsteps of cem_maxwell_op_rk; returns (H, E)."""
        mats = self.materials(eps)
        kH = torch.zeros_like(H)
        kE = torch.zeros_like(E)
        t = t0
        for _ in range(nsteps):
            for r in range(5):
                rH, rE = self.operator(H, E, eps, mats, t + dt * self.rk_c[r])
                kH = self.rk_a[r] * kH + dt * rH
                kE = self.rk_a[r] * kE + dt * rE
                H = H + self.rk_b[r] * kH
                E = E + self.rk_b[r] * kE
            t = t + dt
        return H, E
