"""Torch (float64, CPU) restatement of the two-node nodal update and of the
CMFD operators, differentiable end to end, for tests only.

The nodal update N(phi, dn, k; Sigma) of mod_nodal.f90 (SANM and PNM, static
mode) is restated with whole-core tensors:

    get_source / Lxyz          :901-1043   face currents -> S1..S3
    TLUpd1 / TLUpd2            :1047-1341  first and second leakage moments
    get_B, get_ABEFGH          :1345-1451  buckling matrix, SANM constants
    get_a2matvec, LU_solve,
    get_a4                     :740-897    a2, a4 per node and direction
    get_a1matvec[_first|_last],
    get_a3, nodal_coup_upd     :282-736    a1, a3, the new dn per face

and the coupling coefficients df of coup_coef (mod_cmfd.f90:11-137) and the
CMFD matrix of matrix_setup (:217-304) are built from the same tensors, so
torch.autograd gives every partial derivative the adjoint of the nonlinear
fixed point needs (tests/adjoint_full_ref.py).  Dense linear solves use
torch.linalg.solve (partial pivoting): the same solution as the reference's
no-pivot LU to rounding.

Interior faces carry one coupling coefficient (nod(n)%dn(sf) and
nod(p)%dn(sf+1) are set together, mod_nodal.f90:328-329).  The unique face
variables are held in "canonical" slots of the (nnod, ng, 6) layout: the
minus face (0-based 2u+1) of every node, and the plus face (2u) of a node
whose plus face is a boundary face.
"""
from __future__ import annotations

import numpy as np
import torch

from adjoint_ref import Dense

ALB = 1.0e30
F1EM4 = float(np.float32(10e-5))


class NodalRef:
    def __init__(self, o):
        self.o = o
        d = Dense(o)
        self.d = d
        self.nn, self.ng = d.nn, d.ng
        nn, ng = self.nn, self.ng
        self.kern = o.geti("kern")       # 0 FDM, 1 PNM, 2 SANM
        self.nbr = torch.tensor(d.nbr, dtype=torch.long)               # (nn, 6), -1 outside
        h = np.zeros((nn, 3))
        for n in range(nn):
            for u in range(3):
                h[n, u] = d.h(n, u)
        self.h = torch.tensor(h)
        self.bcf = list(d.bc)                                           # per face 0..5
        self.mat = torch.tensor(o.array("mat").astype(int) - 1)
        self.chi = torch.tensor(o.fortran("chi", (o.geti("nmat"), ng)))
        self.chin = self.chi[self.mat]                                  # (nn, ng)
        self.dc = torch.tensor(o.fortran("dc", (nn, ng, 6)))
        self.vol = torch.tensor(o.array("vdel"))
        # canonical face slots
        canon = np.zeros((nn, 6), dtype=bool)
        for n in range(nn):
            for u in range(3):
                canon[n, 2 * u + 1] = True
                if d.nbr[n, 2 * u] < 0:
                    canon[n, 2 * u] = True
        self.canon = torch.tensor(canon)
        # geometry factors of TLUpd1/TLUpd2 per (node, direction)
        c = np.zeros((4, nn, 3))
        for n in range(nn):
            for u in range(3):
                c[:, n, u] = self._tl_geom(n, u)
        self.c1p, self.c1m, self.c2p, self.c2m = (torch.tensor(c[i]) for i in range(4))

    # -- state from the oracle -------------------------------------------------
    def params(self):
        """The independent cross sections: D, siga, nuf (nn, ng), sigs (nn, ng, ng)."""
        o, nn, ng = self.o, self.nn, self.ng
        D = torch.tensor(o.fortran("D", (nn, ng)))
        sigr = o.fortran("sigr", (nn, ng))
        sigs = o.fortran("sigs", (nn, ng, ng))
        off = sigs.sum(2) - np.einsum("ngg->ng", sigs)
        siga = torch.tensor(sigr - off)
        return dict(D=D, siga=siga, nuf=torch.tensor(o.fortran("nuf", (nn, ng))), sigs=torch.tensor(sigs))

    def state(self):
        o, nn, ng = self.o, self.nn, self.ng
        phi = torch.tensor(o.fortran("f0", (nn, ng)))
        dn = torch.tensor(o.fortran("dn", (nn, ng, 6)))
        return phi, self.to_canon(dn), float(o.getd("Ke"))

    @staticmethod
    def sigr_of(p):
        sigs = p["sigs"]
        off = sigs.sum(2) - torch.diagonal(sigs, dim1=1, dim2=2)
        return p["siga"] + off

    # -- face layout helpers ---------------------------------------------------
    def to_canon(self, full):
        """(nn, ng, 6) -> the same layout with only the canonical slots kept."""
        return full * self.canon[:, None, :]

    def expand(self, dnc):
        """Canonical face variables -> both slots of every interior face."""
        nn = self.nn
        cols = []
        for f in range(6):
            if f % 2 == 1:
                cols.append(dnc[:, :, f])
            else:
                m = self.nbr[:, f]
                inner = m >= 0
                v = torch.where(inner[:, None], dnc[m.clamp(min=0), :, f + 1], dnc[:, :, f])
                cols.append(v)
        return torch.stack(cols, dim=2)

    # -- coup_coef ---------------------------------------------------------------
    def df_of(self, D):
        cols = []
        for f in range(6):
            u = f // 2
            hn = self.h[:, u][:, None]
            m = self.nbr[:, f]
            inner = (m >= 0)[:, None]
            Dm = D[m.clamp(min=0)]
            hm = self.h[m.clamp(min=0), u][:, None]
            v_in = 2.0 * D * Dm / (D * hm + Dm * hn)
            bc = self.bcf[f]
            if bc == 0:
                v_b = 2.0 * ALB * D / (2.0 * D + ALB * hn)
            elif bc == 1:
                v_b = D / (2.0 * D + 0.5 * hn)
            else:
                v_b = torch.zeros_like(D)
            cols.append(torch.where(inner, v_in, v_b))
        return torch.stack(cols, dim=2)

    # -- matrix_setup + TSrc: dense M and F --------------------------------------
    def operators(self, p, dnc):
        nn, ng = self.nn, self.ng
        D = p["D"]
        sigr = self.sigr_of(p)
        df = self.df_of(D)
        dn = self.expand(dnc)
        N = nn * ng
        M = torch.zeros((N, N), dtype=torch.float64)
        idx = torch.arange(nn)
        for g in range(ng):
            diag = sigr[:, g].clone()
            for u in range(3):
                hu = self.h[:, u]
                fp, fm = 2 * u, 2 * u + 1
                diag = diag + (df[:, g, fp] - dn[:, g, fp] + df[:, g, fm] + dn[:, g, fm]) / hu
                for f, sgn in ((fp, 1.0), (fm, -1.0)):
                    m = self.nbr[:, f]
                    ok = m >= 0
                    val = -(df[:, g, f] + sgn * dn[:, g, f]) / hu
                    M = M.index_put((g * nn + idx[ok], g * nn + m[ok]), val[ok], accumulate=True)
            M = M.index_put((g * nn + idx, g * nn + idx), diag, accumulate=True)
            for h in range(ng):
                if h != g:
                    M = M.index_put((g * nn + idx, h * nn + idx), -p["sigs"][:, h, g], accumulate=True)
        F = torch.zeros((N, N), dtype=torch.float64)
        for g in range(ng):
            for h in range(ng):
                F = F.index_put((g * nn + idx, h * nn + idx), self.chin[:, g] * p["nuf"][:, h], accumulate=True)
        return M, F

    # -- the nodal update ----------------------------------------------------------
    def _tl_geom(self, n, u):
        d = self.d
        fp, fm = 2 * u, 2 * u + 1
        first, last = d.nbr[n, fm] < 0, d.nbr[n, fp] < 0
        h0 = d.h(n, u)
        c1p = c1m = c2p = c2m = 0.0
        if first:
            tp = d.h(d.nbr[n, fp], u) / h0
            p1p = tp + 1.0
            if self.bcf[fm] == 2:
                tm = 1.0
                p1m, p2m = tm + 1.0, 2.0 * tm + 1.0
                hp = 2.0 * p1m * p1p * (tm + tp + 1.0)
                c1p, c2p = p1m * p2m / hp, p1m / hp
            else:
                c1p = 1.0 / p1p
        elif last:
            tm = d.h(d.nbr[n, fm], u) / h0
            p1m = tm + 1.0
            if self.bcf[fp] == 2:
                tp = 1.0
                p1p, p2p = tp + 1.0, 2.0 * tp + 1.0
                hp = 2.0 * p1m * p1p * (tm + tp + 1.0)
                c1m, c2m = p1p * p2p / hp, p1p / hp
            else:
                c1m = 1.0 / p1m
        else:
            tm = d.h(d.nbr[n, fm], u) / h0
            tp = d.h(d.nbr[n, fp], u) / h0
            p1m, p2m = tm + 1.0, 2.0 * tm + 1.0
            p1p, p2p = tp + 1.0, 2.0 * tp + 1.0
            hp = 2.0 * p1m * p1p * (tm + tp + 1.0)
            c1p, c1m, c2p, c2m = p1m * p2m / hp, p1p * p2p / hp, p1m / hp, p1p / hp
        return c1p, c1m, c2p, c2m

    def consts(self, D, sigr):
        """(A, B, E, F, G, H), each (nn, 3, ng): get_ABEFGH or the PNM constants."""
        nn, ng = self.nn, self.ng
        if self.kern == 1:
            vals = (1.0 / 15.0, 1.0 / 35.0, 2.0 / 7.0, 2.0 / 5.0, 10.0, 6.0)
            return tuple(torch.full((nn, 3, ng), v, dtype=torch.float64) for v in vals)
        alp = 0.5 * torch.sqrt(sigr / D)[:, None, :] * self.h[:, :, None]
        alp2 = alp * alp
        sh, ch = torch.sinh(alp), torch.cosh(alp)
        m0c = sh / alp
        m1s = 3.0 * (ch / alp - sh / alp2)
        m2c = 5.0 * (sh / alp - 3.0 * ch / alp2 + 3.0 * sh / alp ** 3)
        A = (sh - m1s) / (alp2 * m1s)
        B = (ch - m0c - m2c) / (alp2 * m2c)
        E = m0c / m2c - 3.0 / alp2
        F = (alp * ch - m1s) / (alp2 * m1s)
        G = (alp * sh - 3.0 * m2c) / (ch - m0c - m2c)
        H = (alp * ch - m1s) / (sh - m1s)
        return A, B, E, F, G, H

    def update(self, phi, dnc, k, p):
        """The new canonical dn of nodal_update/nodal_update_pnm (cal_mode 1)."""
        nn, ng = self.nn, self.ng
        D, nuf, sigs = p["D"], p["nuf"], p["sigs"]
        sigr = self.sigr_of(p)
        df = self.df_of(D)
        dn = self.expand(dnc)
        nbr = self.nbr
        # get_source / Lxyz
        L = []
        for u in range(3):
            fp, fm = 2 * u, 2 * u + 1
            mp, mm = nbr[:, fp], nbr[:, fm]
            fpv = phi[mp.clamp(min=0)]
            fmv = phi[mm.clamp(min=0)]
            jp_in = -df[:, :, fp] * (fpv - phi) - dn[:, :, fp] * (fpv + phi)
            jp_b = torch.zeros_like(phi) if self.bcf[fp] == 2 else df[:, :, fp] * phi - dn[:, :, fp] * phi
            jp = torch.where((mp >= 0)[:, None], jp_in, jp_b)
            jm_in = -df[:, :, fm] * (phi - fmv) - dn[:, :, fm] * (phi + fmv)
            jm_b = torch.zeros_like(phi) if self.bcf[fm] == 2 else -df[:, :, fm] * phi - dn[:, :, fm] * phi
            jm = torch.where((mm >= 0)[:, None], jm_in, jm_b)
            L.append((jp - jm) / self.h[:, u][:, None])
        S = torch.stack([L[1] + L[2], L[0] + L[2], L[0] + L[1]], dim=1)   # (nn, 3, ng)
        # per node and direction
        Ac, Bk, Ek, Fk, Gk, Hk = self.consts(D, sigr)
        fac = 0.25 * self.h[:, :, None] ** 2 / D[:, None, :]               # (nn, 3, ng)
        invk = 1.0 / k
        dum = torch.empty((nn, ng, ng), dtype=torch.float64)
        rows = []
        for g in range(ng):
            cols = []
            for h in range(ng):
                if g == h:
                    cols.append(sigr[:, g] - self.chin[:, g] * nuf[:, h] * invk)
                else:
                    cols.append(-sigs[:, h, g] - self.chin[:, g] * nuf[:, h] * invk)
            rows.append(torch.stack(cols, 1))
        dum = torch.stack(rows, 1)                                         # (nn, g, h)
        Bc = fac[:, :, :, None] * dum[:, None, :, :]                       # (nn, 3, g, h)
        a2, a4, L1 = [], [], []
        eye = torch.eye(ng, dtype=torch.float64)
        for u in range(3):
            fp, fm = 2 * u, 2 * u + 1
            mp, mm = nbr[:, fp], nbr[:, fm]
            Su = S[:, u, :]
            dSp = torch.where((mp >= 0)[:, None], Su[mp.clamp(min=0)] - Su, torch.zeros_like(Su))
            dSm = torch.where((mm >= 0)[:, None], Su[mm.clamp(min=0)] - Su, torch.zeros_like(Su))
            fu = fac[:, u, :]
            Lm2 = fu * (self.c2p[:, u, None] * dSp + self.c2m[:, u, None] * dSm)
            L1.append(fu * (self.c1p[:, u, None] * dSp - self.c1m[:, u, None] * dSm))
            Bu = Bc[:, u]
            Mm = Bu * Ek[:, u, :, None] + 3.0 * eye
            rhs = torch.einsum("ngh,nh->ng", Bu, phi) - Ek[:, u] * Lm2 + fu * Su
            a2u = torch.linalg.solve(Mm, rhs)
            a2.append(a2u)
            a4.append(Bk[:, u] * (torch.einsum("ngh,nh->ng", Bu, a2u) + Lm2))
        a2, a4, L1 = torch.stack(a2, 1), torch.stack(a4, 1), torch.stack(L1, 1)
        # per face
        out = torch.zeros((nn, ng, 6), dtype=torch.float64)
        idx = torch.arange(nn)
        for u in range(3):
            fp, fm = 2 * u, 2 * u + 1
            # interior faces: p = node, n = its minus neighbour
            mm = nbr[:, fm]
            ok = mm >= 0
            pi, ni = idx[ok], mm[ok]
            hn, hp = self.h[ni, u][:, None], self.h[pi, u][:, None]
            Pn, Pp = 2.0 * D[ni] / hn, 2.0 * D[pi] / hp
            Bn, Bp = Bc[ni, u], Bc[pi, u]
            An, Ap = Ac[ni, u], Ac[pi, u]
            Fn, Fp = Fk[ni, u], Fk[pi, u]
            Gn, Gp = Gk[ni, u], Gk[pi, u]
            Hn = Hk[ni, u]
            a2n, a2p, a4n, a4p = a2[ni, u], a2[pi, u], a4[ni, u], a4[pi, u]
            L1n, L1p = L1[ni, u], L1[pi, u]
            fn, fpp = phi[ni], phi[pi]
            dcn, dcp = self.dc[ni, :, fp], self.dc[pi, :, fm]
            R11 = -Pn[:, :, None] * (Bn * Fn[:, :, None] + eye)
            R12 = Pp[:, :, None] * (Bp * Fp[:, :, None] + eye)
            R21 = dcn[:, :, None] * (Bn * An[:, :, None] + eye)
            R22 = dcp[:, :, None] * (Bp * Ap[:, :, None] + eye)
            R = torch.cat([torch.cat([R11, R12], 2), torch.cat([R21, R22], 2)], 1)
            x1 = Pn * (3.0 * a2n + Gn * a4n + Fn * L1n) + Pp * (3.0 * a2p + Gp * a4p - Fp * L1p)
            x2 = dcp * (a2p + a4p + fpp - An * L1n) - dcn * (a2n + a4n + fn + Ap * L1p)
            s = torch.linalg.solve(R, torch.cat([x1, x2], 1))
            a1n = s[:, :ng]
            a3 = An * (torch.einsum("ngh,nh->ng", Bn, a1n) + L1n)
            jp = -D[ni] * 2.0 / hn * (a1n + 3.0 * a2n + Hn * a3 + Gn * a4n)
            dnew = (df[ni, :, fp] * (fn - fpp) - jp) / (fn + fpp)
            out[pi, :, fm] = dnew
            # first boundary faces
            fi = idx[~ok]
            if len(fi):
                out[fi, :, fm] = self._boundary(u, fi, True, phi, D, Bc, Ac, Fk, Gk, Hk, a2, a4, L1, df)
            li = idx[nbr[:, fp] < 0]
            if len(li):
                out[li, :, fp] = self._boundary(u, li, False, phi, D, Bc, Ac, Fk, Gk, Hk, a2, a4, L1, df)
        return out

    def _boundary(self, u, ii, first, phi, D, Bc, Ac, Fk, Gk, Hk, a2, a4, L1, df):
        ng = self.ng
        eye = torch.eye(ng, dtype=torch.float64)
        f = 2 * u + 1 if first else 2 * u
        bc = self.bcf[f]
        hh = self.h[ii, u][:, None]
        P = 2.0 * D[ii] / hh
        B = Bc[ii, u]
        A_, F_, G_, H_ = Ac[ii, u], Fk[ii, u], Gk[ii, u], Hk[ii, u]
        a2v, a4v, L1v, fv = a2[ii, u], a4[ii, u], L1[ii, u], phi[ii]
        dcv = self.dc[ii, :, f]
        if first:
            if bc == 2:
                Am = P[:, :, None] * (B * F_[:, :, None] + eye)
                x = P * (3.0 * a2v + G_ * a4v - F_ * L1v)
            elif bc == 1:
                Am = -dcv[:, :, None] * (eye + A_[:, :, None] * B) - 2.0 * P[:, :, None] * (
                    A_[:, :, None] * B * H_[:, :, None] + eye)
                x = 2.0 * P * (A_ * H_ * L1v - 3.0 * a2v - G_ * a4v) - dcv * (a2v + a4v + fv - A_ * L1v)
            else:
                Am = dcv[:, :, None] * (eye + A_[:, :, None] * B)
                x = dcv * (a2v + a4v + fv - A_ * L1v)
        else:
            if bc == 2:
                Am = -P[:, :, None] * (B * F_[:, :, None] + eye)
                x = P * (3.0 * a2v + G_ * a4v + F_ * L1v)
            elif bc == 1:
                Am = dcv[:, :, None] * (eye + A_[:, :, None] * B) + 2.0 * P[:, :, None] * (
                    A_[:, :, None] * B * H_[:, :, None] + eye)
                x = -2.0 * P * (A_ * H_ * L1v + 3.0 * a2v + G_ * a4v) - dcv * (a2v + a4v + fv + A_ * L1v)
            else:
                Am = dcv[:, :, None] * (eye + A_[:, :, None] * B)
                x = -dcv * (a2v + a4v + fv + A_ * L1v)
        a1 = torch.linalg.solve(Am, x)
        a3 = A_ * (torch.einsum("ngh,nh->ng", B, a1) + L1v)
        if first:
            jp = -D[ii] * 2.0 / hh * (a1 - 3.0 * a2v + H_ * a3 - G_ * a4v)
            return -(jp / fv + df[ii, :, f])
        jp = -D[ii] * 2.0 / hh * (a1 + 3.0 * a2v + H_ * a3 + G_ * a4v)
        return -(jp / fv - df[ii, :, f])
