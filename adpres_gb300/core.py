"""Host-side mirror of ADPRES's calculation drivers over the C ABI.

``Core`` owns one adp_handle (one core on one GPU).  Its methods follow the
reference's call sequence: ``xs_updt`` is XS_updt (mod_xsec.f90:11-46),
``outer`` is outer/outer_ad (mod_cmfd.f90:415, :602), ``power`` is PowDis
(:1290) and ``forward``/``adjoint`` are control::forward/adjoint
(mod_control.f90:11-86).  Errors come back as AdpError with the status the
reference would have STOPped on.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import AdpError, dptr, iptr


@dataclass
class Report:
    outers: int
    converged: bool
    nodal_updates: int
    keff: float
    ser: float
    fer: float
    ndmax: float
    loc: tuple
    trace_k: np.ndarray
    trace_ser: np.ndarray
    trace_fer: np.ndarray
    trace_flags: np.ndarray
    trace_ndmax: np.ndarray
    device_ms: float


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


def _fortran(a, dt=np.float64):
    """Column-major (node index fastest) copy, the reference's array layout."""
    return np.asfortranarray(a, dtype=dt).reshape(-1, order="F")


class Core:
    """One static k-eigenvalue core on the current CUDA device."""

    def __init__(self, nxx, nyy, nzz, ix, iy, iz, xdel, ydel, zdel, bc, ng, *, nin=2, nout=500, nac=5,
                 nupd=0, serc=0.0, ferc=0.0, kern=2, precision="fp64"):
        self.L = _lib.load()
        self.nnod = int(len(ix))
        self.ng = int(ng)
        self._keep = [_c(ix, np.int32), _c(iy, np.int32), _c(iz, np.int32), _c(xdel), _c(ydel), _c(zdel)]
        ixa, iya, iza, xd, yd, zd = self._keep
        g = _lib.AdpGeom(int(nxx), int(nyy), int(nzz), self.nnod, iptr(ixa), iptr(iya), iptr(iza), dptr(xd),
                         dptr(yd), dptr(zd), *[int(b) for b in bc])
        prec = {"fp64": _lib.ADP_FP64, "mixed": _lib.ADP_MIXED}[precision]
        o = _lib.AdpOpts(self.ng, int(nin), int(nout), int(nac), int(nupd), float(serc), float(ferc), int(kern), prec)
        h = ctypes.c_void_p()
        st = self.L.adp_create(ctypes.byref(g), ctypes.byref(o), ctypes.byref(h))
        if st != 0:
            raise AdpError(st, _lib.last_error(None))
        self.h = h
        self.nout = int(nout) if nout and nout > 0 else 500
        self.precision = precision
        self._fb_cards = []

    @classmethod
    def from_deck(cls, dk, precision="fp64", **over):
        kw = dict(nin=dk.nin, nout=dk.nout, nac=dk.nac, nupd=dk.nupd, serc=dk.serc, ferc=dk.ferc,
                  kern=dk.kern_code, precision=precision)
        kw.update(over)
        core = cls(dk.nxx, dk.nyy, dk.nzz, dk.ix, dk.iy, dk.iz, dk.xdel, dk.ydel, dk.zdel, dk.bc, dk.ng, **kw)
        core.deck = dk
        if getattr(dk, "feedback", None):
            # XS_updt(bcon, ftem, mtem, cden, bpos) with the deck's feedback cards
            core.fb_set(dk)
            core.fb_updt(dk)
        else:
            core.xs_updt(dk.xsigtr, dk.xsiga, dk.xnuf, dk.xsigf, dk.chi, dk.mat, dk.xsigs, dk.dc)
        return core

    def close(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self.L.adp_destroy(h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st != 0:
            raise AdpError(st, _lib.last_error(self.h))

    # -- cross sections -----------------------------------------------------
    def _sized(self, a, n, what):
        """a as given when it holds n values, else an input error."""
        if a is None or np.size(a) != n:
            raise AdpError(_lib.ADP_ERR_INPUT, f"{what}: expected {n} values")
        return a

    def _xs_args(self, rows, tables, chi, mat, sigs, dc):
        """Column-major copies of the four (rows, ng) tables, chi (nmat, ng),
        mat (nnod), sigs (rows, ng, ng) and dc (nnod, ng, 6) or None, after
        checking their sizes (the library reads exactly these many values)."""
        nmat = int(np.asarray(chi).shape[0]) if np.ndim(chi) else 0
        G, nn = self.ng, self.nnod
        rows = nmat if rows == "mat" else nn
        want = [(t, rows * G) for t in tables] + [(chi, nmat * G), (mat, nn), (sigs, rows * G * G)]
        if dc is not None:
            want.append((dc, nn * G * 6))
        for a, n in want:
            if a is None or np.size(a) != n or n == 0:
                raise AdpError(_lib.ADP_ERR_INPUT, "cross-section array of the wrong size")
        args = [_fortran(t) for t in tables] + [_fortran(chi)]
        return (nmat, args, _c(mat, np.int32), _fortran(sigs), None if dc is None else _fortran(dc))

    def xs_updt(self, xsigtr, xsiga, xnuf, xsigf, chi, mat, xsigs, dc=None):
        """XS_updt from material tables (nmat,ng) / (nmat,ng,ng) and mat (nnod,)."""
        nmat, args, m, s, d = self._xs_args("mat", (xsigtr, xsiga, xnuf, xsigf), chi, mat, xsigs, dc)
        self._check(self.L.adp_xs_updt(self.h, nmat, *[dptr(a) for a in args], iptr(m), dptr(s), dptr(d)))

    def xs_updt_nodes(self, sigtr, siga, nuf, sigf, chi, mat, sigs, dc=None):
        """XS_updt from node tables (nnod,ng) / (nnod,ng,ng)."""
        nmat, args, m, s, d = self._xs_args("node", (sigtr, siga, nuf, sigf), chi, mat, sigs, dc)
        self._check(self.L.adp_xs_updt_nodes(self.h, nmat, *[dptr(a) for a in args], iptr(m), dptr(s), dptr(d)))

    def fb_set(self, dk):
        """Upload the deck's feedback tables (adp_fb_set): the material
        tables, the change tables of its state cards (in the reference's
        order boron, fuel temperature, moderator temperature, coolant
        density) and of %CROD, the bank of every node's column."""
        from .feedback import KEYS, STATE_CARDS
        fb = dk.feedback or {}
        keep = []

        def arr(a, dt=np.float64, fortran=True):
            a = _fortran(a, dt) if fortran else _c(a, dt)
            keep.append(a)
            return a

        nmat, G = int(np.asarray(dk.chi).shape[0]), self.ng

        def table_set(tabs):
            for k in KEYS:
                if np.size(tabs[k]) != nmat * G * (G if k == "sigs" else 1):
                    raise AdpError(_lib.ADP_ERR_INPUT, f"feedback table {k} of the wrong size")
            return [dptr(arr(tabs[k])) for k in KEYS]

        if np.size(dk.chi) != nmat * G or np.size(dk.mat) != self.nnod or (
                dk.dc is not None and np.size(dk.dc) != self.nnod * G * 6):
            raise AdpError(_lib.ADP_ERR_INPUT, "chi, mat or dc of the wrong size")
        t = _lib.AdpFbTables()
        t.nmat = nmat
        base = dict(sigtr=dk.xsigtr, siga=dk.xsiga, nuf=dk.xnuf, sigf=dk.xsigf, sigs=dk.xsigs)
        t.xsigtr, t.xsiga, t.xnuf, t.xsigf, t.xsigs = table_set(base)
        t.chi = dptr(arr(dk.chi))
        t.mat = iptr(arr(dk.mat, np.int32, False))
        t.dc = None if dk.dc is None else dptr(arr(dk.dc))
        cards = [(nm, kind) for nm, kind in STATE_CARDS if nm in fb]
        t.nstate = len(cards)
        if cards:
            t.kind = iptr(arr([kind for _, kind in cards], np.int32, False))
            t.ref = dptr(arr([fb[nm]["ref"] for nm, _ in cards], np.float64, False))
            ptrs = [p for nm, _ in cards for p in table_set(fb[nm]["changes"])]
            t.dsig = (_lib._dp * len(ptrs))(*ptrs)
        if "crod" in fb:
            cr = fb["crod"]
            t.nbank = int(cr["nb"])
            t.rsig = (_lib._dp * 5)(*table_set(cr["changes"]))
            bank = np.asarray(cr["fbmap"])[np.asarray(dk.ix) - 1, np.asarray(dk.iy) - 1]
            t.bank = iptr(arr(bank, np.int32, False))
            t.coreh, t.pos0, t.ssize = float(dk.coreh), float(cr["pos0"]), float(cr["ssize"])
        self._check(self.L.adp_fb_set(self.h, ctypes.byref(t)))
        self._fb_cards = [nm for nm, _ in cards]

    def fb_updt(self, dk, bcon=None, bpos=None):
        """XS_updt on the device from the tables of fb_set at the deck's state
        values (boron `bcon` when given) and bank positions (`bpos` when given)."""
        fb = dk.feedback or {}
        vals = [float(bcon) if (nm == "bcon" and bcon is not None) else float(fb[nm]["value"])
                for nm in self._fb_cards]
        st = _c(vals) if vals else None
        bp = None
        if "crod" in fb:
            bp = _c(fb["crod"]["bpos"] if bpos is None else bpos)
            if bp.size != int(fb["crod"]["nb"]):
                raise AdpError(_lib.ADP_ERR_INPUT, "one bank position per rod bank")
        self._check(self.L.adp_fb_updt(self.h, dptr(st), dptr(bp)))

    def set_xs(self, D, sigr, nuf, sigf, chi, mat, sigs, dc=None):
        nmat, args, m, s, d = self._xs_args("node", (D, sigr, nuf, sigf), chi, mat, sigs, dc)
        self._check(self.L.adp_set_xs(self.h, nmat, *[dptr(a) for a in args], iptr(m), dptr(s), dptr(d)))

    # -- solver -------------------------------------------------------------
    def _report(self, trace):
        cap = self.nout if trace else 0
        bufs = [np.zeros(cap) for _ in range(4)] + [np.zeros(cap, dtype=np.int32)]
        rep = _lib.AdpReport()
        rep.trace_cap = cap
        if cap:
            rep.trace_k, rep.trace_ser, rep.trace_fer, rep.trace_ndmax = (dptr(b) for b in bufs[:4])
            rep.trace_flags = iptr(bufs[4])
        return rep, bufs

    @staticmethod
    def _to_report(rep, bufs):
        n = min(rep.outers, rep.trace_cap)
        tk, ts, tf, tn, tfl = bufs
        return Report(rep.outers, bool(rep.converged), rep.nodal_updates, rep.keff, rep.ser, rep.fer, rep.ndmax,
                      (rep.im, rep.jm, rep.km), tk[:n], ts[:n], tf[:n], tfl[:n], tn[:n], rep.device_ms)

    def outer(self, adjoint=False, popt=1, trace=True, frozen_dn=False) -> Report:
        """outer(popt) / outer_ad(popt); frozen_dn keeps dn fixed (no nodal update)."""
        rep, bufs = self._report(trace)
        mode = int(bool(adjoint)) | (_lib.ADP_FROZEN_DN if frozen_dn else 0)
        st = self.L.adp_outer(self.h, mode, int(popt), ctypes.byref(rep))
        self.last_report = self._to_report(rep, bufs)
        self._check(st)
        return self.last_report

    def adjoint_sens(self, tol=0.0, trace=False, frozen_dn=False):
        """dk/dSigma after a converged forward outer.

        The derivative of k at the fixed point of the CMFD eigenproblem and
        the nodal update (adp_adjoint_sens), or with the coupling
        coefficients dn held at the forward solution (frozen_dn=True,
        adp_adjoint_sens_frozen).  Returns (dkdp (nnod, ng, 4 + ng),
        psi (nnod, ng), Report); dkdp[:, g, c] for c = 0 D, 1 siga, 2 nuf,
        3 sigtr, 4 + h sigs(g->h).
        """
        nn, G = self.nnod, self.ng
        dk = np.zeros(nn * G * (4 + G))
        psi = np.zeros(nn * G)
        rep, bufs = self._report(trace)
        fn = self.L.adp_adjoint_sens_frozen if frozen_dn else self.L.adp_adjoint_sens
        st = fn(self.h, float(tol), dptr(dk), dptr(psi), ctypes.byref(rep))
        r = self._to_report(rep, bufs)
        self.last_adjoint_ms = rep.device_ms
        self._check(st)
        return dk.reshape((nn, G, 4 + G), order="F"), psi.reshape((nn, G), order="F"), r

    def matrix(self):
        """adp_get_matrix: the CMFD matrix (nnod, ng, 7), columns z-, y-, x-, diag, x+, y+, z+."""
        a = np.zeros(self.nnod * self.ng * 7)
        self._check(self.L.adp_get_matrix(self.h, dptr(a)))
        return a.reshape((self.nnod, self.ng, 7), order="F")

    def nodal_step(self):
        """adp_nodal_step: one nodal update at the current state; Report with ndmax and loc."""
        rep, bufs = self._report(False)
        st = self.L.adp_nodal_step(self.h, ctypes.byref(rep))
        r = self._to_report(rep, bufs)
        self._check(st)
        return r

    def nodal_sources(self):
        """adp_get_nodal_sources: S1..S3 of the last nodal update, (nnod, ng, 3)."""
        s = np.zeros(self.nnod * self.ng * 3)
        self._check(self.L.adp_get_nodal_sources(self.h, dptr(s)))
        return s.reshape((self.nnod, self.ng, 3), order="F")

    def set_wait_limit(self, seconds):
        """adp_set_wait_limit: time limit of a grid-barrier wait (0: 2 s)."""
        self._check(self.L.adp_set_wait_limit(self.h, float(seconds)))

    def test_missing_block(self, on=True):
        """adp_test_missing_block: make every barrier wait of the next forward
        outers run out (ADP_ERR_TIMEOUT), for tests of the timeout path."""
        self._check(self.L.adp_test_missing_block(self.h, int(bool(on))))

    def nodal_vjp(self, lam):
        """adp_nodal_vjp: lam (nnod, ng, 6) -> (phibar (nnod, ng), dnbar
        (nnod, ng, 6), kbar, sigbar (nnod, ng, 4 + ng), residual)."""
        nn, G = self.nnod, self.ng
        lam = np.asfortranarray(lam, dtype=np.float64).reshape(-1, order="F")
        if lam.size != nn * G * 6:
            raise ValueError("lam must hold nnod * ng * 6 values")
        pb = np.zeros(nn * G)
        db = np.zeros(nn * G * 6)
        sb = np.zeros(nn * G * (4 + G))
        kb, rs = ctypes.c_double(), ctypes.c_double()
        self._check(self.L.adp_nodal_vjp(self.h, dptr(lam), dptr(pb), dptr(db), ctypes.byref(kb), dptr(sb),
                                         ctypes.byref(rs)))
        return (pb.reshape((nn, G), order="F"), db.reshape((nn, G, 6), order="F"), kb.value,
                sb.reshape((nn, G, 4 + G), order="F"), rs.value)

    def state(self):
        """(f0 (nnod,ng), fs0 (nnod,), keff, dn (nnod,ng,6)) in the reference layouts."""
        f0 = np.zeros(self.nnod * self.ng)
        fs0 = np.zeros(self.nnod)
        dn = np.zeros(self.nnod * self.ng * 6)
        k = ctypes.c_double()
        self._check(self.L.adp_get_state(self.h, dptr(f0), dptr(fs0), ctypes.byref(k), dptr(dn)))
        return (f0.reshape((self.nnod, self.ng), order="F"), fs0, k.value,
                dn.reshape((self.nnod, self.ng, 6), order="F"))

    def flux(self):
        """f0 (nnod, ng) of the current state, without the other state arrays."""
        f0 = np.zeros(self.nnod * self.ng)
        self._check(self.L.adp_get_state(self.h, dptr(f0), None, None, None))
        return f0.reshape((self.nnod, self.ng), order="F")

    def set_state(self, f0=None, fs0=None, keff=None, dn=None):
        nn, G = self.nnod, self.ng
        a = None if f0 is None else _fortran(self._sized(f0, nn * G, "f0 (nnod, ng)"))
        b = None if fs0 is None else _c(self._sized(fs0, nn, "fs0 (nnod)"))
        d = None if dn is None else _fortran(self._sized(dn, nn * G * 6, "dn (nnod, ng, 6)"))
        k = None if keff is None else ctypes.byref(ctypes.c_double(keff))
        self._check(self.L.adp_set_state(self.h, dptr(a), dptr(b), k, dptr(d)))

    def reset(self):
        """Back to the state of a fresh process (dn = 0; next outer starts from f0 = 1, k = 1)."""
        self._check(self.L.adp_reset(self.h))

    def power(self):
        p = np.zeros(self.nnod)
        self._check(self.L.adp_power(self.h, dptr(p)))
        return p

    def timers(self):
        t = _lib.AdpTimers()
        self._check(self.L.adp_get_timers(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    # -- rod ejection transient (mod_trans.f90) -------------------------------
    def trans_init(self, beta, lamb, velo, theta, extr, af):
        """adp_trans_init after the steady state: af (nnod, ng) adjoint weight.
        Returns the t = 0 record (rho absolute, relative power 1)."""
        self._trans_keep = [_c(beta), _c(lamb), _c(self._sized(velo, self.ng, "velo (ng)"))]
        b, l, v = self._trans_keep
        self._sized(l, b.size, "one decay constant per delayed family")
        o = _lib.AdpTransOpts(len(b), dptr(b), dptr(l), dptr(v), float(theta), int(bool(extr)))
        r = _lib.AdpTransResult()
        a = _fortran(self._sized(af, self.nnod * self.ng, "af (nnod, ng)"))
        self._check(self.L.adp_trans_init(self.h, ctypes.byref(o), dptr(a), ctypes.byref(r)))
        return r

    def trans_step(self, dt, omeg_mode):
        """adp_trans_step: one time step after the step's cross sections are set."""
        r = _lib.AdpTransResult()
        self._check(self.L.adp_trans_step(self.h, float(dt), int(omeg_mode), ctypes.byref(r)))
        return r

    def set_launch(self, blocks=0, threads=0):
        self._check(self.L.adp_set_launch(self.h, int(blocks), int(threads)))

    # -- adjoint-weighted edits (mod_trans.f90:648-746) ------------------------
    def reactivity(self, af, sigrp=None):
        """reactivity: (src - lea - rem) / fde of the current state weighted by af (nnod, ng)."""
        nn, G = self.nnod, self.ng
        a = _fortran(self._sized(af, nn * G, "af (nnod, ng)"))
        s = None if sigrp is None else _fortran(self._sized(sigrp, nn * G, "sigrp (nnod, ng)"))
        rho = ctypes.c_double()
        self._check(self.L.adp_reactivity(self.h, dptr(a), dptr(s), ctypes.byref(rho)))
        return rho.value

    def core_beta(self, af, ibeta, mat):
        """calc_beta: delayed fraction weighted by af, ibeta (nmat, nf), mat (nnod,) 1-based."""
        a = _fortran(self._sized(af, self.nnod * self.ng, "af (nnod, ng)"))
        ib = np.asfortranarray(ibeta, dtype=np.float64)
        if ib.ndim != 2:
            raise AdpError(_lib.ADP_ERR_INPUT, "ibeta: a (nmat, nf) table")
        m = _c(self._sized(mat, self.nnod, "mat (nnod)"), np.int32)
        beta = ctypes.c_double()
        self._check(self.L.adp_core_beta(self.h, dptr(a), int(ib.shape[0]), int(ib.shape[1]),
                                         dptr(ib.reshape(-1, order="F")), iptr(m), ctypes.byref(beta)))
        return beta.value

    # -- output edits (mod_io.f90:3267-3644) ----------------------------------
    def _divs(self, name, div):
        if div is None:
            div = getattr(self, "deck", None).extra[name]
        return np.ascontiguousarray(div, dtype=np.int32)

    def asmpow(self, xdiv=None, ydiv=None):
        """AsmPow: (fasm (nx, ny), (imax, jmax)); divisions default to the deck's."""
        xd, yd = self._divs("xdiv", xdiv), self._divs("ydiv", ydiv)
        out = np.zeros(len(xd) * len(yd))
        im, jm = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.adp_edit_asmpow(self.h, len(xd), len(yd), iptr(xd), iptr(yd), dptr(out), ctypes.byref(im),
                                           ctypes.byref(jm)))
        return out.reshape((len(xd), len(yd)), order="F"), (im.value, jm.value)

    def axipow(self, zdiv=None):
        """AxiPow: (faxi (nz,), kmax)."""
        zd = self._divs("zdiv", zdiv)
        out = np.zeros(len(zd))
        km = ctypes.c_int()
        self._check(self.L.adp_edit_axipow(self.h, len(zd), iptr(zd), dptr(out), ctypes.byref(km)))
        return out, km.value

    def asmflux(self, xdiv=None, ydiv=None, norm=1.0):
        """AsmFlux: (fasm (nx, ny, ng), negative)."""
        xd, yd = self._divs("xdiv", xdiv), self._divs("ydiv", ydiv)
        out = np.zeros(len(xd) * len(yd) * self.ng)
        neg = ctypes.c_int()
        self._check(self.L.adp_edit_asmflux(self.h, len(xd), len(yd), iptr(xd), iptr(yd), float(norm), dptr(out),
                                            ctypes.byref(neg)))
        return out.reshape((len(xd), len(yd), self.ng), order="F"), bool(neg.value)

    # -- calculation modes (mod_control.f90:11-86) ---------------------------
    def forward(self):
        rep = self.outer(adjoint=False, popt=1)
        return rep, self.power()

    def adjoint(self):
        rep = self.outer(adjoint=True, popt=1)
        return rep, self.power()


def solve_deck(dk, precision="fp64"):
    """control::forward / control::adjoint for a parsed deck: (report, power, core).

    In mode BCSEARCH (th::cbsearch, mod_th.f90:752-837) the report is the last
    outer of the critical boron search and core.bcsearch holds its iterates
    (bcon, k, outers); in mode RODEJECT the report is the last steady-state
    outer and core.transient holds the time steps (adpres_gb300.transient)."""
    core = Core.from_deck(dk, precision=precision)
    if dk.mode == "BCSEARCH":
        from .feedback import cbsearch
        core.bcsearch = cbsearch(core, dk)
        return core.last_report, core.power(), core
    if dk.mode == "RODEJECT":
        # rod_eject (mod_trans.f90:17-160): core.transient holds the records
        from .transient import rod_eject
        core.transient = rod_eject(core, dk)
        return core.last_report, core.power(), core
    rep, p = core.adjoint() if dk.adjoint else core.forward()
    return rep, p, core
