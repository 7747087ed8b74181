"""ORACLE -- test infrastructure only.

CPU restatement of the ADPRES static k-eigenvalue path (adpres_oracle.cpp),
exposed through ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker of the CUDA path; the product never routes through it.

Parity pin: the restatement reproduces the reference's printed IAEA3D
convergence trace (docs/quick-guides.md:161-191 of the ADPRES project) digit
for digit; see tests/test_oracle_golden.py.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "adpres_oracle.cpp")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libadpres_oracle.so")
# Variants used only to measure how sensitive a deck is to rounding:
#   "fma"       the same source with multiply-add contraction (FMA on x86-64 and Arm);
#   "fma_rhost" also forming BiCGSTAB's (rs, r) as (rs,s) - omega (rs,t), an
#               algebraically equal evaluation that the CUDA path uses.
LIB_FMA = os.path.join(BUILD_DIR, "libadpres_oracle_fma.so")
VARIANTS = {
    "plain": (LIB, ["-ffp-contract=off"]),
    "fma": (LIB_FMA, ["-ffp-contract=fast"]),
    "fma_rhost": (os.path.join(BUILD_DIR, "libadpres_oracle_fma_rhost.so"),
                  ["-ffp-contract=fast", "-DORA_RHO_FROM_S_T"]),
}

# Status codes (same meaning as the product's adp_status values).
ORA_OK = 0
ORA_ERR_INPUT = 1
ORA_ERR_BADXS = 2
ORA_ERR_PIVOT = 3
ORA_ERR_DIVERGED = 4
ORA_ERR_MAXOUTER = 5
ORA_ERR_ZEROPOWER = 6
ORA_ERR_UNSUPPORTED = 7


def build(force: bool = False, variant: str = "plain") -> str:
    """Compile the restatement with g++ into _build/.

    variant "plain" (the oracle): no multiply-add contraction, as the
    reference's gfortran build for x86-64 has none.  The other VARIANTS are
    used only to measure rounding sensitivity.
    """
    os.makedirs(BUILD_DIR, exist_ok=True)
    lib_path, fp = VARIANTS[variant]
    if (not force and os.path.exists(lib_path)
            and os.path.getmtime(lib_path) >= os.path.getmtime(SRC)):
        return lib_path
    tmp = lib_path + ".tmp.%d" % os.getpid()
    if variant != "plain" and platform.machine() in ("x86_64", "AMD64"):
        fp = fp + ["-mfma"]
    cmd = ["g++", "-O2", "-std=c++17"] + fp + ["-fno-fast-math", "-fPIC", "-shared", SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib_path)
    return lib_path


_libs = {}


def lib(variant: str = "plain"):
    if variant not in _libs:
        path = build(variant=variant)
        L = ctypes.CDLL(path)
        vp, cp, ip, dp = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        ipp = ctypes.POINTER(ctypes.c_int)
        L.ora_global_error.restype = cp
        L.ora_load_deck_text.restype = vp
        L.ora_load_deck_text.argtypes = [cp, cp]
        L.ora_load_deck.restype = vp
        L.ora_load_deck.argtypes = [cp]
        L.ora_free.argtypes = [vp]
        L.ora_error.restype = cp
        L.ora_error.argtypes = [vp]
        for name in ("ora_xs_updt", "ora_dsigr_updt"):
            getattr(L, name).argtypes = [vp]
        L.ora_outer.argtypes = [vp, ip, ip, ip]
        L.ora_powdis.argtypes = [vp, dp]
        L.ora_matrix_setup.argtypes = [vp, ip]
        L.ora_nodal_upd.argtypes = [vp, ip]
        L.ora_group_solve.argtypes = [vp, ip, ip, dp]
        L.ora_bicg.argtypes = [vp, ip, ip, dp, dp]
        L.ora_get_matrix7.argtypes = [vp, dp]
        L.ora_get_int.argtypes = [vp, cp]
        L.ora_get_double.restype = ctypes.c_double
        L.ora_get_double.argtypes = [vp, cp]
        L.ora_set_double.argtypes = [vp, cp, ctypes.c_double]
        L.ora_set_int.argtypes = [vp, cp, ip]
        L.ora_array_len.restype = ctypes.c_long
        L.ora_array_len.argtypes = [vp, cp]
        L.ora_get_array.argtypes = [vp, cp, dp]
        L.ora_set_array.argtypes = [vp, cp, dp]
        L.ora_get_iarray.argtypes = [vp, cp, ipp]
        L.ora_get_trace.argtypes = [vp, ipp, dp, dp, dp, ipp, dp, ipp]
        L.ora_reset.argtypes = [vp]
        L.ora_asmpow.argtypes = [vp, dp, dp, ipp, ipp]
        L.ora_reactivity.argtypes = [vp, dp, dp, dp]
        L.ora_cbsearch.argtypes = [vp, dp, dp, ipp, ip, ipp]
        L.ora_xs_updt_at.argtypes = [vp, ctypes.c_double]
        L.ora_rodeject.argtypes = [vp, dp, dp, dp, ipp, ipp, ip, ip, ipp]
        L.ora_calc_beta.argtypes = [vp, dp, ip, dp, dp]
        L.ora_axipow.argtypes = [vp, dp, dp, ipp]
        L.ora_asmflux.argtypes = [vp, dp, ctypes.c_double, dp, ipp]
        _libs[variant] = L
    return _libs[variant]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


@dataclass
class TraceRow:
    p: int
    k: float
    ser: float
    fer: float
    extrapolated: bool
    nodal: bool
    ndmax: float
    loc: tuple


class Oracle:
    """One reference-state instance (the equivalent of one ADPRES process)."""

    def __init__(self, deck_path: str | None = None, text: str | None = None, basedir: str = ".",
                 variant: str = "plain"):
        L = lib(variant)
        if deck_path is not None:
            h = L.ora_load_deck(deck_path.encode())
        else:
            h = L.ora_load_deck_text(text.encode(), basedir.encode())
        if not h:
            msg = L.ora_global_error().decode()
            code = ORA_ERR_UNSUPPORTED if "outside the static" in msg else ORA_ERR_INPUT
            raise OracleError(code, msg)
        self.h = ctypes.c_void_p(h)
        self.L = L

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self.L.ora_free(h)
            self.h = None

    def _check(self, st):
        if st != ORA_OK:
            raise OracleError(st, self.L.ora_error(self.h).decode())

    # -- drivers -----------------------------------------------------------
    def xs_updt(self):
        self._check(self.L.ora_xs_updt(self.h))

    def dsigr_updt(self):
        self._check(self.L.ora_dsigr_updt(self.h))

    def outer(self, adjoint=False, popt=1, max_outers=0):
        self._check(self.L.ora_outer(self.h, int(adjoint), popt, max_outers))

    def run(self):
        """control::forward / control::adjoint (mod_control.f90:11-86), or
        th::cbsearch (mod_th.f90:752-837) in mode BCSEARCH."""
        if self.geti("bcsearch"):
            return self.cbsearch()
        if self.geti("rodeject"):
            return self.rodeject()
        self.xs_updt()
        self.outer(adjoint=bool(self.geti("adjoint")), popt=1)

    def cbsearch(self, cap=64):
        """Critical boron search: list of (bcon, k, outers) iterates; the last is critical."""
        bc, k = np.zeros(cap), np.zeros(cap)
        no = np.zeros(cap, dtype=np.int32)
        n = ctypes.c_int()
        self._check(self.L.ora_cbsearch(self.h, _dp(bc), _dp(k), _ip(no), cap, ctypes.byref(n)))
        m = min(n.value, cap)
        return [(float(bc[i]), float(k[i]), int(no[i])) for i in range(m)]

    def rodeject(self, cap=20000, max_steps=-1):
        """rod_eject (mod_trans.f90:17-160): list of (t, rho, relative power,
        nout reached, outers); rho is in dollars after t = 0 and absolute at t = 0."""
        t, rho, pw = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        mx, no = np.zeros(cap, dtype=np.int32), np.zeros(cap, dtype=np.int32)
        n = ctypes.c_int()
        self._check(self.L.ora_rodeject(self.h, _dp(t), _dp(rho), _dp(pw), _ip(mx), _ip(no), cap, int(max_steps),
                                        ctypes.byref(n)))
        m = min(n.value, cap)
        return [(float(t[i]), float(rho[i]), float(pw[i]), bool(mx[i]), int(no[i])) for i in range(m)]

    def xs_updt_at(self, bcon):
        """XS_updt with the boron concentration bcon (feedback cards applied)."""
        self._check(self.L.ora_xs_updt_at(self.h, float(bcon)))

    def powdis(self):
        p = np.zeros(self.geti("nnod"))
        self._check(self.L.ora_powdis(self.h, _dp(p)))
        return p

    # -- adjoint-weighted edits (mod_trans.f90:648-746) ------------------------
    def reactivity(self, af, sigrp=None):
        """reactivity(af, sigrp): adjoint-weighted balance of the current state."""
        a = np.asfortranarray(af, dtype=np.float64).reshape(-1, order="F")
        s = None if sigrp is None else np.asfortranarray(sigrp, dtype=np.float64).reshape(-1, order="F")
        rho = ctypes.c_double()
        self._check(self.L.ora_reactivity(self.h, _dp(a), _dp(s) if s is not None else None, ctypes.byref(rho)))
        return rho.value

    def calc_beta(self, af, ibeta):
        """calc_beta(af) with delayed fractions ibeta (nmat, nf)."""
        a = np.asfortranarray(af, dtype=np.float64).reshape(-1, order="F")
        ib = np.asfortranarray(ibeta, dtype=np.float64)
        beta = ctypes.c_double()
        self._check(self.L.ora_calc_beta(self.h, _dp(a), int(ib.shape[1]), _dp(ib.reshape(-1, order="F")),
                                         ctypes.byref(beta)))
        return beta.value

    # -- output edits of control::forward (mod_io.f90:3267-3644) ---------------
    def asmpow(self, fn):
        """AsmPow: (fasm (nx, ny), (imax, jmax)) of a node field such as PowDis."""
        nx, ny = self.geti("nx"), self.geti("ny")
        out = np.zeros(nx * ny)
        im, jm = ctypes.c_int(), ctypes.c_int()
        self._check(self.L.ora_asmpow(self.h, _dp(np.ascontiguousarray(fn, dtype=np.float64)), _dp(out),
                                      ctypes.byref(im), ctypes.byref(jm)))
        return out.reshape((nx, ny), order="F"), (im.value, jm.value)

    def axipow(self, fn):
        """AxiPow: (faxi (nz,), kmax)."""
        out = np.zeros(self.geti("nz"))
        km = ctypes.c_int()
        self._check(self.L.ora_axipow(self.h, _dp(np.ascontiguousarray(fn, dtype=np.float64)), _dp(out),
                                      ctypes.byref(km)))
        return out, km.value

    def asmflux(self, f=None, norm=1.0):
        """AsmFlux of f (nnod, ng) (default: the oracle's f0): (fasm (nx, ny, ng), negative)."""
        nx, ny, ng = self.geti("nx"), self.geti("ny"), self.geti("ng")
        out = np.zeros(nx * ny * ng)
        neg = ctypes.c_int()
        fa = None if f is None else np.asfortranarray(f, dtype=np.float64).reshape(-1, order="F")
        self._check(self.L.ora_asmflux(self.h, _dp(fa) if fa is not None else None, float(norm), _dp(out),
                                       ctypes.byref(neg)))
        return out.reshape((nx, ny, ng), order="F"), bool(neg.value)

    def matrix_setup(self, opt=1):
        self._check(self.L.ora_matrix_setup(self.h, opt))

    def nodal_upd(self, nmode=1):
        self._check(self.L.ora_nodal_upd(self.h, nmode))

    def group_solve(self, g, adjoint=False):
        bs = np.zeros(self.geti("nnod"))
        self._check(self.L.ora_group_solve(self.h, g, int(adjoint), _dp(bs)))
        return bs

    def bicg(self, g, b, x, imax=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x, dtype=np.float64)
        self._check(self.L.ora_bicg(self.h, g, imax or self.geti("nin"), _dp(b), _dp(x)))
        return x

    def matrix7(self):
        out = np.zeros((self.geti("ng"), self.geti("nnod"), 7))
        self._check(self.L.ora_get_matrix7(self.h, _dp(out)))
        return out

    def reset(self):
        self.L.ora_reset(self.h)

    # -- accessors ---------------------------------------------------------
    def geti(self, name):
        return self.L.ora_get_int(self.h, name.encode())

    def getd(self, name):
        return self.L.ora_get_double(self.h, name.encode())

    def setd(self, name, v):
        assert self.L.ora_set_double(self.h, name.encode(), float(v)) == 0

    def seti(self, name, v):
        assert self.L.ora_set_int(self.h, name.encode(), int(v)) == 0

    def array(self, name):
        n = self.L.ora_array_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        if self.L.ora_get_array(self.h, name.encode(), _dp(out)) != 0:
            out = np.zeros(n, dtype=np.int32)
            if self.L.ora_get_iarray(self.h, name.encode(), _ip(out)) != 0:
                raise KeyError(name)
        return out

    def set_array(self, name, values):
        n = self.L.ora_array_len(self.h, name.encode())
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        assert v.size == n, (name, v.size, n)
        assert self.L.ora_set_array(self.h, name.encode(), _dp(v)) == 0

    def fortran(self, name, shape):
        """Array in its Fortran (column-major) shape, e.g. ('f0', (nnod, ng))."""
        return self.array(name).reshape(shape, order="F")

    def trace(self):
        n = self.geti("trace_len")
        ip = np.zeros(n, dtype=np.int32)
        k, ser, fer, nd = (np.zeros(n) for _ in range(4))
        fl = np.zeros(n, dtype=np.int32)
        loc = np.zeros(3 * n, dtype=np.int32)
        self.L.ora_get_trace(self.h, _ip(ip), _dp(k), _dp(ser), _dp(fer), _ip(fl), _dp(nd), _ip(loc))
        return [TraceRow(int(ip[t]), float(k[t]), float(ser[t]), float(fer[t]), bool(fl[t] & 1),
                         bool(fl[t] & 2), float(nd[t]), tuple(int(v) for v in loc[3 * t:3 * t + 3]))
                for t in range(n)]
