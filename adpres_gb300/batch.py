"""Batched static solves over the C ABI (adp_batch_*).

``Batch`` holds many independent cores (same group count, kernel and
precision) and solves them in one persistent cooperative launch replayed
from a CUDA graph.  ``autotune`` runs the library's autotuner (block size,
largest team, grain; schedules built from measured per-core times) and can
keep its choice in a JSON cache keyed by the batch's shape, so the next
process with the same batch starts from the tuned configuration.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os

import numpy as np

from . import _lib
from ._lib import AdpError, dptr, iptr
from .core import _c, _fortran

# Tuned configurations measured on GPU models, keyed "<device>:<signature>".
TUNED_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "batch_tuned.json")


def _batch_error(h):
    L = _lib.load()
    buf = ctypes.create_string_buffer(2048)
    L.adp_batch_last_error(h, buf, 2048)
    return buf.value.decode(errors="replace")


def node_tables(dk):
    """Node-wise cross sections (nnod, ng[, ng]) from a deck's material tables."""
    m = dk.mat - 1
    return dict(sigtr=dk.xsigtr[m], siga=dk.xsiga[m], nuf=dk.xnuf[m], sigf=dk.xsigf[m], sigs=dk.xsigs[m])


def _read_cache(path):
    """The tuning cache, or {} when it is absent or unreadable (a cache is
    an optimisation: a damaged one costs a tuning run, not the solve)."""
    try:
        with open(path) as f:
            db = json.load(f)
        return db if isinstance(db, dict) else {}
    except (OSError, ValueError):
        return {}


def _write_cache(path, db):
    """Write the cache through a file of this process and an atomic rename,
    so that processes sharing the path (one per GPU) never read a partial
    file; the last writer's entries win."""
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    tmp = os.path.join(d, ".%s.%d.tmp" % (os.path.basename(path), os.getpid()))
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1)
    os.replace(tmp, path)


class Batch:
    def __init__(self, decks, precision="mixed", **over):
        self.L = _lib.load()
        self.decks = list(decks)
        n = len(self.decks)
        prec = {"fp64": _lib.ADP_FP64, "mixed": _lib.ADP_MIXED}[precision]
        self._keep = []
        geoms = (_lib.AdpGeom * n)()
        opts = (_lib.AdpOpts * n)()
        for i, dk in enumerate(self.decks):
            arrs = [_c(dk.ix, np.int32), _c(dk.iy, np.int32), _c(dk.iz, np.int32), _c(dk.xdel), _c(dk.ydel),
                    _c(dk.zdel)]
            self._keep.append(arrs)
            geoms[i] = _lib.AdpGeom(int(dk.nxx), int(dk.nyy), int(dk.nzz), int(len(dk.ix)), iptr(arrs[0]),
                                    iptr(arrs[1]), iptr(arrs[2]), dptr(arrs[3]), dptr(arrs[4]), dptr(arrs[5]),
                                    *[int(b) for b in dk.bc])
            kw = dict(nin=dk.nin, nout=dk.nout, nac=dk.nac, nupd=dk.nupd, serc=dk.serc, ferc=dk.ferc)
            kw.update(over)
            opts[i] = _lib.AdpOpts(int(dk.ng), int(kw["nin"]), int(kw["nout"]), int(kw["nac"]), int(kw["nupd"]),
                                   float(kw["serc"]), float(kw["ferc"]), int(dk.kern_code), prec)
        h = ctypes.c_void_p()
        st = self.L.adp_batch_create(n, geoms, opts, ctypes.byref(h))
        if st != 0:
            raise AdpError(st, _lib.last_error(None))
        self.h = h
        self.n = n
        self.precision = precision
        self.nnod = [int(len(dk.ix)) for dk in self.decks]
        for i, dk in enumerate(self.decks):
            t = node_tables(dk)
            self.set_xs(i, t["sigtr"], t["siga"], t["nuf"], t["sigf"], dk.chi, dk.mat, t["sigs"], dk.dc)

    def close(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self.L.adp_batch_destroy(h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            raise AdpError(st, _batch_error(self.h))

    def set_xs(self, i, sigtr, siga, nuf, sigf, chi, mat, sigs, dc=None):
        nmat = int(np.asarray(chi).shape[0])
        a = [_fortran(sigtr), _fortran(siga), _fortran(nuf), _fortran(sigf), _fortran(chi)]
        m = _c(mat, np.int32)
        s = _fortran(sigs)
        d = None if dc is None else _fortran(dc)
        self._check(self.L.adp_batch_set_xs(self.h, int(i), nmat, *[dptr(x) for x in a], iptr(m), dptr(s), dptr(d)))

    # -- configuration --------------------------------------------------------
    def config(self):
        c = _lib.AdpBatchConfig()
        self._check(self.L.adp_batch_get_config(self.h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in c._fields_}

    def set_config(self, **kw):
        cfg = self.config()
        cfg.update(kw)
        c = _lib.AdpBatchConfig(**cfg)
        self._check(self.L.adp_batch_set_config(self.h, ctypes.byref(c)))

    def signature(self):
        """Key of the tuning cache: the shapes and options of every core."""
        parts = [self.precision, str(self.n)]
        for dk in self.decks:
            parts.append(f"{dk.nxx}x{dk.nyy}x{dk.nzz}:{len(dk.ix)}:{dk.ng}:{dk.kern_code}")
        return hashlib.sha1("|".join(parts).encode()).hexdigest()

    def autotune(self, cache=None, device=None):
        """Run the library autotuner; with a cache path, reuse or store the choice.

        device: a key of the GPU model (for example "sm103x152": compute
        capability and SM count); with it, the configurations measured on
        that model and shipped with the package (batch_tuned.json) are
        consulted first, read-only, so a fresh machine of a tuned model
        starts tuned."""
        key = self.signature()
        if device:
            key = device + ":" + key
            if os.path.exists(TUNED_PATH):
                with open(TUNED_PATH) as f:
                    shipped = json.load(f)
                if key in shipped:
                    self.apply_config(shipped[key]["config"])
                    return shipped[key]["config"], shipped[key]["ms"], True
        if cache:
            db = _read_cache(cache)
            if key in db:
                self.apply_config(db[key]["config"])
                return db[key]["config"], db[key]["ms"], True
        c = _lib.AdpBatchConfig()
        ms = ctypes.c_double()
        self._check(self.L.adp_batch_autotune(self.h, ctypes.byref(c), ctypes.byref(ms)))
        cfg = {k: getattr(c, k) for k, _ in c._fields_}
        if cache:
            db = _read_cache(cache)
            db[key] = {"config": cfg, "ms": ms.value}
            _write_cache(cache, db)
        return cfg, ms.value, False

    def apply_config(self, cfg, rounds=3):
        """Set a configuration (a cached or shipped one) and settle its
        schedule: `rounds` solves, each followed by a re-plan with the
        per-core times gathered so far (the plan before any solve weighs
        cores by box rows x groups; each re-plan adds the times of the team
        sizes the last plan chose)."""
        self.set_config(**cfg)
        for _ in range(rounds):
            self.solve(check=False)
            self.set_config(**cfg)

    # -- solve and results ----------------------------------------------------
    def solve(self, check=True):
        res = (_lib.AdpBatchResult * self.n)()
        ms = ctypes.c_double()
        st = self.L.adp_batch_solve(self.h, res, ctypes.byref(ms))
        out = [{k: getattr(r, k) for k, _ in r._fields_} for r in res]
        if check:
            self._check(st)
        return out, ms.value

    def trace(self, i):
        """Per-outer (k, ser, fer, flags, ndmax) of core i from the last solve."""
        cap = int(self.decks[i].nout)
        k, ser, fer, nd = (np.zeros(cap) for _ in range(4))
        fl = np.zeros(cap, dtype=np.int32)
        n = self.L.adp_batch_trace(self.h, int(i), cap, dptr(k), dptr(ser), dptr(fer), iptr(fl), dptr(nd))
        if n < 0:
            raise AdpError(_lib.ADP_ERR_INPUT, "adp_batch_trace: bad arguments")
        return k[:n], ser[:n], fer[:n], fl[:n], nd[:n]

    def power(self, i):
        p = np.zeros(self.nnod[i])
        self._check(self.L.adp_batch_power(self.h, int(i), dptr(p)))
        return p

    def state(self, i):
        """(f0 (nnod, ng), keff) of core i after a solve."""
        h = ctypes.c_void_p()
        self._check(self.L.adp_batch_core(self.h, int(i), ctypes.byref(h)))
        dk = self.decks[i]
        f0 = np.zeros(self.nnod[i] * dk.ng)
        k = ctypes.c_double()
        st = self.L.adp_get_state(h, dptr(f0), None, ctypes.byref(k), None)
        if st != 0:
            raise AdpError(st, _lib.last_error(h))
        return f0.reshape((self.nnod[i], dk.ng), order="F"), k.value
