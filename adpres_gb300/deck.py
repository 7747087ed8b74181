"""Reader of ADPRES input decks for the static k-eigenvalue path.

Cards handled as in src/mod_io.f90: %MODE (:580-640), %CASE, %XSEC
(:683-805), %GEOM (:809-1289 with the node ordering of misc, :1293-1365),
%ADF with rotations (:1732-2144), %ITER (:1522-1569), %KERN (:1593-1646)
and %PRNT (:1693-1728); the feedback cards %CROD, %CBCS, %BCON, %FTEM,
%MTEM, %CDEN (:2148-2954) and the transient cards %EJCT, %THET, %EXTR
(:1650-1689, :2332-2482); comments after '!' (:452-492) and the FILE
include keyword (:519-535).  %ESRC (fixed source), %THER (thermal
hydraulics) and %XTAB (branch tables) raise DeckError with
ADP_ERR_UNSUPPORTED.

The result is the reference's sdata state for this path: geometry and node
order, material cross sections, ADFs per node, iteration control.
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field

import numpy as np

from ._lib import ADP_ERR_INPUT, ADP_ERR_BADXS, ADP_ERR_UNSUPPORTED

KNOWN_CARDS = ("MODE", "XSEC", "GEOM", "CASE", "ESRC", "ITER", "PRNT", "ADF", "CROD", "EJCT", "CBCS",
               "FTEM", "MTEM", "CDEN", "BCON", "THER", "XTAB", "KERN", "EXTR", "THET")
OUT_OF_SCOPE = ("ESRC", "THER", "XTAB")

F_1EM5 = float(np.float32(1.e-5))   # default serc/ferc (mod_data.f90:78-79)


class DeckError(ValueError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


@dataclass
class Deck:
    mode: str = "FORWARD"
    kern: str = "SANM"                 # FDM, PNM or SANM
    ng: int = 0
    nmat: int = 0
    xsigtr: np.ndarray = None          # (nmat, ng)
    xsiga: np.ndarray = None
    xnuf: np.ndarray = None
    xsigf: np.ndarray = None
    chi: np.ndarray = None
    xsigs: np.ndarray = None           # (nmat, ng, ng), g -> h
    nx: int = 0
    ny: int = 0
    nz: int = 0
    nxx: int = 0
    nyy: int = 0
    nzz: int = 0
    xdel: np.ndarray = None
    ydel: np.ndarray = None
    zdel: np.ndarray = None
    bc: tuple = (0, 0, 0, 0, 0, 0)     # east, west, north, south, bottom, top
    nnod: int = 0
    ix: np.ndarray = None              # 1-based, reference node order
    iy: np.ndarray = None
    iz: np.ndarray = None
    mat: np.ndarray = None             # 1-based
    dc: np.ndarray = None              # (nnod, ng, 6)
    nin: int = 2
    nout: int = 500
    serc: float = F_1EM5
    ferc: float = F_1EM5
    nac: int = 5
    nupd: int = 0
    prnt: tuple = (1, 1, 1)
    coreh: float = 0.0                 # core height, the sum of zdel
    # feedback cards: "bcon", "ftem", "mtem", "cden" -> dict(value, ref,
    # changes); "crod" -> dict(nb, nstep, pos0, ssize, bpos, fbmap, changes);
    # changes = sigtr, siga, nuf, sigf (nmat, ng) and sigs (nmat, ng, ng)
    feedback: dict = field(default_factory=dict)
    bcbcs: bool = False                # %CBCS given (critical boron search)
    # rod ejection transient (%EJCT, %THET, %EXTR): fbpos, tmove, bspeed,
    # mdir (nb); ttot, tstep1, tdiv, tstep2; beta, lamb (6); velo (ng);
    # theta (default 1, fully implicit); extr
    trans: dict = field(default_factory=lambda: {"theta": 1.0, "extr": False})
    extra: dict = field(default_factory=dict)

    @property
    def kern_code(self) -> int:
        return {"FDM": 0, "PNM": 1, "SANM": 2}[self.kern]

    @property
    def adjoint(self) -> bool:
        return self.mode == "ADJOINT"


def _strip(text: str):
    """inp_comments: (line number, text) of non-blank, non-comment lines."""
    out = []
    for ln, raw in enumerate(text.splitlines(), start=1):
        line = raw[:200].replace("\t", " ").strip()
        c = line.find("!")
        if c < 0:
            if line:
                out.append((ln, line))
        elif c > 0:
            out.append((ln, line[:c]))
    return out


def _read_text(path):
    with open(path) as f:
        return f.read()


def _split(lines, basedir):
    cards = {}
    cur = None
    for ln, text in lines:
        if "FILE" in text or "file" in text:
            parts = text.strip().split(None, 1)
            fname = parts[1].strip() if len(parts) > 1 else ""
            # as given, else beside the deck; an absolute path written on
            # another machine (the sample decks carry their author's) falls
            # back to the file of that name beside the deck
            path = fname if os.path.exists(fname) else os.path.join(basedir, fname)
            if not os.path.exists(path) and os.path.isabs(fname):
                path = os.path.join(basedir, os.path.basename(fname))
            if cur is None:
                raise DeckError(ADP_ERR_INPUT, f"line {ln}: FILE include outside a card")
            try:
                cur.extend(_strip(_read_text(path)))
            except OSError as e:
                raise DeckError(ADP_ERR_INPUT, f"line {ln}: cannot open card file {fname}: {e}")
            continue
        per = text.find("%")
        if per >= 0:
            name = text[per + 1:].strip()
            if name not in KNOWN_CARDS:
                raise DeckError(ADP_ERR_INPUT, f"at line {ln}: this is a wrong input card: {name}")
            cur = cards.setdefault(name, [])
            continue
        if cur is not None:
            cur.append((ln, text))
    return cards


_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eEdD][+-]?\d+)?$")


class _Card:
    """Fortran list-directed reads, one record (line) per READ."""

    def __init__(self, name, lines):
        self.name, self.lines, self.i = name, lines, 0

    def rec(self):
        if self.i >= len(self.lines):
            raise DeckError(ADP_ERR_INPUT, f"card %{self.name}: unexpected end of card")
        ln, text = self.lines[self.i]
        self.i += 1
        text = text.split("/")[0].replace(",", " ")
        toks = []
        for t in text.split():
            if "*" in t and t.index("*") > 0:
                r, v = t.split("*", 1)
                toks.extend([v] * int(r))
            else:
                toks.append(t)
        return _Rec(self.name, ln, toks)


class _Rec:
    def __init__(self, card, ln, toks):
        self.card, self.ln, self.toks, self.pos = card, ln, toks, 0

    def fail(self, what, status=ADP_ERR_INPUT):
        raise DeckError(status, f"card %{self.card} line {self.ln}: {what}")

    def next(self):
        if self.pos >= len(self.toks):
            self.fail("this line needs more input data")
        t = self.toks[self.pos]
        self.pos += 1
        return t

    def i(self):
        t = self.next()
        if not re.fullmatch(r"[+-]?\d+", t):
            self.fail(f"bad integer '{t}'")
        return int(t)

    def d(self):
        t = self.next()
        if not _NUM.match(t):
            self.fail(f"bad real '{t}'")
        return float(t.replace("d", "e").replace("D", "e"))

    def ints(self, n):
        return [self.i() for _ in range(n)]

    def reals(self, n):
        return [self.d() for _ in range(n)]


def parse(text: str, basedir: str = ".") -> Deck:
    cards = _split(_strip(text), basedir)
    for name in cards:
        if name in OUT_OF_SCOPE:
            raise DeckError(ADP_ERR_UNSUPPORTED, f"card %{name} is outside the static k-eigenvalue path")
    dk = Deck()
    if "MODE" not in cards or not cards["MODE"]:
        raise DeckError(ADP_ERR_INPUT, "card %MODE does not present. this card is mandatory")
    dk.mode = cards["MODE"][0][1].strip().upper()
    if dk.mode not in ("FORWARD", "ADJOINT", "BCSEARCH", "RODEJECT"):
        if dk.mode in ("FIXEDSRC",):
            raise DeckError(ADP_ERR_UNSUPPORTED, f"mode {dk.mode} is outside the static k-eigenvalue path")
        raise DeckError(ADP_ERR_INPUT, f"mode {dk.mode} is unidentified")
    if "KERN" in cards:
        r = _Card("KERN", cards["KERN"]).rec()
        k = r.next()[:4].upper()
        if k not in ("FDM", "PNM", "SANM"):
            r.fail("could not recognize nodal kernel: " + k)
        dk.kern = k
    if "XSEC" not in cards:
        raise DeckError(ADP_ERR_INPUT, "card %XSEC or %XTAB does not present. this card is mandatory")
    _xsec(dk, cards["XSEC"])
    if "GEOM" not in cards:
        raise DeckError(ADP_ERR_INPUT, "card %GEOM does not present. this card is mandatory")
    mnum, pasm, zpln = _geom(dk, cards["GEOM"])
    if "PRNT" in cards:
        r = _Card("PRNT", cards["PRNT"]).rec()
        dk.prnt = tuple(r.ints(3))
    _misc(dk, mnum)
    dk.coreh = 0.0
    for z in dk.zdel:
        dk.coreh = dk.coreh + float(z)
    dk.feedback = {}
    if "CROD" in cards:
        _crod(dk, cards["CROD"])
    if "CBCS" in cards:
        dk.feedback["bcon"] = _state_card(dk, "CBCS", cards["CBCS"], has_value=False)
        dk.bcbcs = True
    elif "BCON" in cards:
        dk.feedback["bcon"] = _state_card(dk, "BCON", cards["BCON"], has_value=True)
    for nm in ("FTEM", "MTEM", "CDEN"):
        if nm in cards:
            dk.feedback[nm.lower()] = _state_card(dk, nm, cards[nm], has_value=True)
    # card checks of mode BCSEARCH (mod_io.f90:196-214)
    if dk.mode == "BCSEARCH" and not dk.bcbcs:
        raise DeckError(ADP_ERR_INPUT, "mode BCSEARCH needs card %CBCS")
    if dk.mode != "BCSEARCH" and dk.bcbcs:
        raise DeckError(ADP_ERR_INPUT, "card %CBCS is not necessary for this calculation mode")
    if dk.mode == "BCSEARCH" and "BCON" in cards:
        raise DeckError(ADP_ERR_INPUT, "card %BCON must not present for this calculation mode")
    # card checks of mode RODEJECT (mod_io.f90:227-245)
    if dk.mode == "RODEJECT" and "EJCT" not in cards:
        raise DeckError(ADP_ERR_INPUT, "mode RODEJECT needs card %EJCT")
    if dk.mode == "RODEJECT" and "CROD" not in cards:
        raise DeckError(ADP_ERR_INPUT, "mode RODEJECT needs card %CROD")
    if dk.mode != "RODEJECT" and "EJCT" in cards:
        raise DeckError(ADP_ERR_INPUT, "card %EJCT is not necessary for this calculation mode")
    if "EJCT" in cards:
        _ejct(dk, cards["EJCT"])
    if "ITER" in cards:
        r = _Card("ITER", cards["ITER"]).rec()
        dk.nout, dk.nin = r.i(), r.i()
        dk.serc, dk.ferc = r.d(), r.d()
        dk.nac, dk.nupd = r.i(), r.i()
        r.i(), r.i()   # th_niter, nth: thermal-hydraulics only
        if dk.nout < dk.nupd and dk.kern != "FDM":
            r.fail("max. number of outer iteration should be bigger than nodal update interval")
    if "THET" in cards:
        r = _Card("THET", cards["THET"]).rec()
        th = r.d()
        if th < 0.001:
            r.fail("theta value is too small")
        if th > 1.0:
            r.fail("theta value shall not greater than 1.0")
        dk.trans["theta"] = th
    dk.trans["extr"] = "EXTR" in cards
    dk.dc = np.ones((dk.nnod, dk.ng, 6))
    if "ADF" in cards:
        _adf(dk, cards["ADF"], mnum, pasm, zpln)
    return dk


def _ejct(dk, lines):
    """%EJCT (mod_io.f90:2332-2482): per bank the final position, start time
    and speed; ttot, tstep1, tdiv, tstep2; beta and lambda of the six
    families; the group velocities (an optional print flag follows)."""
    c = _Card("EJCT", lines)
    cr = dk.feedback["crod"]
    nb = cr["nb"]
    fbpos, tmove, bspeed, mdir = np.zeros(nb), np.zeros(nb), np.zeros(nb), np.zeros(nb, dtype=np.int64)
    for i in range(nb):
        r = c.rec()
        fbpos[i], tmove[i], bspeed[i] = r.d(), r.d(), r.d()
        if fbpos[i] > float(cr["nstep"]):
            r.fail("wrong final control rod position")
        d = fbpos[i] - cr["bpos"][i]
        mdir[i] = 0 if abs(d) < 1.e-5 else (2 if d > 1.e-5 else 1)
    r = c.rec()
    ttot, tstep1, tdiv, tstep2 = r.d(), r.d(), r.d(), r.d()
    beta = np.array(c.rec().reals(6))
    lamb = np.array(c.rec().reals(6))
    velo = np.array(c.rec().reals(dk.ng))
    if ttot < tstep1 or ttot < tstep2:
        r.fail("total simulation time shall be greater than the time steps")
    if tdiv < tstep1:
        r.fail("when to start the second time step shall be greater than the first time step")
    if tdiv > ttot:
        r.fail("when to start the second time step shall be less than the total time")
    if _nint(tdiv / tstep1) + _nint((ttot - tdiv) / tstep2) > 10000:
        r.fail("too many time steps (more than 10000)")
    dk.trans.update(fbpos=fbpos, tmove=tmove, bspeed=bspeed, mdir=mdir, ttot=ttot, tstep1=tstep1, tdiv=tdiv,
                    tstep2=tstep2, beta=beta, lamb=lamb, velo=velo)


def _nint(x):
    """Fortran NINT: nearest integer, halves away from zero."""
    return int(np.floor(x + 0.5)) if x >= 0 else -int(np.floor(-x + 0.5))


def _changes(dk, c):
    """nmat x ng records: changes of sigtr, siga, nuf, sigf and sigs(g, 1..ng)."""
    ng, nm = dk.ng, dk.nmat
    ch = {k: np.zeros((nm, ng)) for k in ("sigtr", "siga", "nuf", "sigf")}
    ch["sigs"] = np.zeros((nm, ng, ng))
    for i in range(nm):
        for g in range(ng):
            v = c.rec().reals(4 + ng)
            ch["sigtr"][i, g], ch["siga"][i, g], ch["nuf"][i, g], ch["sigf"][i, g] = v[:4]
            ch["sigs"][i, g, :] = v[4:]
    return ch


def _state_card(dk, name, lines, has_value):
    """%CBCS (reference only), %BCON, %FTEM, %MTEM, %CDEN (value and reference),
    then the per-material changes (mod_io.f90:2486-2954)."""
    c = _Card(name, lines)
    r = c.rec()
    if has_value:
        val, ref = r.d(), r.d()
    else:
        ref = r.d()
        val = ref
    return dict(value=val, ref=ref, changes=_changes(dk, c))


def _crod(dk, lines):
    """%CROD (mod_io.f90:2148-2328): banks, steps, zero position and step size,
    bank positions, the assembly bank map (north row first) and the changes of
    a fully rodded node."""
    c = _Card("CROD", lines)
    r = c.rec()
    nb, nstep = r.i(), r.i()
    r = c.rec()
    pos0, ssize = r.d(), r.d()
    r = c.rec()
    bpos = r.reals(nb)
    for b in bpos:
        if b > float(np.float32(nstep)):
            r.fail("control rod bank position is larger than the number of steps")
        if b < 0.0:
            r.fail("control rod bank position is negative")
        if dk.coreh < b * ssize:
            r.fail("core height is lower than the control rod position")
    bmap = np.zeros((dk.nx, dk.ny), dtype=np.int64)
    for j in range(dk.ny - 1, -1, -1):
        rr = c.rec()
        bmap[:, j] = rr.ints(dk.nx)
        if (bmap[:, j] > nb).any():
            rr.fail("control rod bank number is larger than the number of banks")
    xdiv, ydiv = dk.extra["xdiv"], dk.extra["ydiv"]
    fbmap = np.repeat(np.repeat(bmap, xdiv, axis=0), ydiv, axis=1)   # (nxx, nyy)
    dk.feedback["crod"] = dict(nb=nb, nstep=nstep, pos0=pos0, ssize=ssize, bpos=np.array(bpos), fbmap=fbmap,
                               changes=_changes(dk, c))


def load(path: str) -> Deck:
    return parse(_read_text(path), os.path.dirname(os.path.abspath(path)))


def _xsec(dk, lines):
    c = _Card("XSEC", lines)
    r = c.rec()
    dk.ng, dk.nmat = r.i(), r.i()
    if dk.ng < 1 or dk.nmat < 1:
        r.fail("bad group or material count")
    for _, text in lines:
        if "/" in text or "\\" in text:
            raise DeckError(ADP_ERR_INPUT, "slash or backslash not accepted in %XSEC card")
    ng, nm = dk.ng, dk.nmat
    dk.xsigtr, dk.xsiga, dk.xnuf, dk.xsigf, dk.chi = (np.zeros((nm, ng)) for _ in range(5))
    dk.xsigs = np.zeros((nm, ng, ng))
    for i in range(nm):
        for g in range(ng):
            r = c.rec()
            v = r.reals(5 + ng)
            dk.xsigtr[i, g], dk.xsiga[i, g], dk.xnuf[i, g], dk.xsigf[i, g], dk.chi[i, g] = v[:5]
            dk.xsigs[i, g, :] = v[5:]
            if dk.xsigtr[i, g] <= 0.0:
                raise DeckError(ADP_ERR_BADXS, f"transport cross section is zero or negative in material {i + 1} group {g + 1}")
    if not (dk.xnuf > 0).any():
        raise DeckError(ADP_ERR_BADXS, "the problem has no fission material (nu*fission all zero)")
    if not (dk.xsigf > 0).any():
        raise DeckError(ADP_ERR_BADXS, "the problem has no fission material (fission xsec all zero)")


def _geom(dk, lines):
    c = _Card("GEOM", lines)
    r = c.rec()
    dk.nx, dk.ny, dk.nz = r.ints(3)
    for v, nm, lo, hi in ((dk.nx, "nx", 2, 33), (dk.ny, "ny", 2, 33), (dk.nz, "nz", 2, 40)):
        if v < lo:
            r.fail(f"{nm} shall be at least {lo}")
        if v > hi:
            r.fail(f"{nm} shall be maximum {hi}")
    xsize = c.rec().reals(dk.nx)
    xdiv = c.rec().ints(dk.nx)
    ysize = c.rec().reals(dk.ny)
    ydiv = c.rec().ints(dk.ny)
    zsize = c.rec().reals(dk.nz)
    zdiv = c.rec().ints(dk.nz)
    if min(xdiv + ydiv + zdiv) < 1:
        r.fail("division must be >= 1")
    dk.nxx, dk.nyy, dk.nzz = sum(xdiv), sum(ydiv), sum(zdiv)
    for v, nm in ((dk.nxx, "nxx"), (dk.nyy, "nyy"), (dk.nzz, "nzz")):
        if v > 800:
            r.fail(f"{nm} shall be maximum 800")

    def deltas(size, div):
        # div = size/REAL(div): the divisor is a default real (exact for small integers)
        return np.concatenate([np.full(d, s / float(np.float32(d))) for s, d in zip(size, div)])

    dk.xdel, dk.ydel, dk.zdel = deltas(xsize, xdiv), deltas(ysize, ydiv), deltas(zsize, zdiv)
    np_ = c.rec().i()
    zpln = c.rec().ints(dk.nz)
    for z in zpln:
        if z > np_:
            r.fail("planar is greater than number of planar")
        if z < 1:
            r.fail("planar should be at least 1")
    pasm = np.zeros((np_, dk.nx, dk.ny), dtype=np.int64)
    for k in range(np_):
        for j in range(dk.ny - 1, -1, -1):          # north row first
            pasm[k, :, j] = c.rec().ints(dk.nx)
    if (pasm > dk.nmat).any():
        raise DeckError(ADP_ERR_INPUT, "material is greater than number of material")
    if (pasm < 0).any():
        raise DeckError(ADP_ERR_INPUT, "negative material found")
    xa = np.repeat(np.arange(dk.nx), xdiv)
    ya = np.repeat(np.arange(dk.ny), ydiv)
    za = np.repeat(np.arange(dk.nz), zdiv)
    planar = np.array(zpln)[za] - 1
    mnum = pasm[planar[None, None, :], xa[:, None, None], ya[None, :, None]]   # (nxx, nyy, nzz)
    act = mnum[:, :, 0] != 0
    ysmin = np.full(dk.nyy, dk.nxx, dtype=np.int64)
    ysmax = np.zeros(dk.nyy, dtype=np.int64)
    for j in range(dk.nyy):
        nz_ = np.nonzero(act[:, j])[0]
        if nz_.size:
            ysmin[j], ysmax[j] = nz_[0] + 1, nz_[-1] + 1
    xsmin = np.full(dk.nxx, dk.nyy, dtype=np.int64)
    xsmax = np.zeros(dk.nxx, dtype=np.int64)
    for i in range(dk.nxx):
        nz_ = np.nonzero(act[i, :])[0]
        if nz_.size:
            xsmin[i], xsmax[i] = nz_[0] + 1, nz_[-1] + 1
    for j in range(dk.nyy):
        if (mnum[ysmin[j] - 1:ysmax[j], j, :] == 0).any():
            raise DeckError(ADP_ERR_INPUT, "zero material found inside core")
    for i in range(dk.nxx):
        if (mnum[i, xsmin[i] - 1:xsmax[i], :] == 0).any():
            raise DeckError(ADP_ERR_INPUT, "zero material found inside core")
    if ((ysmax - ysmin) < 1).any():
        raise DeckError(ADP_ERR_INPUT, "x row with fewer than two nodes")
    if ((xsmax - xsmin) < 1).any():
        raise DeckError(ADP_ERR_INPUT, "y column with fewer than two nodes")
    r = c.rec()
    dk.bc = tuple(r.ints(6))
    if any(b > 2 or b < 0 for b in dk.bc):
        r.fail("wrong boundary conditions")
    dk.extra.update(ysmin=ysmin, ysmax=ysmax, xsmin=xsmin, xsmax=xsmax, xdiv=xdiv, ydiv=ydiv, zdiv=zdiv)
    return mnum, pasm, zpln


def _misc(dk, mnum):
    ysmin, ysmax = dk.extra["ysmin"], dk.extra["ysmax"]
    ix, iy, iz, mat = [], [], [], []
    for k in range(1, dk.nzz + 1):
        for j in range(1, dk.nyy + 1):
            i = np.arange(ysmin[j - 1], ysmax[j - 1] + 1)
            ix.append(i)
            iy.append(np.full(i.size, j))
            iz.append(np.full(i.size, k))
            mat.append(mnum[i - 1, j - 1, k - 1])
    dk.ix = np.concatenate(ix).astype(np.int32)
    dk.iy = np.concatenate(iy).astype(np.int32)
    dk.iz = np.concatenate(iz).astype(np.int32)
    dk.mat = np.concatenate(mat).astype(np.int32)
    dk.nnod = int(dk.ix.size)
    dk.nupd = int(np.ceil(np.float32(dk.nxx + dk.nyy + dk.nzz) / np.float32(2.5)))


def _rotate(rot, a):
    x1, x2, x3, x4 = a[..., 0].copy(), a[..., 1].copy(), a[..., 2].copy(), a[..., 3].copy()
    if rot == 1:
        a[..., 0], a[..., 1], a[..., 2], a[..., 3] = x4, x3, x1, x2
    elif rot == 2:
        a[..., 0], a[..., 1], a[..., 2], a[..., 3] = x2, x1, x4, x3
    elif rot == 3:
        a[..., 0], a[..., 1], a[..., 2], a[..., 3] = x3, x4, x2, x1


def _adf(dk, lines, mnum, pasm, zpln):
    c = _Card("ADF", lines)
    ng, nm = dk.ng, dk.nmat
    mdc = np.zeros((nm, ng, 6))
    for i in range(nm):
        for g in range(ng):
            mdc[i, g] = c.rec().reals(6)
    xdc = np.zeros((dk.nx, dk.ny, dk.nz, ng, 6))
    for k in range(dk.nz):
        asm = pasm[zpln[k] - 1]
        for j in range(dk.ny):
            for i in range(dk.nx):
                if asm[i, j] != 0:
                    xdc[i, j, k] = mdc[asm[i, j] - 1]
    while True:
        rot = c.rec().i()
        if rot < 1:
            break
        while True:
            r = c.rec()
            x1, x2, y1, y2, z1, z2 = r.ints(6)
            if min(x1, x2, y1, y2, z1, z2) < 1:
                break
            if x1 > dk.nx or x2 > dk.nx or y1 > dk.ny or y2 > dk.ny or z1 > dk.nz or z2 > dk.nz:
                r.fail("wrong position for ADF rotation: out of dimension of the core")
            if x2 < x1 or y2 < y1 or z2 < z1:
                continue
            _rotate(rot, xdc[x1 - 1:x2, y1 - 1:y2, z1 - 1:z2])
    # Node faces on assembly boundaries take the assembly ADF; the z values
    # are placed as mod_io.f90:2077-2078 places them (DC5 on the first node
    # of the assembly, DC6 on the last).
    xdiv, ydiv, zdiv = dk.extra["xdiv"], dk.extra["ydiv"], dk.extra["zdiv"]
    tx = np.concatenate([[1], 1 + np.cumsum(xdiv)])
    ty = np.concatenate([[1], 1 + np.cumsum(ydiv)])
    tz = np.concatenate([[1], 1 + np.cumsum(zdiv)])
    xa = np.repeat(np.arange(dk.nx), xdiv)
    ya = np.repeat(np.arange(dk.ny), ydiv)
    za = np.repeat(np.arange(dk.nz), zdiv)
    dc = np.ones((dk.nnod, ng, 6))
    for n in range(dk.nnod):
        xt, yt, zt = dk.ix[n], dk.iy[n], dk.iz[n]
        i, j, k = xa[xt - 1], ya[yt - 1], za[zt - 1]
        v = np.ones((ng, 6))
        a = xdc[i, j, k]
        if xt == tx[i]:
            v[:, 1] = a[:, 1]
        if xt == tx[i + 1] - 1:
            v[:, 0] = a[:, 0]
        if yt == ty[j]:
            v[:, 3] = a[:, 3]
        if yt == ty[j + 1] - 1:
            v[:, 2] = a[:, 2]
        if zt == tz[k]:
            v[:, 4] = a[:, 4]
        if zt == tz[k + 1] - 1:
            v[:, 5] = a[:, 5]
        dc[n] = v
    dk.dc = dc
