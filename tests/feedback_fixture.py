"""A Deck rebuilt from the critical boron search fixture
(tests/golden/decks/CBCsearch.npz, written by tests/golden/make_feedback.py),
so that tests run without the reference's sample decks."""
import os

import numpy as np

from adpres_gb300 import deck
from conftest import GOLDEN

KERNS = {0: "FDM", 1: "PNM", 2: "SANM"}


def fixture(name="CBCsearch"):
    return np.load(os.path.join(GOLDEN, "decks", name + ".npz"))


def unpack_changes(a):
    a = np.asarray(a)
    ch = {k: np.ascontiguousarray(a[:, :, i]) for i, k in enumerate(("sigtr", "siga", "nuf", "sigf"))}
    ch["sigs"] = np.ascontiguousarray(a[:, :, 4:])
    return ch


def deck_from_fixture(fx, mode="BCSEARCH"):
    ng, nm, nn = int(fx["ng"]), int(fx["nmat"]), int(fx["nnod"])
    F = lambda a, shape: np.asarray(a).reshape(shape, order="F")
    nin, nout, nac, nupd = (int(v) for v in fx["iter_int"])
    serc, ferc = (float(v) for v in fx["iter_real"])
    dk = deck.Deck(mode=mode, kern=KERNS[int(fx["kern"])], ng=ng, nmat=nm,
                   xsigtr=F(fx["xsigtr"], (nm, ng)), xsiga=F(fx["xsiga"], (nm, ng)), xnuf=F(fx["xnuf"], (nm, ng)),
                   xsigf=F(fx["xsigf"], (nm, ng)), chi=F(fx["chi"], (nm, ng)), xsigs=F(fx["xsigs"], (nm, ng, ng)),
                   nxx=int(fx["nxx"]), nyy=int(fx["nyy"]), nzz=int(fx["nzz"]), xdel=np.asarray(fx["xdel"]),
                   ydel=np.asarray(fx["ydel"]), zdel=np.asarray(fx["zdel"]), bc=tuple(int(b) for b in fx["bc"]),
                   nnod=nn, ix=np.asarray(fx["ix"]), iy=np.asarray(fx["iy"]), iz=np.asarray(fx["iz"]),
                   mat=np.asarray(fx["mat"]), dc=F(fx["dc"], (nn, ng, 6)), nin=nin, nout=nout, serc=serc, ferc=ferc,
                   nac=nac, nupd=nupd, coreh=float(fx["coreh"]), bcbcs=True)
    if "tr_scal" in fx:
        ttot, tstep1, tdiv, tstep2, theta, extr = (float(v) for v in fx["tr_scal"])
        dk.bcbcs = False
        dk.trans = dict(fbpos=np.asarray(fx["tr_fbpos"]), tmove=np.asarray(fx["tr_tmove"]),
                        bspeed=np.asarray(fx["tr_bspeed"]), mdir=np.asarray(fx["tr_mdir"]), ttot=ttot, tstep1=tstep1,
                        tdiv=tdiv, tstep2=tstep2, beta=np.asarray(fx["tr_beta"]), lamb=np.asarray(fx["tr_lamb"]),
                        velo=np.asarray(fx["tr_velo"]), theta=theta, extr=bool(extr))
    for nm_ in (str(s) for s in fx["fb_names"]):
        ch = unpack_changes(fx["fb_%s_ch" % nm_])
        if nm_ == "crod":
            nb, nstep, pos0, ssize = (float(v) for v in fx["fb_crod_scal"])
            dk.feedback["crod"] = dict(nb=int(nb), nstep=int(nstep), pos0=pos0, ssize=ssize,
                                       bpos=np.asarray(fx["fb_crod_bpos"]), fbmap=np.asarray(fx["fb_crod_fbmap"]),
                                       changes=ch)
        else:
            val, ref = (float(v) for v in fx["fb_%s_scal" % nm_])
            dk.feedback[nm_] = dict(value=val, ref=ref, changes=ch)
    return dk
