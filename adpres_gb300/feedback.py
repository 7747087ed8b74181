"""Cross-section feedback and the critical boron search, on the host.

``xs_update`` is XS_updt (mod_xsec.f90:11-46) with the deck's feedback
cards: node tables from the material tables (base_updt), then per node
x += change(mat) * dv for boron (bcon - rbcon), fuel temperature
(sqrt(T) - sqrt(Tref)), moderator temperature and coolant density
(bcon_updt, ftem_updt, mtem_updt, cden_updt, :394-521), then the control
rods (crod_updt, :230-303) at the given bank positions: fully rodded nodes get the rod changes, the
node holding the tip a volume fraction of them, and negative siga, nuf,
sigf and sigs of rodded columns become 0.  The result goes to the device
through adp_xs_updt_nodes, which forms D and sigr and checks them.

``Core.fb_set``/``Core.fb_updt`` run the same update on the device from
resident tables (adp_fb_set, adp_fb_updt) with the same operations in the
same order, so both give the same node tables to the bit; the searches and
the transient use the device form and hand over only the state values and
the bank positions.

``cbsearch`` is th::cbsearch (mod_th.f90:752-837): a secant search of the
boron concentration that makes k = 1, each step an XS update and a
warm-started outer(0) on the GPU.
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import (AdpError, ADP_ERR_INPUT, ADP_ERR_MAXOUTER, ADP_FB_BORON, ADP_FB_COOL_DENS,
                   ADP_FB_FUEL_TEMP, ADP_FB_MOD_TEMP)

KEYS = ("sigtr", "siga", "nuf", "sigf", "sigs")
# the state cards in the order XS_updt applies them (mod_xsec.f90:24-40)
STATE_CARDS = (("bcon", ADP_FB_BORON), ("ftem", ADP_FB_FUEL_TEMP), ("mtem", ADP_FB_MOD_TEMP),
               ("cden", ADP_FB_COOL_DENS))


def _rod_tip(rodh, zdel):
    """The plane holding the rod tip, walking down from the top, and the
    rodded fraction of it; (-1, None) when every plane is fully rodded."""
    dum = 0.0
    for k in range(len(zdel) - 1, -1, -1):
        if rodh >= dum and rodh <= dum + zdel[k]:
            return k, (rodh - dum) / zdel[k]
        dum = dum + zdel[k]
    return -1, None


def xs_update(dk, bcon=None, bpos=None):
    """Node tables sigtr, siga, nuf, sigf (nnod, ng) and sigs (nnod, ng, ng).

    Up to the control rods a node's values are those of its material, so the
    state updates run on the material tables (the same operands and order
    as the reference's per-node loops) and are gathered to the nodes once."""
    tab = dict(sigtr=dk.xsigtr, siga=dk.xsiga, nuf=dk.xnuf, sigf=dk.xsigf, sigs=dk.xsigs)
    fb = getattr(dk, "feedback", {}) or {}

    def state(ch, dv):
        for k in KEYS:
            tab[k] = tab[k] + ch[k] * dv

    if "bcon" in fb:
        b = fb["bcon"]["value"] if bcon is None else bcon
        state(fb["bcon"]["changes"], b - fb["bcon"]["ref"])
    if "ftem" in fb:
        f = fb["ftem"]
        state(f["changes"], math.sqrt(f["value"]) - math.sqrt(f["ref"]))
    for nm in ("mtem", "cden"):
        if nm in fb:
            state(fb[nm]["changes"], fb[nm]["value"] - fb[nm]["ref"])
    m = dk.mat - 1
    t = {k: tab[k][m] for k in KEYS}
    if "crod" in fb:
        _crod_update(dk, fb["crod"], t, bpos)
    return t


def _crod_update(dk, cr, t, bpos=None):
    """Each node is in one column, so the reference's column loop is a per-bank
    selection: planes above the tip get x + c, the tip's plane x + w*c.
    bpos: bank positions (steps) when they differ from the card's."""
    ch = cr["changes"]
    bpos = cr["bpos"] if bpos is None else bpos
    m = dk.mat - 1
    z = np.asarray(dk.iz) - 1
    bank = np.asarray(cr["fbmap"])[np.asarray(dk.ix) - 1, np.asarray(dk.iy) - 1]
    zdel = [float(v) for v in dk.zdel]
    for b in range(1, int(cr["nb"]) + 1):
        sel = bank == b
        if not sel.any():
            continue
        kt, vf = _rod_tip(dk.coreh - cr["pos0"] - bpos[b - 1] * cr["ssize"], zdel)
        full = np.nonzero(sel & (z > kt))[0]
        part = np.nonzero(sel & (z == kt))[0]
        for k in KEYS:
            a = t[k]
            a[full] = a[full] + ch[k][m[full]]
            if len(part):
                a[part] = a[part] + vf * ch[k][m[part]]
    rodded = np.nonzero(bank > 0)[0]
    for k in ("siga", "nuf", "sigf", "sigs"):
        r = t[k][rodded]
        r[r < 0.0] = 0.0
        t[k][rodded] = r


def cbsearch(core, dk=None, max_steps=20):
    """Critical boron search on the GPU: list of (bcon, k, outers); the last is critical.

    Sets core.cbsearch_device_ms to the summed device time of the outer calls."""
    dk = dk if dk is not None else core.deck
    if "bcon" not in dk.feedback:
        raise AdpError(ADP_ERR_INPUT, "critical boron search needs the boron feedback card (%CBCS)")
    fb = dk.feedback["bcon"]
    steps = []
    core.cbsearch_device_ms = 0.0
    core.fb_set(dk)

    def solve(b):
        core.fb_updt(dk, bcon=b)
        rep = core.outer(popt=0, trace=False)
        core.cbsearch_device_ms += rep.device_ms
        steps.append((b, rep.keff, rep.outers))
        return rep

    bcon = fb["ref"]
    rep = solve(bcon)
    bc1, ke1 = bcon, rep.keff
    bcon = bcon + (rep.keff - 1.0) * bcon
    rep = solve(bcon)
    bc2, ke2 = bcon, rep.keff
    n = 3
    while True:
        bcon = bc2 + (1.0 - ke2) / (ke1 - ke2) * (bc1 - bc2)
        rep = solve(bcon)
        bc1, bc2, ke1, ke2 = bc2, bcon, ke2, rep.keff
        if abs(rep.keff - 1.0) < 1.0e-5 and rep.ser < 1.0e-5 and rep.fer < 1.0e-5:
            return steps
        n += 1
        if bcon > 3000.0:
            raise AdpError(ADP_ERR_INPUT, "critical boron concentration exceeds the limit (3000 ppm)")
        if bcon < 0.0:
            raise AdpError(ADP_ERR_INPUT, "critical boron concentration is not found (less than zero)")
        if n == max_steps:
            raise AdpError(ADP_ERR_MAXOUTER, "maximum iteration for critical boron search is reaching maximum")
