"""The rod ejection transient, rod_eject (mod_trans.f90:17-160) without
thermal-hydraulics, driven from the host over the C ABI.

The steady state: XS_updt at the %CROD bank positions, a forward outer(0),
KNE1 when k is not one (nu*sigf and its rod change divided by k until
|k - 1| < 1e-5), outer_ad(0) for the adjoint weight, and outer(0) again.
adp_trans_init then forms the precursors, the initial power and the
reactivity.  Each step of the two phases (tstep1 up to tdiv, tstep2 up to
ttot) moves the banks as trans_calc does (mod_trans.f90:366-381), recomputes
the node cross sections at the new positions on the device (adp_fb_updt
from the tables of adp_fb_set) and runs adp_trans_step: removal of the
step, external source, outer_tr on the GPU, precursors, power and
reactivity.
"""
from __future__ import annotations

import copy
import time

import numpy as np

from ._lib import AdpError, ADP_ERR_INPUT
from .deck import _nint


def _working_deck(dk):
    """A copy whose nu*sigf and rod nu*sigf change KNE1 may rescale."""
    w = copy.copy(dk)
    w.xnuf = dk.xnuf.copy()
    w.feedback = dict(dk.feedback)
    cr = dict(dk.feedback["crod"])
    cr["changes"] = dict(cr["changes"])
    cr["changes"]["nuf"] = cr["changes"]["nuf"].copy()
    w.feedback["crod"] = cr
    return w


def move_banks(bpos, tr, ht, t2):
    """The bank motion of trans_calc (mod_trans.f90:366-381)."""
    for n in range(len(bpos)):
        if tr["mdir"][n] == 1:
            if t2 - tr["tmove"][n] > 1.e-5 and tr["fbpos"][n] - bpos[n] < 1.e-5:
                bpos[n] = bpos[n] - ht * tr["bspeed"][n]
                if bpos[n] < tr["fbpos"][n]:
                    bpos[n] = tr["fbpos"][n]
        elif tr["mdir"][n] == 2:
            if t2 - tr["tmove"][n] > 1.e-5 and tr["fbpos"][n] - bpos[n] > 1.e-5:
                bpos[n] = bpos[n] + ht * tr["bspeed"][n]
                if bpos[n] > tr["fbpos"][n]:
                    bpos[n] = tr["fbpos"][n]


def rod_eject(core, dk=None, max_steps=None):
    """Records (t, rho, relative power, nout reached, outers, device ms); rho
    is absolute at t = 0 and in dollars afterwards, as the reference prints.
    Sets core.rod_eject_wall = (steady state s, time steps s), host clock."""
    t_start = time.perf_counter()
    dk = dk if dk is not None else core.deck
    tr = dk.trans
    w = _working_deck(dk)
    bpos = np.array(dk.feedback["crod"]["bpos"], dtype=np.float64)

    def set_xs():
        core.fb_updt(w, bpos=bpos)

    core.fb_set(w)
    set_xs()
    rep = core.outer(popt=0, trace=False)
    if abs(rep.keff - 1.0) > 1.e-5:
        # KNE1 (mod_trans.f90:483-518)
        stopped = None
        for i in range(1, 11):
            k = rep.keff
            w.xnuf = w.xnuf / k
            w.feedback["crod"]["changes"]["nuf"] = w.feedback["crod"]["changes"]["nuf"] / k
            core.fb_set(w)
            set_xs()
            rep = core.outer(popt=0, trace=False)
            if abs(rep.keff - 1.0) < 1.e-5:
                stopped = i
                break
        if stopped == 10:
            raise AdpError(ADP_ERR_INPUT, "k-eff still not equal to one")
    core.outer(adjoint=True, popt=0, trace=False)
    af = core.flux()
    core.outer(popt=0, trace=False)
    r0 = core.trans_init(tr["beta"], tr["lamb"], tr["velo"], tr["theta"], tr["extr"], af)
    out = [(0.0, r0.rho, 1.0, False, 0, 0.0)]
    t_steady = time.perf_counter()
    core.rod_eject_wall = (t_steady - t_start, 0.0)

    def step(ht, t2, omeg_mode):
        move_banks(bpos, tr, ht, t2)
        set_xs()
        r = core.trans_step(ht, omeg_mode)
        out.append((t2, r.rho_dollar, r.relpow, bool(r.maxi), r.outers, r.device_ms))
        core.rod_eject_wall = (t_steady - t_start, time.perf_counter() - t_steady)

    n = 0
    for i in range(1, _nint(tr["tdiv"] / tr["tstep1"]) + 1):
        if max_steps is not None and n >= max_steps:
            return out
        step(tr["tstep1"], float(np.float32(i)) * tr["tstep1"], 1 if i > 1 else 0)
        n += 1
    for i in range(1, _nint((tr["ttot"] - tr["tdiv"]) / tr["tstep2"]) + 1):
        if max_steps is not None and n >= max_steps:
            return out
        step(tr["tstep2"], tr["tdiv"] + float(np.float32(i)) * tr["tstep2"], 1)
        n += 1
    return out
