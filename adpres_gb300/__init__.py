"""GB300 (sm_103a) implementation of the ADPRES static k-eigenvalue path.

CMFD power iteration with BiCGSTAB inner solves and the SANM/PNM two-node
nodal update, behind the C ABI in include/adpres_gb300.h.  This package is
the host side: the ctypes binding (``_lib``), the deck reader (``deck``),
synthetic core generators (``synth``) and the ``Core`` driver (``core``).
"""
from . import deck  # noqa: F401
from ._lib import AdpError  # noqa: F401

__all__ = ["deck", "AdpError", "Core", "solve_deck"]


def __getattr__(name):
    if name in ("Core", "solve_deck"):
        from . import core
        return getattr(core, name)
    raise AttributeError(name)
