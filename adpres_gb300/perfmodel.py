"""Algorithmic memory traffic of the persistent CMFD kernel.

Bytes are counted per box row (one node of the padded box, one group) as
the words the kernel must move if every neighbour read hits in cache:

  P0  group source + initial residual (TSrc + r = b - A x):
      FP64 matrix (7 words), x, fs0, the source weight, (G-1) x (sigma_s,
      flux of the other group) read; r, rs written.
  per BiCGSTAB iteration (bicg, mod_cmfd.f90:1228-1241):
      A: r, p, v, rs + 7 coefficients read; p, v written     (13 words)
      B: r, v + 7 coefficients read; s, t written            (11 words)
      C: x, p, s, t, rs read; x, r written                   ( 7 words)
  per outer: FSrc + norms read G fluxes, G weights, fs0c, vdel and write
      fs0 (2G + 3 words); extrapolation every nac outers reads fs0, fs0c,
      vdel and writes fs0 (4 words / nac).

FP64 storage: every word is 8 bytes.  Mixed storage: the matrix copy used
by the Krylov steps and the Krylov vectors are 4 bytes; the flux x, the
sources and the FP64 matrix read by P0 stay 8 bytes.
"""
from __future__ import annotations


def bytes_per_row_outer(ng: int, nin: int, nac: int, precision: str) -> float:
    G = ng
    if precision == "fp64":
        p0 = 8 * (7 + 1 + 1 + 1 + 2 * (G - 1)) + 8 * 2
        it = 8 * 31
    else:
        p0 = 8 * (7 + 1 + 1 + 1 + 2 * (G - 1)) + 4 * 2
        a = 4 * (4 + 7) + 4 * 2
        b = 4 * (2 + 7) + 4 * 2
        c = (8 + 4 * 4) + (8 + 4)
        it = a + b + c
    fis = 8 * (2 * G + 3) + 8 * 4 / nac
    return G * (p0 + nin * it) + fis


def bicg_bytes_per_row_iteration(precision: str) -> float:
    """The canonical per-row BiCGSTAB traffic (31 words)."""
    if precision == "fp64":
        return 248.0
    return 4 * (4 + 7) + 4 * 2 + 4 * (2 + 7) + 4 * 2 + (8 + 4 * 4) + (8 + 4)


def p0_skipped_bytes_per_row_outer(xsigs, chi, mat) -> float:
    """Bytes of the P0 terms the kernel leaves out on a given core (forward
    solve): per outer and box row, 16 B (sigma_s and the other group's flux)
    for every scattering plane h -> g that is zero in every material in use,
    and 16 B (the source weight and fs0) for every group whose chi is zero
    in every material in use.  The canonical count above includes them."""
    import numpy as np
    used = np.unique(np.asarray(mat)) - 1
    xs = np.asarray(xsigs)[used]
    ch = np.asarray(chi)[used]
    G = ch.shape[1]
    zs = sum(1 for h in range(G) for g in range(G) if h != g and not np.any(xs[:, h, g] != 0.0))
    zc = sum(1 for g in range(G) if not np.any(ch[:, g] != 0.0))
    return 16.0 * (zs + zc)


def canonical_bytes_per_node_outer(ng: int, nin: int, w: int) -> float:
    """Canonical algorithmic bytes of one outer per node: w-byte words, 31
    per BiCGSTAB step (fused in three phases), 2G + 11 for each group's
    source and initial residual, 3G + 3 for the fission source and the norms:
    w [G (31 nin + 2G + 11) + 3G + 3].  w = 8 for FP64 storage, 4 for the
    FP32-storage form of the mixed path."""
    G = ng
    return float(w * (G * (31 * nin + 2 * G + 11) + 3 * G + 3))
