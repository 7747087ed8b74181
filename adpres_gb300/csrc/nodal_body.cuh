// Two-node nonlinear nodal update (SANM and PNM), mod_nodal.f90: the
// per-item device functions shared by the single-core kernels (nodal.cu)
// and the batched kernel (batch.cu).  Each *_items function processes
// items start, start + stride, ... of its stage.
//
// The reference sweeps x, y and z lines sequentially (mod_nodal.f90:53-125),
// but every new coupling coefficient dn depends only on per-node quantities
// of the two nodes of its interface, all computed from the transverse
// leakages S1..S3 that get_source builds once from the old dn before the
// sweeps (:49, :1009-1043).  The update is therefore split into
//   k_tl_source : get_source / Lxyz               (per node)
//   k_node_prep : get_B, get_a2matvec, LU_solve, get_a4, TLUpd1/TLUpd2
//                 -> a2, a4 and the first moment L1 (per node and direction)
//   k_interface : get_a1matvec[_first|_last], LU_solve, get_a3,
//                 nodal_coup_upd -> new dn, and the ndmax candidates
//                 (per node and direction: its minus face, plus the line's
//                 last face)
//   k_nodal_finish : ndmax with the sweep's first-maximum tie rule, the
//                 divergence check and the convergence test of the outer.
// The SANM constants (get_ABEFGH, :1409-1451) depend only on the cross
// sections and node sizes and are computed once per cross-section set.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"

namespace adp {

// PNM constants (mod_nodal.f90:180-181)
__device__ __forceinline__ void pnm_consts(double* c) {
  c[0] = 1.0 / 15.0;
  c[1] = 1.0 / 35.0;
  c[2] = 2.0 / 7.0;
  c[3] = 2.0 / 5.0;
  c[4] = 10.0;
  c[5] = 6.0;
}

// get_ABEFGH (mod_nodal.f90:1409-1451), stored as sanm[u][k][g][b], k = A,B,E,F,G,H
__device__ __forceinline__ void sanm_consts_items(const NodalParams& P, int start, int stride) {
  const int NB = P.G.NB, ng = P.ng;
  const int total = P.nnod * 3 * ng;
  for (int q = start; q < total; q += stride) {
    const int n = q % P.nnod, ug = q / P.nnod, u = ug % 3, g = ug / 3;
    const int b = P.act[n];
    const double dn = hdir(P.G, u, b);
    const double alp = 0.5 * sqrt(P.sigr[(size_t)g * NB + b] / P.D[(size_t)g * NB + b]) * dn;
    const double alp2 = alp * alp;
    const double sh = sinh(alp), ch = cosh(alp);
    const double m0c = sh / alp;
    const double m1s = 3.0 * (ch / alp - sh / alp2);
    const double m2c = 5.0 * (sh / alp - 3.0 * ch / alp2 + 3.0 * sh / (alp * alp * alp));
    double* out = (double*)P.sanm + ((size_t)u * 6 * ng + g) * NB + b;
    const size_t st = (size_t)ng * NB;
    out[0 * st] = (sh - m1s) / (alp2 * m1s);
    out[1 * st] = (ch - m0c - m2c) / (alp2 * m2c);
    out[2 * st] = (m0c / m2c - 3.0 / alp2);
    out[3 * st] = (alp * ch - m1s) / (alp2 * m1s);
    out[4 * st] = (alp * sh - 3.0 * m2c) / (ch - m0c - m2c);
    out[5 * st] = (alp * ch - m1s) / (sh - m1s);
  }
}

__device__ __forceinline__ const double* latest_phi(const NodalParams& P) {
  return P.phi[*(const volatile int*)&P.ctl->cur];
}

// ---------------------------------------------------------------------------
// get_source / Lxyz (mod_nodal.f90:901-1043)
// ---------------------------------------------------------------------------
// Net leakage of node b per direction (Lxyz): currents from df, dn and the
// flux F of one group; df, dn are that group's [6][NB] planes.
__device__ __forceinline__ void net_leakage(const BoxGeom& G, const double* F, const double* df, const double* dn,
                                            int b, double (&L)[3]) {
  const int NB = G.NB;
  const unsigned m = G.nbm[b];
  const double fn = F[b];
  for (int u = 0; u < 3; ++u) {
    const int fp = 2 * u, fm = 2 * u + 1;
    const double dfp = df[(size_t)fp * NB + b], dnp = dn[(size_t)fp * NB + b];
    const double dfm = df[(size_t)fm * NB + b], dnm = dn[(size_t)fm * NB + b];
    double jp, jm;
    if (!(m & (1u << fp))) {
      jp = (G.bcf[fp] == 2) ? 0.0 : dfp * fn - dnp * fn;
    } else {
      const double fpv = F[b + face_off(G, fp)];
      jp = -dfp * (fpv - fn) - dnp * (fpv + fn);
    }
    if (!(m & (1u << fm))) {
      jm = (G.bcf[fm] == 2) ? 0.0 : -dfm * fn - dnm * fn;
    } else {
      const double fmv = F[b + face_off(G, fm)];
      jm = -dfm * (fn - fmv) - dnm * (fn + fmv);
    }
    L[u] = (jp - jm) / hdir(G, u, b);
  }
}

__device__ __forceinline__ void tl_source_items(const NodalParams& P, int start, int stride) {
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  const double* phi = latest_phi(P);
  const int total = P.nnod * ng;
  for (int q = start; q < total; q += stride) {
    const int n = q % P.nnod, g = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    double L[3];
    net_leakage(G, phi + (size_t)g * P.NBH, P.df + (size_t)g * 6 * NB, P.dn + (size_t)g * 6 * NB, b, L);
    if (P.cmode == 2) {
      // transient: the step's external source joins the leakage (mod_nodal.f90:1031-1035)
      const double e = P.exsrc[(size_t)g * NB + b];
      P.S[((size_t)0 * ng + g) * NB + b] = L[1] + L[2] - e;
      P.S[((size_t)1 * ng + g) * NB + b] = L[0] + L[2] - e;
      P.S[((size_t)2 * ng + g) * NB + b] = L[0] + L[1] - e;
    } else {
      P.S[((size_t)0 * ng + g) * NB + b] = L[1] + L[2];
      P.S[((size_t)1 * ng + g) * NB + b] = L[0] + L[2];
      P.S[((size_t)2 * ng + g) * NB + b] = L[0] + L[1];
    }
  }
}

// Line position of a node along direction u.
struct LinePos {
  bool first, last, refl_first, refl_last;
  int offp;        // box offset of the plus neighbour
};

__device__ __forceinline__ LinePos line_pos(const BoxGeom& G, int u, int b) {
  const unsigned m = G.nbm[b];
  LinePos L;
  L.first = !(m & (1u << (2 * u + 1)));
  L.last = !(m & (1u << (2 * u)));
  L.refl_first = G.bcf[2 * u + 1] == 2;
  L.refl_last = G.bcf[2 * u] == 2;
  L.offp = face_off(G, 2 * u);
  return L;
}

// Geometry factors of the transverse-leakage moments of node b along u
// (TLUpd1, mod_nodal.f90:1047-1199; TLUpd2, :1203-1341).  With S the
// zeroth-order source along u and n, p, m the node and its plus and minus
// neighbours:
//   first moment  = c1p (S_p - S_n) + c1m (S_n - S_m)
//   second moment = c2p (S_p - S_n) + c2m (S_m - S_n)
// multiplied by 0.25 h^2 / D_g.  A reflective line end mirrors the missing
// neighbour (tm or tp = 1); any other line end uses the one-sided forms.
// The factors do not depend on the group, so they are formed once per
// node and direction.
struct TLGeom {
  double c1p, c1m, c2p, c2m;
  int offp;
  bool has_p, has_m;
};

__device__ __forceinline__ TLGeom tl_geom(const BoxGeom& G, int u, int b) {
  const LinePos L = line_pos(G, u, b);
  TLGeom T;
  T.offp = L.offp;
  T.has_p = !L.last;
  T.has_m = !L.first;
  T.c1p = T.c1m = T.c2p = T.c2m = 0.0;
  const double h0 = hdir(G, u, b);
  if (L.first) {
    const double tp = hdir(G, u, b + L.offp) / h0;
    const double p1p = tp + 1.0;
    if (L.refl_first) {
      const double tm = 1.0, p1m = tm + 1.0, p2m = 2.0 * tm + 1.0;
      const double hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
      T.c1p = p1m * p2m / hp;
      T.c2p = p1m / hp;
    } else {
      T.c1p = 1.0 / p1p;
    }
  } else if (L.last) {
    const double tm = hdir(G, u, b - L.offp) / h0;
    const double p1m = tm + 1.0;
    if (L.refl_last) {
      const double tp = 1.0, p1p = tp + 1.0, p2p = 2.0 * tp + 1.0;
      const double hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
      T.c1m = p1p * p2p / hp;
      T.c2m = p1p / hp;
    } else {
      T.c1m = 1.0 / p1m;
    }
  } else {
    const double tm = hdir(G, u, b - L.offp) / h0;
    const double tp = hdir(G, u, b + L.offp) / h0;
    const double p1m = tm + 1.0, p2m = 2.0 * tm + 1.0;
    const double p1p = tp + 1.0, p2p = 2.0 * tp + 1.0;
    const double hp = 2.0 * p1m * p1p * (tm + tp + 1.0);
    T.c1p = p1m * p2m / hp;
    T.c1m = p1p * p2p / hp;
    T.c2p = p1m / hp;
    T.c2m = p1p / hp;
  }
  return T;
}

// get_B (mod_nodal.f90:1345-1405): buckling matrix of node b in direction u,
// B(g,h) = 0.25 h^2 / D_g * (sigr_g delta_gh - sigs(h->g) - chi_g nuf_h / k)
// (forward, cmode 1), the transposed group coupling (adjoint, cmode 0), or
// the transient form (cmode 2).
template <int NG>
__device__ __forceinline__ void get_B(const NodalParams& P, int b, double invKe, const double (&fac)[NG],
                                      double (&B)[NG][NG]) {
  const int NB = P.G.NB;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
#pragma unroll
    for (int h = 0; h < NG; ++h) {
      double dum;
      if (P.cmode == 2) {
        // transient (mod_nodal.f90:1379-1390): prompt and delayed fission of
        // the step, no eigenvalue; the diagonal carries chi twice, as the
        // reference writes it
        const double w = P.wnode[b], chi = P.chin[(size_t)g * NB + b];
        if (g == h) dum = P.sigr[(size_t)g * NB + b] - w * chi * chi * P.nuf[(size_t)h * NB + b];
        else dum = -P.sigs[((size_t)h * NG + g) * NB + b] - w * chi * P.nuf[(size_t)h * NB + b];
      } else if (g == h) {
        dum = P.sigr[(size_t)g * NB + b] - P.chin[(size_t)g * NB + b] * P.nuf[(size_t)h * NB + b] * invKe;
      } else if (P.cmode == 1) {
        dum = -P.sigs[((size_t)h * NG + g) * NB + b] - P.chin[(size_t)g * NB + b] * P.nuf[(size_t)h * NB + b] * invKe;
      } else {
        dum = -P.sigs[((size_t)g * NG + h) * NB + b] - P.chin[(size_t)h * NB + b] * P.nuf[(size_t)g * NB + b] * invKe;
      }
      B[g][h] = fac[g] * dum;
    }
  }
}

// Constant k (0..5 = A,B,E,F,G,H) of node b, direction u, group g.
__device__ __forceinline__ double nconst(const NodalParams& P, int u, int k, int g, int b) {
  if (P.pnm) {
    double c[6];
    pnm_consts(c);
    return c[k];
  }
  return P.sanm[(((size_t)u * 6 + k) * P.ng + g) * P.G.NB + b];
}

__device__ __forceinline__ double bc_at(const NodalParams& P, int u, int g, int h, int b) {
  return P.Bc[(((size_t)u * P.ng + g) * P.ng + h) * P.G.NB + b];
}

// LU_solve (mod_nodal.f90:829-897): Doolittle elimination without pivoting,
// L stored in place of the eliminated entries, one reciprocal per pivot.
// Returns false when an input diagonal is below the reference's 10e-5
// (single precision) threshold.
template <int M>
__device__ __forceinline__ bool lu_solve(double (&U)[M][M], double (&x)[M]) {
#pragma unroll
  for (int i = 0; i < M; ++i)
    if (fabs(U[i][i]) < kF1em4) return false;
  double inv[M];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    inv[i] = 1.0 / U[i][i];
#pragma unroll
    for (int j = i + 1; j < M; ++j) {
      const double piv = U[j][i] * inv[i];
#pragma unroll
      for (int k = i + 1; k < M; ++k) U[j][k] = U[j][k] - piv * U[i][k];
      U[j][i] = piv;
    }
  }
#pragma unroll
  for (int i = 1; i < M; ++i) {
    double isum = 0.0;
#pragma unroll
    for (int k = 0; k < i; ++k) isum = isum + U[i][k] * x[k];
    x[i] = x[i] - isum;
  }
  x[M - 1] = x[M - 1] * inv[M - 1];
#pragma unroll
  for (int i = M - 2; i >= 0; --i) {
    double isum = 0.0;
#pragma unroll
    for (int k = i + 1; k < M; ++k) isum = isum + U[i][k] * x[k];
    x[i] = (x[i] - isum) * inv[i];
  }
  return true;
}

__device__ __forceinline__ void record_error(OuterCtl* C, int code, int b) {
  if (atomicCAS(&C->status, 0, code) == 0) C->err_node = b;
}

// ---------------------------------------------------------------------------
// Per node and direction: the buckling matrix (stored for k_interface),
// a2 (get_a2matvec + LU_solve), a4 (get_a4) and the first transverse-leakage
// moment (TLUpd1).
// ---------------------------------------------------------------------------
template <int NG>
__device__ __forceinline__ void node_prep_items(const NodalParams& P, int start, int stride) {
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const double* phi = latest_phi(P);
  const double invKe = 1.0 / *(const volatile double*)&P.ctl->Ke;
  const int total = P.nnod * 3;
  for (int q = start; q < total; q += stride) {
    const int n = q % P.nnod, u = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    const double h = hdir(G, u, b);
    double fac[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) fac[g] = 0.25 * (h * h) / P.D[(size_t)g * NB + b];
    double Bc[NG][NG];
    get_B<NG>(P, b, invKe, fac, Bc);
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) P.Bc[(((size_t)u * NG + g) * NG + hh) * NB + b] = Bc[g][hh];
    const TLGeom T = tl_geom(G, u, b);
    const double* S = P.S + (size_t)u * NG * NB;
    double M[NG][NG], rhs[NG], Lm2[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const double Ev = nconst(P, u, 2, g, b);
      const double Sn = S[(size_t)g * NB + b];
      const double dSp = T.has_p ? S[(size_t)g * NB + b + T.offp] - Sn : 0.0;
      const double dSm = T.has_m ? S[(size_t)g * NB + b - T.offp] - Sn : 0.0;
      double Bf = 0.0;
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) {
        M[g][hh] = (hh == g) ? Bc[g][hh] * Ev + 3.0 : Bc[g][hh] * Ev;
        Bf = Bf + Bc[g][hh] * phi[(size_t)hh * P.NBH + b];
      }
      Lm2[g] = fac[g] * (T.c2p * dSp + T.c2m * dSm);                          // TLUpd2
      rhs[g] = Bf - Ev * Lm2[g] + fac[g] * Sn;
      P.L1[((size_t)u * NG + g) * NB + b] = fac[g] * (T.c1p * dSp - T.c1m * dSm);  // TLUpd1
    }
    if (!lu_solve<NG>(M, rhs)) {
      record_error(P.ctl, ADP_ERR_PIVOT, b);
      continue;
    }
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      double Bf = 0.0;
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) Bf = Bf + Bc[g][hh] * rhs[hh];
      const size_t o = ((size_t)u * NG + g) * NB + b;
      P.a2[o] = rhs[g];
      P.a4[o] = nconst(P, u, 1, g, b) * (Bf + Lm2[g]);
    }
  }
}

struct NdBest {
  double val;
  long long key;
  int loc;
};

__device__ __forceinline__ void nd_consider(NdBest& best, double val, long long key, int loc) {
  if (val > best.val || (val == best.val && key < best.key)) {
    best.val = val;
    best.key = key;
    best.loc = loc;
  }
}

// Per-node, per-direction, per-group quantities of one side of a face.
struct Side {
  double A, F, Gc, H, a2, a4, L1, f, D;
};

__device__ __forceinline__ Side side_at(const NodalParams& P, const double* phi, int u, int g, int b) {
  const int NB = P.G.NB;
  const size_t o = ((size_t)u * P.ng + g) * NB + b;
  Side s;
  s.A = nconst(P, u, 0, g, b);
  s.F = nconst(P, u, 3, g, b);
  s.Gc = nconst(P, u, 4, g, b);
  s.H = nconst(P, u, 5, g, b);
  s.a2 = P.a2[o];
  s.a4 = P.a4[o];
  s.L1 = P.L1[o];
  s.f = phi[(size_t)g * P.NBH + b];
  s.D = P.D[(size_t)g * NB + b];
  return s;
}

// ---------------------------------------------------------------------------
// Per node and direction: the minus face of the node (the interior
// interface with its predecessor, or the first boundary face of the line),
// plus the last boundary face when the node ends its line.  Per-node
// quantities are read from memory where they are used, to keep the 2G x 2G
// system in registers.
// ---------------------------------------------------------------------------
template <int NG>
__device__ __forceinline__ void interface_items(const NodalParams& P, int start, int stride, NdBest& best) {
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const double* phi = latest_phi(P);
  const int total = P.nnod * 3;
  for (int q = start; q < total; q += stride) {
    const int n = q % P.nnod, u = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    const LinePos L = line_pos(G, u, b);
    const int sf = 2 * u;         // plus face of u (X+, Y+, Z+); sf+1 is the minus face
    const long long ev = P.evbase[(size_t)u * NB + b];
    const double two_hp = 2.0 / hdir(G, u, b);
    if (!L.first) {
      // interior interface n = predecessor, p = b (get_coefs + get_a1matvec)
      const int bn = b - L.offp;
      const double two_hn = 2.0 / hdir(G, u, bn);
      double R[2 * NG][2 * NG], x[2 * NG];
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const Side sn = side_at(P, phi, u, g, bn), sp = side_at(P, phi, u, g, b);
        const double Pn = sn.D * two_hn, Pp = sp.D * two_hp;
        const double dcn = P.dc[((size_t)g * 6 + sf) * NB + bn];
        const double dcp = P.dc[((size_t)g * 6 + sf + 1) * NB + b];
#pragma unroll
        for (int hh = 0; hh < NG; ++hh) {
          const double Bn = bc_at(P, u, g, hh, bn), Bp = bc_at(P, u, g, hh, b);
          if (hh == g) {
            R[g][g] = -Pn * (Bn * sn.F + 1.0);
            R[g][g + NG] = Pp * (Bp * sp.F + 1.0);
            R[g + NG][g] = dcn * (Bn * sn.A + 1.0);
            R[g + NG][g + NG] = dcp * (Bp * sp.A + 1.0);
          } else {
            R[g][hh] = -Pn * Bn * sn.F;
            R[g][hh + NG] = Pp * Bp * sp.F;
            R[g + NG][hh] = dcn * Bn * sn.A;
            R[g + NG][hh + NG] = dcp * Bp * sp.A;
          }
        }
        x[g] = Pn * (3.0 * sn.a2 + sn.Gc * sn.a4 + sn.F * sn.L1) + Pp * (3.0 * sp.a2 + sp.Gc * sp.a4 - sp.F * sp.L1);
        // ADF pairing of mod_nodal.f90:693-694 kept as written there
        x[g + NG] = dcp * (sp.a2 + sp.a4 + sp.f - sn.A * sn.L1) - dcn * (sn.a2 + sn.a4 + sn.f + sp.A * sp.L1);
      }
      if (!lu_solve<2 * NG>(R, x)) {
        record_error(P.ctl, ADP_ERR_PIVOT, bn);
      } else {
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          const Side sn = side_at(P, phi, u, g, bn);
          const double fp = phi[(size_t)g * P.NBH + b];
          double Bf = 0.0;
#pragma unroll
          for (int hh = 0; hh < NG; ++hh) Bf = Bf + bc_at(P, u, g, hh, bn) * x[hh];
          const double a3 = sn.A * (Bf + sn.L1);
          const double jp = -sn.D * two_hn * (x[g] + 3.0 * sn.a2 + sn.H * a3 + sn.Gc * sn.a4);
          const size_t on = ((size_t)g * 6 + sf) * NB + bn;
          const double ndpr = P.dn[on];
          const double dnew = (P.df[on] * (sn.f - fp) - jp) / (sn.f + fp);
          P.dn[on] = dnew;
          P.dn[((size_t)g * 6 + sf + 1) * NB + b] = dnew;
          nd_consider(best, fabs(dnew - ndpr), ev * NG + g, bn);
        }
      }
    } else {
      // first boundary face of the line (get_coefs_first + get_a1matvec_first)
      const int bc = G.bcf[sf + 1];
      double A[NG][NG], x[NG];
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const Side sp = side_at(P, phi, u, g, b);
        const double Pp = sp.D * two_hp;
        const double dcv = P.dc[((size_t)g * 6 + sf + 1) * NB + b];
#pragma unroll
        for (int hh = 0; hh < NG; ++hh) {
          const double Bc = bc_at(P, u, g, hh, b);
          if (bc == 2) A[g][hh] = (hh == g) ? Pp * (Bc * sp.F + 1.0) : Pp * Bc * sp.F;
          else if (bc == 1)
            A[g][hh] = (hh == g) ? -dcv * (1.0 + sp.A * Bc) - 2.0 * Pp * (sp.A * Bc * sp.H + 1.0)
                                 : -dcv * sp.A * Bc - 2.0 * Pp * sp.A * Bc * sp.H;
          else A[g][hh] = (hh == g) ? dcv * (1.0 + sp.A * Bc) : dcv * sp.A * Bc;
        }
        if (bc == 2) x[g] = Pp * (3.0 * sp.a2 + sp.Gc * sp.a4 - sp.F * sp.L1);
        else if (bc == 1)
          x[g] = 2.0 * Pp * (sp.A * sp.H * sp.L1 - 3.0 * sp.a2 - sp.Gc * sp.a4) - dcv * (sp.a2 + sp.a4 + sp.f - sp.A * sp.L1);
        else x[g] = dcv * (sp.a2 + sp.a4 + sp.f - sp.A * sp.L1);
      }
      if (!lu_solve<NG>(A, x)) {
        record_error(P.ctl, ADP_ERR_PIVOT, b);
      } else {
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          const Side sp = side_at(P, phi, u, g, b);
          double Bf = 0.0;
#pragma unroll
          for (int hh = 0; hh < NG; ++hh) Bf = Bf + bc_at(P, u, g, hh, b) * x[hh];
          const double a3 = sp.A * (Bf + sp.L1);
          const double jp = -sp.D * two_hp * (x[g] - 3.0 * sp.a2 + sp.H * a3 - sp.Gc * sp.a4);
          const size_t op = ((size_t)g * 6 + sf + 1) * NB + b;
          const double ndpr = P.dn[op];
          const double dnew = -(jp / sp.f + P.df[op]);
          P.dn[op] = dnew;
          nd_consider(best, fabs(dnew - ndpr), ev * NG + g, b);
        }
      }
    }
    if (L.last) {
      // last boundary face of the line (get_coefs_last + get_a1matvec_last)
      const int bc = G.bcf[sf];
      double A[NG][NG], x[NG];
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const Side sn = side_at(P, phi, u, g, b);
        const double Pn = sn.D * two_hp;
        const double dcv = P.dc[((size_t)g * 6 + sf) * NB + b];
#pragma unroll
        for (int hh = 0; hh < NG; ++hh) {
          const double Bc = bc_at(P, u, g, hh, b);
          if (bc == 2) A[g][hh] = (hh == g) ? -Pn * (Bc * sn.F + 1.0) : -Pn * Bc * sn.F;
          else if (bc == 1)
            A[g][hh] = (hh == g) ? dcv * (1.0 + sn.A * Bc) + 2.0 * Pn * (sn.A * Bc * sn.H + 1.0)
                                 : dcv * sn.A * Bc + 2.0 * Pn * sn.A * Bc * sn.H;
          else A[g][hh] = (hh == g) ? dcv * (1.0 + sn.A * Bc) : dcv * sn.A * Bc;
        }
        if (bc == 2) x[g] = Pn * (3.0 * sn.a2 + sn.Gc * sn.a4 + sn.F * sn.L1);
        else if (bc == 1)
          x[g] = -2.0 * Pn * (sn.A * sn.H * sn.L1 + 3.0 * sn.a2 + sn.Gc * sn.a4) - dcv * (sn.a2 + sn.a4 + sn.f + sn.A * sn.L1);
        else x[g] = -dcv * (sn.a2 + sn.a4 + sn.f + sn.A * sn.L1);
      }
      if (!lu_solve<NG>(A, x)) {
        record_error(P.ctl, ADP_ERR_PIVOT, b);
      } else {
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          const Side sn = side_at(P, phi, u, g, b);
          double Bf = 0.0;
#pragma unroll
          for (int hh = 0; hh < NG; ++hh) Bf = Bf + bc_at(P, u, g, hh, b) * x[hh];
          const double a3 = sn.A * (Bf + sn.L1);
          const double jp = -sn.D * two_hp * (x[g] + 3.0 * sn.a2 + sn.H * a3 + sn.Gc * sn.a4);
          const size_t on = ((size_t)g * 6 + sf) * NB + b;
          const double ndpr = P.dn[on];
          const double dnew = -(jp / sn.f - P.df[on]);
          P.dn[on] = dnew;
          nd_consider(best, fabs(dnew - ndpr), (ev + 1) * NG + g, b);
        }
      }
    }
  }
}

// Block reduction of (value, key, location); thread 0 stores the block's
// best in slot `slot` of the partial arrays.
__device__ __forceinline__ void nd_block_reduce(const NodalParams& P, NdBest best, int slot) {
  __shared__ double sv[32];
  __shared__ long long sk[32];
  __shared__ int sl[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    NdBest other;
    other.val = __shfl_xor_sync(0xffffffffu, best.val, o);
    other.key = __shfl_xor_sync(0xffffffffu, best.key, o);
    other.loc = __shfl_xor_sync(0xffffffffu, best.loc, o);
    nd_consider(best, other.val, other.key, other.loc);
  }
  if (lane == 0) {
    sv[w] = best.val;
    sk[w] = best.key;
    sl[w] = best.loc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    NdBest bb{sv[0], sk[0], sl[0]};
    for (int k = 1; k < nw; ++k) nd_consider(bb, sv[k], sk[k], sl[k]);
    P.nd_val[slot] = bb.val;
    P.nd_key[slot] = bb.key;
    P.nd_loc[slot] = bb.loc;
  }
  __syncthreads();
}

// ndmax with its location, the divergence check (mod_nodal.f90:131-142) and
// the convergence test of the outer that triggered the update
// (mod_cmfd.f90:495-505).
// Run by the 32 lanes of one warp: the lanes scan the partials, then a
// shuffle reduction; (value descending, sweep key ascending) is a total
// order, so the winner does not depend on the scan order.  Lane 0 then
// updates the control block.
__device__ __forceinline__ void nodal_finish_warp(const NodalParams& P, int nparts) {
  OuterCtl* C = P.ctl;
  const int lane = threadIdx.x & 31;
  NdBest bb{0.0, 0x7fffffffffffffffLL, -1};
  for (int k = lane; k < nparts; k += 32)
    nd_consider(bb, __ldcg(P.nd_val + k), __ldcg(P.nd_key + k), __ldcg(P.nd_loc + k));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, bb.val, o);
    const long long key = __shfl_xor_sync(0xffffffffu, bb.key, o);
    const int loc = __shfl_xor_sync(0xffffffffu, bb.loc, o);
    nd_consider(bb, v, key, loc);
  }
  if (lane != 0) return;
  C->ndmax = bb.val;
  if (bb.val > 0.0 && bb.loc >= 0) {
    const int b = bb.loc;
    C->im = b % P.G.nxx + 1;
    C->jm = (b / P.G.nxx) % P.G.nyy + 1;
    C->km = b / P.G.plane + 1;
  }
  C->nodal_updates += 1;
  C->nodal_due = 0;
  const int q = *(volatile int*)&C->p - 1;
  if (q >= 0 && q < P.nout) {
    P.tr_ndmax[q] = bb.val;
    P.tr_flags[q] |= 2;
  }
  if (bb.val > 1.e3) {
    set_status(C, ADP_ERR_DIVERGED);
    return;
  }
  const bool conv = *(volatile double*)&C->ser < P.serc && *(volatile double*)&C->fer < P.ferc && bb.val < kF1em2;
  C->converged = conv ? 1 : 0;
  C->max_reached = (!conv && q + 1 >= P.nout) ? 1 : 0;
}

}  // namespace adp
