// Reverse-mode derivative of the two-node nodal update and the kernels of
// the adjoint of the nonlinear fixed point (CMFD eigenproblem + nodal update).
//
// The nodal update (nodal_update / nodal_update_pnm, mod_nodal.f90:18-278) is
// a function N(phi, d, k; Sigma) of the flux, the coupling coefficients d of
// the faces, the eigenvalue and the cross sections.  Given an adjoint lam of
// the new coupling coefficients, the kernels here form lam^T N_phi, lam^T N_d,
// lam^T N_k and lam^T N_Sigma by running the update's stages backwards:
//
//   k_nadj_iface<G>  nodal_coup_upd, get_a3, LU_solve, get_a1matvec*      per face
//   k_nadj_node<G>   get_a4, LU_solve, get_a2matvec, TLUpd1/2, get_B,
//                    get_ABEFGH                                            per node, direction
//   k_nadj_lbar      get_source (S1..S3 -> leakages)                       per node, group
//   k_nadj_leak      Lxyz (leakages -> face currents -> phi, d, df)         per node, group
//   k_nadj_params    coup_coef (df -> D), sums over directions             per node, group
//
// Each stage is a gather: a face writes the adjoints of its two sides into
// per-(node, direction) slots, a (node, direction) item writes what it owes
// its neighbours into its own slots and the next stage reads them, so every
// sum is formed in a fixed order by one thread and no atomics are needed.
// The forward quantities (S, a2, a4, L1, Bc) come from k_tl_source and
// k_node_prep run at the state being differentiated; the face systems are
// re-formed and re-factored here.
//
// Canonical face slots: the coupling coefficient of an interior face is one
// variable (nod(n)%dn(sf) and nod(p)%dn(sf+1) are set together,
// mod_nodal.f90:328-329).  Adjoints of face variables live in the
// [g][6][NB] layout at the minus face (2u+1) of every node and at the plus
// face (2u) of a node whose plus face is a boundary face; other slots stay 0.
#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"
#include "nodal_body.cuh"

namespace adp {

// ---- small dense algebra ---------------------------------------------------

// Doolittle factorisation without pivoting in place (L below the diagonal,
// unit diagonal implied; U on and above), inv[i] = 1 / U[i][i].  Same
// elimination as lu_solve.  The forward update already passed its pivot
// test at this state; a zero pivot here gives inf, caught by the host's
// finiteness check of the result.
template <int M>
__device__ __forceinline__ void lu_factor(double (&U)[M][M], double (&inv)[M]) {
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
}

// x <- (LU)^{-1} x
template <int M>
__device__ __forceinline__ void lu_apply(const double (&U)[M][M], const double (&inv)[M], double (&x)[M]) {
#pragma unroll
  for (int i = 1; i < M; ++i) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < i; ++k) s = fma(U[i][k], x[k], s);
    x[i] -= s;
  }
#pragma unroll
  for (int i = M - 1; i >= 0; --i) {
    double s = 0.0;
#pragma unroll
    for (int k = i + 1; k < M; ++k) s = fma(U[i][k], x[k], s);
    x[i] = (x[i] - s) * inv[i];
  }
}

// y <- (LU)^{-T} y: U^T w = y (forward), then L^T z = w (backward).
template <int M>
__device__ __forceinline__ void lu_apply_T(const double (&U)[M][M], const double (&inv)[M], double (&y)[M]) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < i; ++k) s = fma(U[k][i], y[k], s);
    y[i] = (y[i] - s) * inv[i];
  }
#pragma unroll
  for (int i = M - 2; i >= 0; --i) {
    double s = 0.0;
#pragma unroll
    for (int k = i + 1; k < M; ++k) s = fma(U[k][i], y[k], s);
    y[i] -= s;
  }
}

// ---- SANM constants and their derivative in alpha ---------------------------
// get_ABEFGH (mod_nodal.f90:1409-1451) evaluated on (value, d/dalpha) pairs.
struct Dl {
  double v, d;
};
__device__ __forceinline__ Dl operator+(Dl a, Dl b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dl operator-(Dl a, Dl b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dl operator*(Dl a, Dl b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dl operator*(double c, Dl a) { return {c * a.v, c * a.d}; }
__device__ __forceinline__ Dl operator/(Dl a, Dl b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
__device__ __forceinline__ Dl operator/(double c, Dl b) { return {c / b.v, -c * b.d / (b.v * b.v)}; }

// d(A, B, E, F, G, H)/dalpha at alpha
__device__ __forceinline__ void sanm_dconsts(double alpha, double (&dc)[6]) {
  const Dl a{alpha, 1.0};
  const Dl a2 = a * a;
  const Dl sh{sinh(alpha), cosh(alpha)}, ch{cosh(alpha), sinh(alpha)};
  const Dl m0c = sh / a;
  const Dl m1s = 3.0 * (ch / a - sh / a2);
  const Dl m2c = 5.0 * (sh / a - 3.0 * ch / a2 + 3.0 * sh / (a2 * a));
  dc[0] = ((sh - m1s) / (a2 * m1s)).d;
  dc[1] = ((ch - m0c - m2c) / (a2 * m2c)).d;
  dc[2] = (m0c / m2c - 3.0 / a2).d;
  dc[3] = ((a * ch - m1s) / (a2 * m1s)).d;
  dc[4] = ((a * sh - 3.0 * m2c) / (ch - m0c - m2c)).d;
  dc[5] = ((a * ch - m1s) / (sh - m1s)).d;
}

// ---- per-side adjoint record ----------------------------------------------
// Adjoints of the per-(node, direction, group) quantities a face reads:
// a2, a4, L1, the constants A, F, G, H, D (through P = 2D/h and the
// current), the flux, and the buckling matrix Bc.
template <int NG>
struct SideBar {
  double a2[NG], a4[NG], L1[NG], A[NG], F[NG], Gc[NG], H[NG], D[NG], f[NG], Bc[NG][NG];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      a2[g] = a4[g] = L1[g] = A[g] = F[g] = Gc[g] = H[g] = D[g] = f[g] = 0.0;
#pragma unroll
      for (int h = 0; h < NG; ++h) Bc[g][h] = 0.0;
    }
  }
};

template <int NG>
constexpr int side_nq() { return 9 * NG + NG * NG; }

// slot q of side s (0: the node as p of its minus face, 1: as n of its plus
// face), direction u, box row b
__device__ __forceinline__ size_t side_ix(int nq, int NB, int s, int u, int q, int b) {
  return (((size_t)s * 3 + u) * nq + q) * NB + b;
}

template <int NG>
__device__ __forceinline__ void side_store(double* dst, int NB, int s, int u, int b, const SideBar<NG>& t) {
  constexpr int nq = side_nq<NG>();
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    dst[side_ix(nq, NB, s, u, 0 * NG + g, b)] = t.a2[g];
    dst[side_ix(nq, NB, s, u, 1 * NG + g, b)] = t.a4[g];
    dst[side_ix(nq, NB, s, u, 2 * NG + g, b)] = t.L1[g];
    dst[side_ix(nq, NB, s, u, 3 * NG + g, b)] = t.A[g];
    dst[side_ix(nq, NB, s, u, 4 * NG + g, b)] = t.F[g];
    dst[side_ix(nq, NB, s, u, 5 * NG + g, b)] = t.Gc[g];
    dst[side_ix(nq, NB, s, u, 6 * NG + g, b)] = t.H[g];
    dst[side_ix(nq, NB, s, u, 7 * NG + g, b)] = t.D[g];
    dst[side_ix(nq, NB, s, u, 8 * NG + g, b)] = t.f[g];
#pragma unroll
    for (int h = 0; h < NG; ++h) dst[side_ix(nq, NB, s, u, 9 * NG + g * NG + h, b)] = t.Bc[g][h];
  }
}

template <int NG>
__device__ __forceinline__ void side_add(const double* src, int NB, int s, int u, int b, SideBar<NG>& t) {
  constexpr int nq = side_nq<NG>();
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    t.a2[g] += src[side_ix(nq, NB, s, u, 0 * NG + g, b)];
    t.a4[g] += src[side_ix(nq, NB, s, u, 1 * NG + g, b)];
    t.L1[g] += src[side_ix(nq, NB, s, u, 2 * NG + g, b)];
    t.A[g] += src[side_ix(nq, NB, s, u, 3 * NG + g, b)];
    t.F[g] += src[side_ix(nq, NB, s, u, 4 * NG + g, b)];
    t.Gc[g] += src[side_ix(nq, NB, s, u, 5 * NG + g, b)];
    t.H[g] += src[side_ix(nq, NB, s, u, 6 * NG + g, b)];
    t.D[g] += src[side_ix(nq, NB, s, u, 7 * NG + g, b)];
    t.f[g] += src[side_ix(nq, NB, s, u, 8 * NG + g, b)];
#pragma unroll
    for (int h = 0; h < NG; ++h) t.Bc[g][h] += src[side_ix(nq, NB, s, u, 9 * NG + g * NG + h, b)];
  }
}

// ---------------------------------------------------------------------------
// Stage 1: faces.  Item (b, u) takes the minus face of b (interior with its
// predecessor, or the line's first boundary face) and, when b ends its line,
// the last boundary face.
// ---------------------------------------------------------------------------

// Reverse of the boundary face forms of get_a1matvec_first / _last
// (mod_nodal.f90:483-626) with nodal_coup_upd's boundary branches
// (:338-368).  first: the node is p of its minus face; otherwise n of its
// plus face.  Returns |dn_new - dn| for the fixed-point residual.
template <int NG>
__device__ __forceinline__ double bface_adj(const NadjParams& Q, const double* phi, int u, int b, bool first,
                                            SideBar<NG>& t) {
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const int f = first ? 2 * u + 1 : 2 * u;
  const int bc = G.bcf[f];
  const double two_h = 2.0 / hdir(G, u, b);
  double Am[NG][NG], x[NG];
  Side sd[NG];
  double dcv[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    sd[g] = side_at(P, phi, u, g, b);
    dcv[g] = P.dc[((size_t)g * 6 + f) * NB + b];
    const double Pv = sd[g].D * two_h;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) {
      const double Bc = bc_at(P, u, g, hh, b);
      const double dl = (hh == g) ? 1.0 : 0.0;
      if (first) {
        if (bc == 2) Am[g][hh] = Pv * (Bc * sd[g].F + dl);
        else if (bc == 1) Am[g][hh] = -dcv[g] * (dl + sd[g].A * Bc) - 2.0 * Pv * (sd[g].A * Bc * sd[g].H + dl);
        else Am[g][hh] = dcv[g] * (dl + sd[g].A * Bc);
      } else {
        if (bc == 2) Am[g][hh] = -Pv * (Bc * sd[g].F + dl);
        else if (bc == 1) Am[g][hh] = dcv[g] * (dl + sd[g].A * Bc) + 2.0 * Pv * (sd[g].A * Bc * sd[g].H + dl);
        else Am[g][hh] = dcv[g] * (dl + sd[g].A * Bc);
      }
    }
    const Side& s = sd[g];
    if (first) {
      if (bc == 2) x[g] = Pv * (3.0 * s.a2 + s.Gc * s.a4 - s.F * s.L1);
      else if (bc == 1) x[g] = 2.0 * Pv * (s.A * s.H * s.L1 - 3.0 * s.a2 - s.Gc * s.a4) - dcv[g] * (s.a2 + s.a4 + s.f - s.A * s.L1);
      else x[g] = dcv[g] * (s.a2 + s.a4 + s.f - s.A * s.L1);
    } else {
      if (bc == 2) x[g] = Pv * (3.0 * s.a2 + s.Gc * s.a4 + s.F * s.L1);
      else if (bc == 1) x[g] = -2.0 * Pv * (s.A * s.H * s.L1 + 3.0 * s.a2 + s.Gc * s.a4) - dcv[g] * (s.a2 + s.a4 + s.f + s.A * s.L1);
      else x[g] = -dcv[g] * (s.a2 + s.a4 + s.f + s.A * s.L1);
    }
  }
  double inv[NG];
  lu_factor<NG>(Am, inv);
  double a1[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) a1[g] = x[g];
  lu_apply<NG>(Am, inv, a1);
  // forward tail and its reverse
  const double sgn = first ? -1.0 : 1.0;   // a2 and a4 enter the current with this sign
  double a1b[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) a1b[g] = 0.0;
  double resid = 0.0;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const Side& s = sd[g];
    double Bf = 0.0;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) Bf = Bf + bc_at(P, u, g, hh, b) * a1[hh];
    const double a3 = s.A * (Bf + s.L1);
    const double T = a1[g] + sgn * 3.0 * s.a2 + s.H * a3 + sgn * s.Gc * s.a4;
    const double jp = -s.D * two_h * T;
    const size_t slot = ((size_t)g * 6 + f) * NB + b;
    const double df = P.df[slot];
    const double dnew = first ? -(jp / s.f + df) : -(jp / s.f - df);
    resid = fmax(resid, fabs(dnew - P.dn[slot]));
    const double lam = Q.lam[slot];
    // dnew = -(jp / f) -/+ df
    const double Jb = -lam / s.f;
    t.f[g] += lam * jp / (s.f * s.f);
    Q.dfbar[slot] = first ? -lam : lam;
    const double Tb = Jb * (-s.D * two_h);
    t.D[g] += Jb * (-two_h * T);
    a1b[g] += Tb;
    t.a2[g] += sgn * 3.0 * Tb;
    t.H[g] += Tb * a3;
    const double a3b = Tb * s.H;
    t.Gc[g] += sgn * Tb * s.a4;
    t.a4[g] += sgn * Tb * s.Gc;
    // a3 = A (Bc a1 + L1)
    t.A[g] += a3b * (Bf + s.L1);
    const double q = a3b * s.A;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) {
      t.Bc[g][hh] += q * a1[hh];
      a1b[hh] += q * bc_at(P, u, g, hh, b);
    }
    t.L1[g] += q;
  }
  // a1 = Am^{-1} x
  double xb[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) xb[g] = a1b[g];
  lu_apply_T<NG>(Am, inv, xb);
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const Side& s = sd[g];
    const double Pv = s.D * two_h;
    double Pb = 0.0;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) {
      const double Bc = bc_at(P, u, g, hh, b);
      const double dl = (hh == g) ? 1.0 : 0.0;
      const double Ab = -xb[g] * a1[hh];
      if (bc == 2) {
        const double sg = first ? 1.0 : -1.0;
        t.Bc[g][hh] += Ab * sg * Pv * s.F;
        t.F[g] += Ab * sg * Pv * Bc;
        Pb += Ab * sg * (Bc * s.F + dl);
      } else if (bc == 1) {
        const double sg = first ? -1.0 : 1.0;
        t.Bc[g][hh] += Ab * sg * (dcv[g] * s.A + 2.0 * Pv * s.A * s.H);
        t.A[g] += Ab * sg * (dcv[g] * Bc + 2.0 * Pv * Bc * s.H);
        t.H[g] += Ab * sg * 2.0 * Pv * s.A * Bc;
        Pb += Ab * sg * 2.0 * (s.A * Bc * s.H + dl);
      } else {
        t.Bc[g][hh] += Ab * dcv[g] * s.A;
        t.A[g] += Ab * dcv[g] * Bc;
      }
    }
    const double X = xb[g];
    if (bc == 2) {
      const double sg = first ? -1.0 : 1.0;   // sign of the F L1 term
      Pb += X * (3.0 * s.a2 + s.Gc * s.a4 + sg * s.F * s.L1);
      t.a2[g] += 3.0 * X * Pv;
      t.Gc[g] += X * Pv * s.a4;
      t.a4[g] += X * Pv * s.Gc;
      t.F[g] += sg * X * Pv * s.L1;
      t.L1[g] += sg * X * Pv * s.F;
    } else if (bc == 1) {
      if (first) {
        Pb += X * 2.0 * (s.A * s.H * s.L1 - 3.0 * s.a2 - s.Gc * s.a4);
        t.A[g] += X * (2.0 * Pv * s.H * s.L1 + dcv[g] * s.L1);
        t.H[g] += X * 2.0 * Pv * s.A * s.L1;
        t.L1[g] += X * (2.0 * Pv * s.A * s.H + dcv[g] * s.A);
      } else {
        Pb += X * (-2.0) * (s.A * s.H * s.L1 + 3.0 * s.a2 + s.Gc * s.a4);
        t.A[g] += X * (-2.0 * Pv * s.H * s.L1 - dcv[g] * s.L1);
        t.H[g] += X * (-2.0 * Pv * s.A * s.L1);
        t.L1[g] += X * (-2.0 * Pv * s.A * s.H - dcv[g] * s.A);
      }
      t.a2[g] += X * (-6.0 * Pv - dcv[g]);
      t.Gc[g] += X * (-2.0 * Pv * s.a4);
      t.a4[g] += X * (-2.0 * Pv * s.Gc - dcv[g]);
      t.f[g] += -X * dcv[g];
    } else {
      const double sg = first ? 1.0 : -1.0;
      t.a2[g] += sg * X * dcv[g];
      t.a4[g] += sg * X * dcv[g];
      t.f[g] += sg * X * dcv[g];
      t.A[g] -= X * dcv[g] * s.L1;
      t.L1[g] -= X * dcv[g] * s.A;
    }
    t.D[g] += Pb * two_h;
  }
  return resid;
}

// Reverse of get_coefs / get_a1matvec (mod_nodal.f90:447-479, 630-698) and
// the interior branch of nodal_coup_upd (:322-337) for the face between
// bn (n) and b (p).
template <int NG>
__device__ __forceinline__ double iface_adj(const NadjParams& Q, const double* phi, int u, int bn, int b,
                                           SideBar<NG>& nb, SideBar<NG>& pb) {
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const int sf = 2 * u;
  const double two_hn = 2.0 / hdir(G, u, bn), two_hp = 2.0 / hdir(G, u, b);
  double R[2 * NG][2 * NG], x[2 * NG];
  Side sn[NG], sp[NG];
  double dcn[NG], dcp[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    sn[g] = side_at(P, phi, u, g, bn);
    sp[g] = side_at(P, phi, u, g, b);
    const double Pn = sn[g].D * two_hn, Pp = sp[g].D * two_hp;
    dcn[g] = P.dc[((size_t)g * 6 + sf) * NB + bn];
    dcp[g] = P.dc[((size_t)g * 6 + sf + 1) * NB + b];
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) {
      const double Bn = bc_at(P, u, g, hh, bn), Bp = bc_at(P, u, g, hh, b);
      const double dl = (hh == g) ? 1.0 : 0.0;
      R[g][hh] = -Pn * (Bn * sn[g].F + dl);
      R[g][hh + NG] = Pp * (Bp * sp[g].F + dl);
      R[g + NG][hh] = dcn[g] * (Bn * sn[g].A + dl);
      R[g + NG][hh + NG] = dcp[g] * (Bp * sp[g].A + dl);
    }
    const Side &a = sn[g], &c = sp[g];
    x[g] = Pn * (3.0 * a.a2 + a.Gc * a.a4 + a.F * a.L1) + Pp * (3.0 * c.a2 + c.Gc * c.a4 - c.F * c.L1);
    x[g + NG] = dcp[g] * (c.a2 + c.a4 + c.f - a.A * a.L1) - dcn[g] * (a.a2 + a.a4 + a.f + c.A * c.L1);
  }
  double inv[2 * NG];
  lu_factor<2 * NG>(R, inv);
  double s[2 * NG];
#pragma unroll
  for (int i = 0; i < 2 * NG; ++i) s[i] = x[i];
  lu_apply<2 * NG>(R, inv, s);
  double sb[2 * NG];
#pragma unroll
  for (int i = 0; i < 2 * NG; ++i) sb[i] = 0.0;
  double resid = 0.0;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const Side& a = sn[g];
    const double fp = sp[g].f;
    double Bf = 0.0;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) Bf = Bf + bc_at(P, u, g, hh, bn) * s[hh];
    const double a3 = a.A * (Bf + a.L1);
    const double T = s[g] + 3.0 * a.a2 + a.H * a3 + a.Gc * a.a4;
    const double jp = -a.D * two_hn * T;
    const size_t on = ((size_t)g * 6 + sf) * NB + bn;        // n's slot of the face
    const size_t slot = ((size_t)g * 6 + sf + 1) * NB + b;   // canonical slot
    const double df = P.df[on];
    const double sig = a.f + fp;
    const double dnew = (df * (a.f - fp) - jp) / sig;
    resid = fmax(resid, fabs(dnew - P.dn[slot]));
    const double lam = Q.lam[slot];
    const double numb = lam / sig, sigb = -lam * dnew / sig;
    Q.dfbar[slot] = numb * (a.f - fp);
    nb.f[g] += numb * df + sigb;
    pb.f[g] += -numb * df + sigb;
    const double Jb = -numb;
    const double Tb = Jb * (-a.D * two_hn);
    nb.D[g] += Jb * (-two_hn * T);
    sb[g] += Tb;
    nb.a2[g] += 3.0 * Tb;
    nb.H[g] += Tb * a3;
    const double a3b = Tb * a.H;
    nb.Gc[g] += Tb * a.a4;
    nb.a4[g] += Tb * a.Gc;
    nb.A[g] += a3b * (Bf + a.L1);
    const double q = a3b * a.A;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) {
      nb.Bc[g][hh] += q * s[hh];
      sb[hh] += q * bc_at(P, u, g, hh, bn);
    }
    nb.L1[g] += q;
  }
  // s = R^{-1} x
  double xb[2 * NG];
#pragma unroll
  for (int i = 0; i < 2 * NG; ++i) xb[i] = sb[i];
  lu_apply_T<2 * NG>(R, inv, xb);
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const Side &a = sn[g], &c = sp[g];
    const double Pn = a.D * two_hn, Pp = c.D * two_hp;
    double Pnb = 0.0, Ppb = 0.0;
#pragma unroll
    for (int hh = 0; hh < NG; ++hh) {
      const double Bn = bc_at(P, u, g, hh, bn), Bp = bc_at(P, u, g, hh, b);
      const double dl = (hh == g) ? 1.0 : 0.0;
      const double r11 = -xb[g] * s[hh], r12 = -xb[g] * s[hh + NG];
      const double r21 = -xb[g + NG] * s[hh], r22 = -xb[g + NG] * s[hh + NG];
      nb.Bc[g][hh] += r11 * (-Pn * a.F) + r21 * dcn[g] * a.A;
      nb.F[g] += r11 * (-Pn * Bn);
      Pnb += r11 * (-(Bn * a.F + dl));
      pb.Bc[g][hh] += r12 * Pp * c.F + r22 * dcp[g] * c.A;
      pb.F[g] += r12 * Pp * Bp;
      Ppb += r12 * (Bp * c.F + dl);
      nb.A[g] += r21 * dcn[g] * Bn;
      pb.A[g] += r22 * dcp[g] * Bp;
    }
    const double X = xb[g], Y = xb[g + NG];
    Pnb += X * (3.0 * a.a2 + a.Gc * a.a4 + a.F * a.L1);
    nb.a2[g] += 3.0 * X * Pn;
    nb.Gc[g] += X * Pn * a.a4;
    nb.a4[g] += X * Pn * a.Gc;
    nb.F[g] += X * Pn * a.L1;
    nb.L1[g] += X * Pn * a.F;
    Ppb += X * (3.0 * c.a2 + c.Gc * c.a4 - c.F * c.L1);
    pb.a2[g] += 3.0 * X * Pp;
    pb.Gc[g] += X * Pp * c.a4;
    pb.a4[g] += X * Pp * c.Gc;
    pb.F[g] -= X * Pp * c.L1;
    pb.L1[g] -= X * Pp * c.F;
    // the ADF pairing of mod_nodal.f90:693-694 as written there
    pb.a2[g] += Y * dcp[g];
    pb.a4[g] += Y * dcp[g];
    pb.f[g] += Y * dcp[g];
    nb.A[g] -= Y * dcp[g] * a.L1;
    nb.L1[g] -= Y * dcp[g] * a.A;
    nb.a2[g] -= Y * dcn[g];
    nb.a4[g] -= Y * dcn[g];
    nb.f[g] -= Y * dcn[g];
    pb.A[g] -= Y * dcn[g] * c.L1;
    pb.L1[g] -= Y * dcn[g] * c.A;
    nb.D[g] += Pnb * two_hn;
    pb.D[g] += Ppb * two_hp;
  }
  return resid;
}

template <int NG>
__global__ void __launch_bounds__(128) k_nadj_iface(NadjParams Q) {
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const double* phi = latest_phi(P);
  const int total = P.nnod * 3;
  double resid = 0.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % P.nnod, u = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    const LinePos L = line_pos(G, u, b);
    SideBar<NG> pb;
    pb.zero();
    if (!L.first) {
      const int bn = b - L.offp;
      SideBar<NG> nb;
      nb.zero();
      resid = fmax(resid, iface_adj<NG>(Q, phi, u, bn, b, nb, pb));
      side_store<NG>(Q.side, NB, 1, u, bn, nb);
    } else {
      resid = fmax(resid, bface_adj<NG>(Q, phi, u, b, true, pb));
    }
    side_store<NG>(Q.side, NB, 0, u, b, pb);
    if (L.last) {
      SideBar<NG> nb;
      nb.zero();
      resid = fmax(resid, bface_adj<NG>(Q, phi, u, b, false, nb));
      side_store<NG>(Q.side, NB, 1, u, b, nb);
    }
  }
  double acc[1] = {resid};
  block_partials<1, 1u>(acc, Q.rpart);
}

// ---------------------------------------------------------------------------
// Stage 2: per node and direction, the reverse of k_node_prep (get_B,
// get_ABEFGH, get_a2matvec, LU_solve, get_a4, TLUpd1, TLUpd2).
// Writes, in slots [u][q][b] of Q.nodeu (q below), the adjoints of the node's
// flux, D, sigr, nuf and sigs, and of the zeroth-order source S_u: its own
// (Sself) and what it owes the plus (toP) and minus (toM) neighbours.
// ---------------------------------------------------------------------------
template <int NG>
struct NodeQ {
  static constexpr int phi = 0, D = NG, sigr = 2 * NG, nuf = 3 * NG, sigs = 4 * NG;
  static constexpr int sself = 4 * NG + NG * NG, toP = 5 * NG + NG * NG, toM = 6 * NG + NG * NG;
  static constexpr int nq = 7 * NG + NG * NG;
};

__device__ __forceinline__ size_t nodeu_ix(int nq, int NB, int u, int q, int b) {
  return ((size_t)u * nq + q) * NB + b;
}

template <int NG>
__global__ void __launch_bounds__(128) k_nadj_node(NadjParams Q) {
  using NQ = NodeQ<NG>;
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const double* phi = latest_phi(P);
  const double Ke = *(const volatile double*)&P.ctl->Ke;
  const double invKe = 1.0 / Ke;
  const int total = P.nnod * 3;
  double kacc = 0.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % P.nnod, u = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    SideBar<NG> t;
    t.zero();
    side_add<NG>(Q.side, NB, 0, u, b, t);
    side_add<NG>(Q.side, NB, 1, u, b, t);
    const double h = hdir(G, u, b);
    double fac[NG], Dv[NG], sig[NG], Ek[NG], Bk[NG], Sn[NG], dSp[NG], dSm[NG], Lm2[NG], f[NG], a2[NG];
    double Bc[NG][NG], M[NG][NG];
    const TLGeom T = tl_geom(G, u, b);
    const double* S = P.S + (size_t)u * NG * NB;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      Dv[g] = P.D[(size_t)g * NB + b];
      sig[g] = P.sigr[(size_t)g * NB + b];
      fac[g] = 0.25 * (h * h) / Dv[g];
      Ek[g] = nconst(P, u, 2, g, b);
      Bk[g] = nconst(P, u, 1, g, b);
      Sn[g] = S[(size_t)g * NB + b];
      dSp[g] = T.has_p ? S[(size_t)g * NB + b + T.offp] - Sn[g] : 0.0;
      dSm[g] = T.has_m ? S[(size_t)g * NB + b - T.offp] - Sn[g] : 0.0;
      Lm2[g] = fac[g] * (T.c2p * dSp[g] + T.c2m * dSm[g]);
      f[g] = phi[(size_t)g * P.NBH + b];
      a2[g] = P.a2[((size_t)u * NG + g) * NB + b];
    }
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) {
        Bc[g][hh] = bc_at(P, u, g, hh, b);
        M[g][hh] = (hh == g) ? Bc[g][hh] * Ek[g] + 3.0 : Bc[g][hh] * Ek[g];
      }
    double Bcb[NG][NG], a2b[NG], Lm2b[NG], Bkb[NG], Ekb[NG], facb[NG], fb[NG], Sself[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      a2b[g] = t.a2[g];
      Lm2b[g] = 0.0;
      Ekb[g] = 0.0;
      facb[g] = 0.0;
      fb[g] = t.f[g];
      Sself[g] = 0.0;
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) Bcb[g][hh] = t.Bc[g][hh];
    }
    // a4 = B (Bc a2 + Lm2)
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      double Bf = 0.0;
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) Bf = Bf + Bc[g][hh] * a2[hh];
      Bkb[g] = t.a4[g] * (Bf + Lm2[g]);
      const double tt = t.a4[g] * Bk[g];
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) {
        Bcb[g][hh] += tt * a2[hh];
        a2b[hh] += tt * Bc[g][hh];
      }
      Lm2b[g] += tt;
    }
    // a2 = M^{-1} rhs
    double inv[NG];
    lu_factor<NG>(M, inv);
    double rb[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) rb[g] = a2b[g];
    lu_apply_T<NG>(M, inv, rb);
#pragma unroll
    for (int g = 0; g < NG; ++g) {
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) {
        const double Mb = -rb[g] * a2[hh];
        Bcb[g][hh] += Mb * Ek[g] + rb[g] * f[hh];
        Ekb[g] += Mb * Bc[g][hh];
        fb[hh] += rb[g] * Bc[g][hh];
      }
      // rhs = Bc f - E Lm2 + fac S
      Ekb[g] -= rb[g] * Lm2[g];
      Lm2b[g] -= rb[g] * Ek[g];
      facb[g] += rb[g] * Sn[g];
      Sself[g] += rb[g] * fac[g];
    }
    // Lm2 = fac (c2p dSp + c2m dSm), L1 = fac (c1p dSp - c1m dSm)
    double toP[NG], toM[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const double L1b = t.L1[g];
      facb[g] += Lm2b[g] * (T.c2p * dSp[g] + T.c2m * dSm[g]) + L1b * (T.c1p * dSp[g] - T.c1m * dSm[g]);
      const double dSpb = fac[g] * (Lm2b[g] * T.c2p + L1b * T.c1p);
      const double dSmb = fac[g] * (Lm2b[g] * T.c2m - L1b * T.c1m);
      toP[g] = T.has_p ? dSpb : 0.0;
      toM[g] = T.has_m ? dSmb : 0.0;
      Sself[g] -= toP[g] + toM[g];
    }
    // Bc = fac * dum (get_B, cmode 1)
    double sigrb[NG], nufb[NG], sigsb[NG][NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      sigrb[g] = 0.0;
      nufb[g] = 0.0;
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) sigsb[g][hh] = 0.0;
    }
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const double chi = P.chin[(size_t)g * NB + b];
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) {
        const double nuf = P.nuf[(size_t)hh * NB + b];
        const double dum = (hh == g) ? sig[g] - chi * nuf * invKe
                                     : -P.sigs[((size_t)hh * NG + g) * NB + b] - chi * nuf * invKe;
        facb[g] += Bcb[g][hh] * dum;
        const double db = Bcb[g][hh] * fac[g];
        if (hh == g) sigrb[g] += db;
        else sigsb[hh][g] -= db;               // sigs(h -> g), stored [from][to]
        nufb[hh] -= db * chi * invKe;
        kacc += db * chi * nuf * invKe * invKe;
      }
    }
    double Db[NG];
#pragma unroll
    for (int g = 0; g < NG; ++g) Db[g] = t.D[g] - facb[g] * fac[g] / Dv[g];
    if (!P.pnm) {
      // constants of get_ABEFGH through alpha = sqrt(sigr / D) h / 2
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const double alp = 0.5 * sqrt(sig[g] / Dv[g]) * h;
        double dc[6];
        sanm_dconsts(alp, dc);
        const double ab = t.A[g] * dc[0] + Bkb[g] * dc[1] + Ekb[g] * dc[2] + t.F[g] * dc[3] + t.Gc[g] * dc[4] +
                          t.H[g] * dc[5];
        sigrb[g] += ab * alp / (2.0 * sig[g]);
        Db[g] -= ab * alp / (2.0 * Dv[g]);
      }
    }
    double* o = Q.nodeu;
    constexpr int nq = NQ::nq;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      o[nodeu_ix(nq, NB, u, NQ::phi + g, b)] = fb[g];
      o[nodeu_ix(nq, NB, u, NQ::D + g, b)] = Db[g];
      o[nodeu_ix(nq, NB, u, NQ::sigr + g, b)] = sigrb[g];
      o[nodeu_ix(nq, NB, u, NQ::nuf + g, b)] = nufb[g];
      o[nodeu_ix(nq, NB, u, NQ::sself + g, b)] = Sself[g];
      o[nodeu_ix(nq, NB, u, NQ::toP + g, b)] = toP[g];
      o[nodeu_ix(nq, NB, u, NQ::toM + g, b)] = toM[g];
#pragma unroll
      for (int hh = 0; hh < NG; ++hh) o[nodeu_ix(nq, NB, u, NQ::sigs + g * NG + hh, b)] = sigsb[g][hh];
    }
  }
  double acc[1] = {kacc};
  block_partials<1, 0u>(acc, Q.kpart);
}

// ---------------------------------------------------------------------------
// Stage 3: S_u adjoints gathered per node, then the leakages of get_source
// (S1 = L2 + L3, S2 = L1 + L3, S3 = L1 + L2).
// ---------------------------------------------------------------------------
__global__ void k_nadj_lbar(NadjParams Q, int nq, int q_sself, int q_top, int q_tom) {
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  const int total = P.nnod * ng;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % P.nnod, g = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    const unsigned m = G.nbm[b];
    double Sb[3];
    for (int u = 0; u < 3; ++u) {
      const int off = face_off(G, 2 * u);
      double v = Q.nodeu[nodeu_ix(nq, NB, u, q_sself + g, b)];
      if (m & (1u << (2 * u + 1))) v += Q.nodeu[nodeu_ix(nq, NB, u, q_top + g, b - off)];
      if (m & (1u << (2 * u))) v += Q.nodeu[nodeu_ix(nq, NB, u, q_tom + g, b + off)];
      Sb[u] = v;
    }
    Q.Lbar[((size_t)0 * ng + g) * NB + b] = Sb[1] + Sb[2];
    Q.Lbar[((size_t)1 * ng + g) * NB + b] = Sb[0] + Sb[2];
    Q.Lbar[((size_t)2 * ng + g) * NB + b] = Sb[0] + Sb[1];
  }
}

// ---------------------------------------------------------------------------
// Stage 4: Lxyz backwards.  A face current J enters the leakage of both
// nodes of an interior face; its adjoint is formed by each node from the two
// leakage adjoints, and the node adds J's flux derivatives to its own flux
// adjoint.  The node owning the face's canonical slot also writes the
// adjoint of the face's d and adds that of df.
// ---------------------------------------------------------------------------
__global__ void k_nadj_leak(NadjParams Q, int nq, int q_phi) {
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  const double* phi = latest_phi(P);
  const int total = P.nnod * ng;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % P.nnod, g = q / P.nnod;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    const unsigned m = G.nbm[b];
    const double* F = phi + (size_t)g * P.NBH;
    const double fb0 = F[b];
    double pb = 0.0;
    for (int u = 0; u < 3; ++u) pb += Q.nodeu[nodeu_ix(nq, NB, u, q_phi + g, b)];
    for (int u = 0; u < 3; ++u) {
      const double hb = hdir(G, u, b);
      const double Lb = Q.Lbar[((size_t)u * ng + g) * NB + b];
      const int fp = 2 * u, fm = 2 * u + 1;
      const int off = face_off(G, fp);
      const size_t sp = ((size_t)g * 6 + fp) * NB + b, sm = ((size_t)g * 6 + fm) * NB + b;
      // plus face
      if (m & (1u << fp)) {
        const int bm = b + off;
        const double Jb = Lb / hb - Q.Lbar[((size_t)u * ng + g) * NB + bm] / hdir(G, u, bm);
        pb += Jb * (P.df[sp] - P.dn[sp]);
      } else {
        double dnb = 0.0;
        if (G.bcf[fp] != 2) {
          const double Jb = Lb / hb;
          pb += Jb * (P.df[sp] - P.dn[sp]);
          dnb = -Jb * fb0;
          Q.dfbar[sp] += Jb * fb0;
        }
        Q.dnbar[sp] = dnb;
      }
      // minus face (canonical slot of this node)
      double dnb = 0.0;
      if (m & (1u << fm)) {
        const int bm = b - off;
        const double fmv = F[bm];
        const double Jb = -Lb / hb + Q.Lbar[((size_t)u * ng + g) * NB + bm] / hdir(G, u, bm);
        pb += Jb * (-P.df[sm] - P.dn[sm]);
        dnb = -Jb * (fb0 + fmv);
        Q.dfbar[sm] += -Jb * (fb0 - fmv);
      } else if (G.bcf[fm] != 2) {
        const double Jb = -Lb / hb;
        pb += Jb * (-P.df[sm] - P.dn[sm]);
        dnb = -Jb * fb0;
        Q.dfbar[sm] += -Jb * fb0;
      }
      Q.dnbar[sm] = dnb;
    }
    Q.phibar[(size_t)g * NB + b] = pb;
  }
}

// ---------------------------------------------------------------------------
// Stage 5: cross-section adjoints per node, in the layout of dkdp
// out[(c * ng + g) * nnod + n]: c = 0 D, 1 siga, 2 nuf, 3 sigtr, 4 + h sigs(g -> h).
// D collects the df of coup_coef (mod_cmfd.f90:11-137) of the node's six
// faces; siga and sigs(g -> h) enter through sigr = siga + sum sigs.
// Block 0 also reduces N_k^T lam and the fixed-point residual.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ddf_dDn(bool interior, int bc, double Dn, double Dm, double hn, double hm) {
  if (interior) {
    const double den = Dn * hm + Dm * hn;
    return 2.0 * Dm * Dm * hn / (den * den);
  }
  if (bc == 0) {
    const double alb = 1.e30, den = 2.0 * Dn + alb * hn;
    return 2.0 * alb * alb * hn / (den * den);
  }
  if (bc == 1) {
    const double den = 2.0 * Dn + 0.5 * hn;
    return 0.5 * hn / (den * den);
  }
  return 0.0;
}

__global__ void k_nadj_params(NadjParams Q, int nq, int q_D, int q_sigr, int q_nuf, int q_sigs, int kblk,
                              int rblk) {
  const NodalParams& P = Q.N;
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng, nn = P.nnod;
  if (blockIdx.x == 0) {
    double tk[1], tr[1];
    grid_totals<1, 0u>(Q.kpart, kblk, tk);
    grid_totals<1, 1u>(Q.rpart, rblk, tr);
    if (threadIdx.x == 0) {
      Q.scal[0] = tk[0];
      Q.scal[1] = tr[0];
    }
  }
  const int total = nn * ng;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % nn, g = q / nn;
    const int b = P.act[n];
    if (!node_ok(P.ctl, G, b)) continue;
    const unsigned m = G.nbm[b];
    const double Dn = P.D[(size_t)g * NB + b];
    double Db = 0.0, sr = 0.0, nf = 0.0;
    for (int u = 0; u < 3; ++u) {
      Db += Q.nodeu[nodeu_ix(nq, NB, u, q_D + g, b)];
      sr += Q.nodeu[nodeu_ix(nq, NB, u, q_sigr + g, b)];
      nf += Q.nodeu[nodeu_ix(nq, NB, u, q_nuf + g, b)];
    }
    for (int f = 0; f < 6; ++f) {
      const int u = f >> 1;
      const double hn = hdir(G, u, b);
      if (m & (1u << f)) {
        const int bm = b + face_off(G, f);
        const int owner = (f & 1) ? b : bm;                 // canonical slot: the minus face of the p node
        const double dfb = Q.dfbar[((size_t)g * 6 + (2 * u + 1)) * NB + owner];
        Db += dfb * ddf_dDn(true, 0, Dn, P.D[(size_t)g * NB + bm], hn, hdir(G, u, bm));
      } else {
        const double dfb = Q.dfbar[((size_t)g * 6 + f) * NB + b];
        Db += dfb * ddf_dDn(false, G.bcf[f], Dn, 0.0, hn, 0.0);
      }
    }
    double* out = Q.out;
    out[((size_t)0 * ng + g) * nn + n] = Db;
    out[((size_t)1 * ng + g) * nn + n] = sr;
    out[((size_t)2 * ng + g) * nn + n] = nf;
    out[((size_t)3 * ng + g) * nn + n] = -3.0 * Dn * Dn * Db;
    for (int h = 0; h < ng; ++h) {
      double v = 0.0;
      if (h != g) {
        v = sr;   // sigs(g -> h) is part of sigr of group g
        for (int u = 0; u < 3; ++u) v += Q.nodeu[nodeu_ix(nq, NB, u, q_sigs + g * ng + h, b)];
      }
      out[((size_t)(4 + h) * ng + g) * nn + n] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// w^T (dM/dd_f) phi per canonical face slot (matrix_setup, mod_cmfd.f90:
// 245-298): an interior face between n and p enters row n with
// -(phi_n + phi_p)/h_n and row p with (phi_n + phi_p)/h_p; a boundary face
// only its own row's diagonal, +phi/h on a minus face and -phi/h on a plus
// face.  out = scale * that.
// ---------------------------------------------------------------------------
__global__ void k_face_contract(BoxGeom G, int ng, int nnod, long long NBH, const int* act, const double* phi,
                                const double* w, double scale, double* out) {
  const int NB = G.NB;
  const int total = nnod * ng;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % nnod, g = q / nnod;
    const int b = act[n];
    const unsigned m = G.nbm[b];
    const double* F = phi + (size_t)g * NBH;
    const double* W = w + (size_t)g * NBH;
    for (int u = 0; u < 3; ++u) {
      const int fp = 2 * u, fm = 2 * u + 1;
      const double hb = hdir(G, u, b);
      double c;
      if (m & (1u << fm)) {
        const int bm = b + face_off(G, fm);
        c = (F[b] + F[bm]) * (W[b] / hb - W[bm] / hdir(G, u, bm));
      } else {
        c = W[b] * F[b] / hb;
      }
      out[((size_t)g * 6 + fm) * NB + b] = scale * c;
      if (!(m & (1u << fp))) out[((size_t)g * 6 + fp) * NB + b] = -scale * W[b] * F[b] / hb;
    }
  }
}

// lam_new = Kd (1 + s) + dnbar - cG at the canonical slots; partials of
// |lam_new - lam|^2 and |lam_new|^2.
__global__ void k_lam_update(BoxGeom G, int ng, int nnod, const int* act, const double* Kd, const double* dnbar,
                             const double* cG, const double* scal, double* lam, double* dlam, double* part) {
  const int NB = G.NB;
  const double s1 = 1.0 + scal[0];
  double acc[2] = {0.0, 0.0};
  const int total = nnod * ng;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % nnod, g = q / nnod;
    const int b = act[n];
    const unsigned m = G.nbm[b];
    for (int f = 0; f < 6; ++f) {
      const bool canon = (f & 1) || !(m & (1u << f));
      if (!canon) continue;
      const size_t i = ((size_t)g * 6 + f) * NB + b;
      const double v = Kd[i] * s1 + dnbar[i] - cG[i];
      const double d = v - lam[i];
      acc[0] = fma(d, d, acc[0]);
      acc[1] = fma(v, v, acc[1]);
      lam[i] = v;
      dlam[i] = d;
    }
  }
  block_partials<2, 0u>(acc, part);
}

// lam += c dlam at the canonical slots: the extrapolation of a linearly
// converging iteration by its observed contraction d, c = d / (1 - d), as
// fiss_extrp does for the fission source (mod_cmfd.f90:308-335).
__global__ void k_lam_extrap(BoxGeom G, int ng, int nnod, const int* act, const double* dlam, double c, double* lam) {
  const int NB = G.NB;
  const int total = nnod * ng;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int n = q % nnod, g = q / nnod;
    const int b = act[n];
    const unsigned m = G.nbm[b];
    for (int f = 0; f < 6; ++f) {
      if (!((f & 1) || !(m & (1u << f)))) continue;
      const size_t i = ((size_t)g * 6 + f) * NB + b;
      lam[i] = fma(c, dlam[i], lam[i]);
    }
  }
}

// Partials of (phi . v) and (phi . phi) over the active rows, v = phibar.
__global__ void k_gpt_dots(BoxGeom G, int ng, int nnod, long long NBH, const int* act, const double* phi,
                           const double* v, double* part) {
  const int NB = G.NB;
  double acc[2] = {0.0, 0.0};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnod; n += gridDim.x * blockDim.x) {
    const int b = act[n];
    for (int g = 0; g < ng; ++g) {
      const double f = phi[(size_t)g * NBH + b];
      acc[0] = fma(f, v[(size_t)g * NB + b], acc[0]);
      acc[1] = fma(f, f, acc[1]);
    }
  }
  block_partials<2, 0u>(acc, part);
}

// The GPT source: v minus its component along phi (the solvability
// condition phi^T v = 0 of the singular system, exact up to rounding since
// N is homogeneous of degree 0 in phi).
__global__ void k_gpt_source(BoxGeom G, int ng, int nnod, long long NBH, const int* act, const double* phi,
                             const double* v, const double* part, int nblk, double* src) {
  double tot[2];
  grid_totals<2, 0u>(part, nblk, tot);
  const double a = tot[1] > 0.0 ? tot[0] / tot[1] : 0.0;
  const int NB = G.NB;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnod; n += gridDim.x * blockDim.x) {
    const int b = act[n];
    for (int g = 0; g < ng; ++g) src[(size_t)g * NB + b] = v[(size_t)g * NB + b] - a * phi[(size_t)g * NBH + b];
  }
}

// Partials of Gam^T F phi = sum_b (sum_g chi_g Gam_g)(sum_h nuf_h phi_h) and
// of psi^T F phi.
__global__ void k_gpt_fdots(BoxGeom G, int ng, int nnod, long long NBH, const int* act, const double* chin,
                            const double* nuf, const double* phi, const double* gam, const double* psi,
                            double* part) {
  const int NB = G.NB;
  double acc[2] = {0.0, 0.0};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnod; n += gridDim.x * blockDim.x) {
    const int b = act[n];
    double ff = 0.0, fg = 0.0, fp = 0.0;
    for (int g = 0; g < ng; ++g) {
      const double c = chin[(size_t)g * NB + b];
      ff = fma(nuf[(size_t)g * NB + b], phi[(size_t)g * NBH + b], ff);
      fg = fma(c, gam[(size_t)g * NBH + b], fg);
      fp = fma(c, psi[(size_t)g * NBH + b], fp);
    }
    acc[0] = fma(fg, ff, acc[0]);
    acc[1] = fma(fp, ff, acc[1]);
  }
  block_partials<2, 0u>(acc, part);
}

// Gam -= c psi and fs_Gam -= c (sum_g chi_g psi_g), c = Gam^T F phi / psi^T F phi:
// the component along the fundamental adjoint mode, which the source
// iteration leaves undamped.
__global__ void k_gpt_project(BoxGeom G, int ng, int nnod, long long NBH, const int* act, const double* chin,
                              const double* psi, const double* part, int nblk, double* gam, double* fsg) {
  double tot[2];
  grid_totals<2, 0u>(part, nblk, tot);
  const double c = tot[1] != 0.0 ? tot[0] / tot[1] : 0.0;
  const int NB = G.NB;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnod; n += gridDim.x * blockDim.x) {
    const int b = act[n];
    double fp = 0.0;
    for (int g = 0; g < ng; ++g) {
      const double p = psi[(size_t)g * NBH + b];
      fp = fma(chin[(size_t)g * NB + b], p, fp);
      gam[(size_t)g * NBH + b] -= c * p;
    }
    fsg[b] -= c * fp;
  }
}

// nuf / k: the adjoint fission weight of the GPT source iteration, which
// runs in the fixed-eigenvalue (no k update) mode of the outer kernel.
__global__ void k_scale_planes(const double* in, double s, double* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = in[i] * s;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int blocks_for(long long items, int threads, int cap) {
  long long b = (items + threads - 1) / threads;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

template <int NG>
static cudaError_t nadj_ng(const NadjParams& Q, cudaStream_t st) {
  using NQ = NodeQ<NG>;
  const int total = Q.N.nnod * 3;
  const int b1 = blocks_for(total, 128, kMaxBlocks);
  k_nadj_iface<NG><<<b1, 128, 0, st>>>(Q);
  const int b2 = blocks_for(total, 128, kMaxBlocks);
  k_nadj_node<NG><<<b2, 128, 0, st>>>(Q);
  const int b3 = blocks_for((long long)Q.N.nnod * NG, 256, 8192);
  k_nadj_lbar<<<b3, 256, 0, st>>>(Q, NQ::nq, NQ::sself, NQ::toP, NQ::toM);
  k_nadj_leak<<<b3, 256, 0, st>>>(Q, NQ::nq, NQ::phi);
  k_nadj_params<<<b3, 256, 0, st>>>(Q, NQ::nq, NQ::D, NQ::sigr, NQ::nuf, NQ::sigs, b2, b1);
  return cudaGetLastError();
}

size_t nadj_side_doubles(int ng, long long NB) { return (size_t)2 * 3 * (9 * ng + ng * ng) * NB; }
size_t nadj_nodeu_doubles(int ng, long long NB) { return (size_t)3 * (7 * ng + ng * ng) * NB; }

cudaError_t launch_nodal_adjoint(const NadjParams& Q, cudaStream_t st) {
  switch (Q.N.ng) {
    case 1: return nadj_ng<1>(Q, st);
    case 2: return nadj_ng<2>(Q, st);
    case 3: return nadj_ng<3>(Q, st);
    case 4: return nadj_ng<4>(Q, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_face_contract(const BoxGeom& G, int ng, int nnod, long long NBH, const int* act,
                                 const double* phi, const double* w, double scale, double* out, cudaStream_t st) {
  k_face_contract<<<blocks_for((long long)nnod * ng, 256, 8192), 256, 0, st>>>(G, ng, nnod, NBH, act, phi, w, scale,
                                                                             out);
  return cudaGetLastError();
}

cudaError_t launch_lam_update(const BoxGeom& G, int ng, int nnod, const int* act, const double* Kd,
                              const double* dnbar, const double* cG, const double* scal, double* lam, double* dlam,
                              double* part, cudaStream_t st) {
  k_lam_update<<<blocks_for((long long)nnod * ng, 256, kMaxBlocks), 256, 0, st>>>(G, ng, nnod, act, Kd, dnbar, cG,
                                                                                  scal, lam, dlam, part);
  return cudaGetLastError();
}

cudaError_t launch_lam_extrap(const BoxGeom& G, int ng, int nnod, const int* act, const double* dlam, double c,
                              double* lam, cudaStream_t st) {
  k_lam_extrap<<<blocks_for((long long)nnod * ng, 256, 8192), 256, 0, st>>>(G, ng, nnod, act, dlam, c, lam);
  return cudaGetLastError();
}

int lam_update_blocks(int ng, int nnod) { return blocks_for((long long)nnod * ng, 256, kMaxBlocks); }

cudaError_t launch_gpt_source(const BoxGeom& G, int ng, int nnod, long long NBH, const int* act, const double* phi,
                              const double* v, double* part, double* src, cudaStream_t st) {
  const int nb = blocks_for(nnod, 256, kMaxBlocks);
  k_gpt_dots<<<nb, 256, 0, st>>>(G, ng, nnod, NBH, act, phi, v, part);
  k_gpt_source<<<nb, 256, 0, st>>>(G, ng, nnod, NBH, act, phi, v, part, nb, src);
  return cudaGetLastError();
}

cudaError_t launch_gpt_project(const BoxGeom& G, int ng, int nnod, long long NBH, const int* act,
                               const double* chin, const double* nuf, const double* phi, const double* psi,
                               double* part, double* gam, double* fsg, cudaStream_t st) {
  const int nb = blocks_for(nnod, 256, kMaxBlocks);
  k_gpt_fdots<<<nb, 256, 0, st>>>(G, ng, nnod, NBH, act, chin, nuf, phi, gam, psi, part);
  k_gpt_project<<<nb, 256, 0, st>>>(G, ng, nnod, NBH, act, chin, psi, part, nb, gam, fsg);
  return cudaGetLastError();
}

cudaError_t launch_scale_planes(const double* in, double s, double* out, long long n, cudaStream_t st) {
  k_scale_planes<<<blocks_for(n, 256, 8192), 256, 0, st>>>(in, s, out, n);
  return cudaGetLastError();
}

}  // namespace adp
