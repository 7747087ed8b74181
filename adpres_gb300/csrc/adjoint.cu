// Discrete adjoint of the converged forward CMFD eigenproblem and the
// sensitivity of k to every node's cross sections.
//
// With the nodal coupling coefficients dn frozen at the converged forward
// state, the CMFD equations (matrix_setup + TSrc, mod_cmfd.f90:217-304,
// :1006-1033) are the generalized eigenproblem
//     M phi = (1/k) F phi,
//     (M phi)_g = A_g phi_g - sum_{h/=g} sigs(h->g) phi_h,
//     (F phi)_g = chi_g sum_h nuf_h phi_h.
// Its discrete adjoint M^T psi = (1/k) F^T psi has the source structure of
// outer_ad / TSrcAd (mod_cmfd.f90:602-699, :1037-1064) with the transposed
// stencil A_g^T, so it is solved by the same persistent kernel given A^T.
// Then, for a parameter p of node n,
//     dk/dp = k^2 psi^T (lambda dF/dp - dM/dp) phi / (psi^T F phi),  lambda = 1/k.
// The reference has no sensitivity edit; its closest relative is the
// adjoint-weighted reactivity of mod_trans.f90:648-688.
#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"

namespace adp {

// A^T in the same 7-slot layout: the coefficient of x[b + off_c] in row b of
// A^T is the coefficient of x[b] in row b + off_c of A, i.e. that row's
// opposite slot.
__global__ void k_transpose(BoxGeom G, int ng, const double* A, double* AT, float* AT32, float2* AT2) {
  const int NB = G.NB;
  const long long total = (long long)NB * ng;
  const int off[7] = {-G.plane, -G.nxx, -1, 0, 1, G.nxx, G.plane};
  const int face[7] = {FZM, FYM, FXM, -1, FXP, FYP, FZP};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(q / NB), b = (int)(q - (long long)g * NB);
    const unsigned m = G.nbm[b];
    const double* Ag = A + (size_t)g * 7 * NB;
    for (int c = 0; c < 7; ++c) {
      double v = 0.0;
      if (c == 3) v = Ag[(size_t)3 * NB + b];
      else if ((m & NB_ACTIVE) && (m & (1u << face[c]))) v = Ag[(size_t)(6 - c) * NB + b + off[c]];
      AT[(size_t)g * 7 * NB + (size_t)c * NB + b] = v;
      if (AT32) {
        const float hi = (float)v;
        AT32[(size_t)g * 7 * NB + (size_t)c * NB + b] = hi;
        if (AT2) AT2[(size_t)g * 7 * NB + (size_t)c * NB + b] = make_float2(hi, (float)(v - (double)hi));
      }
    }
  }
}

cudaError_t launch_transpose(const BoxGeom& G, int ng, const double* A, double* AT, float* AT32, float2* AT2,
                             cudaStream_t st) {
  long long total = (long long)G.NB * ng;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 65535 * 4) blocks = 65535 * 4;
  k_transpose<<<blocks, 256, 0, st>>>(G, ng, A, AT, AT32, AT2);
  return cudaGetLastError();
}

// psi^T F phi = sum_n (sum_g chi_g psi_g)(sum_h nuf_h phi_h), block partials.
__global__ void k_sens_den(SensParams P, double* part) {
  const BoxGeom& G = P.G;
  double acc[1] = {0.0};
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < G.NB; b += gridDim.x * blockDim.x) {
    double fa = 0.0, ff = 0.0;
    for (int g = 0; g < P.ng; ++g) {
      fa = fma(P.chin[(size_t)g * G.NB + b], P.psi[(size_t)g * P.NBH + b], fa);
      ff = fma(P.nuf[(size_t)g * G.NB + b], P.phi[(size_t)g * P.NBH + b], ff);
    }
    acc[0] = fma(fa, ff, acc[0]);
  }
  block_partials<1, 0u>(acc, part);
}

// dF of the harmonic-mean coupling coefficient of coup_coef
// (mod_cmfd.f90:54-55) with respect to the node's own D:
//   df = 2 Dn Dm / (Dn hm + Dm hn)  ->  d df / d Dn = 2 Dm^2 hn / (Dn hm + Dm hn)^2
// and of the boundary forms (:45-50): zero flux 2 alb^2 h / (2 Dn + alb h)^2,
// zero incoming current 0.5 h / (2 Dn + 0.5 h)^2, reflective 0.
__device__ __forceinline__ double ddf_dD(bool interior, int bc, double Dn, double Dm, double hn, double hm) {
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

// The contraction w^T (lambda dF/dp - dM/dp) phi of one node and group for
// every parameter p of the column layout of dkdp(nnod, ng, 4 + ng):
// c = 0 D, 1 siga, 2 nuf, 3 sigtr (through D = 1/(3 sigtr),
// dD/dsigtr = -3 D^2, mod_xsec.f90:199-226) and 4 + h the g -> h scattering
// (through sigr and the scattering source).  P.psi is the weight w.
__device__ __forceinline__ void sens_raw(const SensParams& P, int n, int g, double* v) {
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  const double lam = 1.0 / P.keff;
  const int b = P.act[n];
  const unsigned m = G.nbm[b];
  double fsa = 0.0;   // sum_g chi_g w_g at this node
  for (int h = 0; h < ng; ++h) fsa = fma(P.chin[(size_t)h * NB + b], P.psi[(size_t)h * P.NBH + b], fsa);
  const double ph = P.phi[(size_t)g * P.NBH + b], ps = P.psi[(size_t)g * P.NBH + b];
  const double Dn = P.D[(size_t)g * NB + b];
  // D: every face of the node; an interior face enters its own row and
  // the neighbour's row with the same (harmonic-mean) coefficient.
  double nD = 0.0;
  for (int f = 0; f < 6; ++f) {
    const int u = f >> 1;
    const double hn = hdir(G, u, b);
    if (m & (1u << f)) {
      const int bm = b + face_off(G, f);
      const double Dm = P.D[(size_t)g * NB + bm], hm = hdir(G, u, bm);
      const double phm = P.phi[(size_t)g * P.NBH + bm], psm = P.psi[(size_t)g * P.NBH + bm];
      const double d = ddf_dD(true, 0, Dn, Dm, hn, hm);
      nD += d * (ps * (ph - phm) / hn + psm * (phm - ph) / hm);
    } else {
      const double d = ddf_dD(false, G.bcf[f], Dn, 0.0, hn, 0.0);
      nD += d * ps * ph / hn;
    }
  }
  v[0] = -nD;
  v[1] = -ps * ph;          // siga (through sigr)
  v[2] = lam * fsa * ph;    // nuf of group g
  v[3] = -3.0 * Dn * Dn * v[0];
  for (int h = 0; h < ng; ++h) v[4 + h] = (h != g) ? -(ps - P.psi[(size_t)h * P.NBH + b]) * ph : 0.0;
}

// Per node and group: out[(c * ng + g) * nnod + n] =
// k^2 / (psi^T F phi) * psi^T (lambda dF/dp - dM/dp) phi, the derivative at
// frozen dn.
__global__ void k_sens(SensParams P, const double* part, int nblk, double* out) {
  double tot[1];
  grid_totals<1, 0u>(part, nblk, tot);
  const double den = tot[0];
  const int ng = P.ng, nn = P.nnod;
  const double k = P.keff, scale = k * k / den;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nn * ng; q += gridDim.x * blockDim.x) {
    const int n = q % nn, g = q / nn;
    double v[4 + kMaxGroups];
    sens_raw(P, n, g, v);
    for (int c = 0; c < 4 + ng; ++c) out[((size_t)c * ng + g) * nn + n] = scale * v[c];
  }
}

// The derivative through the nodal update: out = KS (1 + s) + NS +
// Gam^T (lambda dF/dp - dM/dp) phi, with KS the frozen-dn derivative, s =
// lam^T dN/dk (scal[0]), NS = lam^T dN/dp and P.psi = Gam.
__global__ void k_sens_total(SensParams P, const double* KS, const double* NS, const double* scal, double* out) {
  const int ng = P.ng, nn = P.nnod;
  const double s1 = 1.0 + scal[0];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nn * ng; q += gridDim.x * blockDim.x) {
    const int n = q % nn, g = q / nn;
    double v[4 + kMaxGroups];
    sens_raw(P, n, g, v);
    for (int c = 0; c < 4 + ng; ++c) {
      const size_t i = ((size_t)c * ng + g) * nn + n;
      out[i] = KS[i] * s1 + NS[i] + v[c];
    }
  }
}

cudaError_t launch_sens_total(const SensParams& P, const double* KS, const double* NS, const double* scal, double* out,
                              cudaStream_t st) {
  int b2 = (P.nnod * P.ng + 255) / 256;
  if (b2 > 4096) b2 = 4096;
  k_sens_total<<<b2, 256, 0, st>>>(P, KS, NS, scal, out);
  return cudaGetLastError();
}

cudaError_t launch_sens(const SensParams& P, double* part, double* out, cudaStream_t st) {
  int blocks = (P.G.NB + 255) / 256;
  if (blocks > kMaxBlocks) blocks = kMaxBlocks;
  k_sens_den<<<blocks, 256, 0, st>>>(P, part);
  int b2 = (P.nnod * P.ng + 255) / 256;
  if (b2 > 4096) b2 = 4096;
  k_sens<<<b2, 256, 0, st>>>(P, part, blocks, out);
  return cudaGetLastError();
}

}  // namespace adp
