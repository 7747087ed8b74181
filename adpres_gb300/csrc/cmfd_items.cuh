// Elementwise CMFD stages as per-item device functions, shared by the
// single-core kernels (cmfd.cu) and the batched kernel (batch.cu).
//   assemble_items  : matrix_setup (mod_cmfd.f90:217-304) with coup_coef
//                     (:11-137) when requested; one item per (node, group),
//                     inactive box positions get all-zero rows; row slots in
//                     reference column order [z-, y-, x-, diag, x+, y+, z+].
//   init_flux_items : first-call start f0 = 1, fs0 = FSrc(f0)
//                     (mod_cmfd.f90:448-454, :635-641), or f0 = a given
//                     flux (the discrete adjoint's warm start); one item
//                     per row.
//   xs_updt_items   : Dsigr_updt (mod_xsec.f90:199-226) with the node checks
//                     of check_xs (:90-168); one item per (node, group).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"

namespace adp {

__device__ __forceinline__ void assemble_items(const AssembleParams& P, long long start, long long stride) {
  const BoxGeom& G = P.G;
  const int NB = G.NB;
  const long long total = (long long)NB * P.ng;
  for (long long q = start; q < total; q += stride) {
    const int g = (int)(q / NB), b = (int)(q - (long long)g * NB);
    const unsigned m = G.nbm[b];
    double* df = P.df + (size_t)g * 6 * NB;
    const double* dn = P.dn + (size_t)g * 6 * NB;
    double* A = P.A + (size_t)g * 7 * NB;
    if (!(m & NB_ACTIVE)) {
      for (int c = 0; c < 7; ++c) {
        A[(size_t)c * NB + b] = 0.0;
        if (P.A32) P.A32[(size_t)g * 7 * NB + (size_t)c * NB + b] = 0.0f;
        if (P.A2) P.A2[(size_t)g * 7 * NB + (size_t)c * NB + b] = make_float2(0.0f, 0.0f);
      }
      continue;
    }
    if (!node_ok(P.ctl, G, b)) continue;
    const int i = b % G.nxx, j = (b / G.nxx) % G.nyy, k = b / G.plane;
    const double h[3] = {G.xdel[i], G.ydel[j], G.zdel[k]};
    if (P.with_coupling) {
      const double alb = 1.e30;
      const double Dn = P.D[(size_t)g * NB + b];
      for (int f = 0; f < 6; ++f) {
        const int u = f >> 1;
        double v;
        if (m & (1u << f)) {
          const int nb = b + face_off(G, f);
          const double d2 = P.D[(size_t)g * NB + nb];
          const double hn = hdir(G, u, nb);
          v = 2.0 * Dn * d2 / (Dn * hn + d2 * h[u]);
        } else {
          const int bc = G.bcf[f];
          if (bc == 0) v = 2.0 * alb * Dn / (2.0 * Dn + alb * h[u]);
          else if (bc == 1) v = Dn / (2.0 * Dn + 0.5 * h[u]);
          else v = 0.0;
        }
        df[(size_t)f * NB + b] = v;
      }
    }
    double F[6], N[6];
    for (int f = 0; f < 6; ++f) { F[f] = df[(size_t)f * NB + b]; N[f] = dn[(size_t)f * NB + b]; }
    double a[7];
    a[0] = (m & (1u << FZM)) ? -(F[FZM] - N[FZM]) / h[2] : 0.0;
    a[1] = (m & (1u << FYM)) ? -(F[FYM] - N[FYM]) / h[1] : 0.0;
    a[2] = (m & (1u << FXM)) ? -(F[FXM] - N[FXM]) / h[0] : 0.0;
    a[3] = (F[FXP] + F[FXM] - N[FXP] + N[FXM]) / h[0] + (F[FYP] + F[FYM] - N[FYP] + N[FYM]) / h[1] +
           (F[FZP] + F[FZM] - N[FZP] + N[FZM]) / h[2] + P.sigr[(size_t)g * NB + b];
    a[4] = (m & (1u << FXP)) ? -(F[FXP] + N[FXP]) / h[0] : 0.0;
    a[5] = (m & (1u << FYP)) ? -(F[FYP] + N[FYP]) / h[1] : 0.0;
    a[6] = (m & (1u << FZP)) ? -(F[FZP] + N[FZP]) / h[2] : 0.0;
    for (int c = 0; c < 7; ++c) {
      A[(size_t)c * NB + b] = a[c];
      if (P.A32) {
        const float hi = (float)a[c];
        P.A32[(size_t)g * 7 * NB + (size_t)c * NB + b] = hi;
        if (P.A2) P.A2[(size_t)g * 7 * NB + (size_t)c * NB + b] = make_float2(hi, (float)(a[c] - (double)hi));
      }
    }
  }
}

__device__ __forceinline__ void init_flux_items(const OuterParams& P, int start, int stride) {
  const BoxGeom& G = P.G;
  for (int b = start; b < G.NB; b += stride) {
    const bool act = G.nbm[b] & NB_ACTIVE;
    double fs = 0.0;
    for (int g = 0; g < P.ng; ++g) {
      const double x = act ? (P.init_phi ? P.init_phi[(size_t)g * P.NBH + b] : 1.0) : 0.0;
      P.phi[0][(size_t)g * P.NBH + b] = x;
      P.phi[1][(size_t)g * P.NBH + b] = x;
      fs = fs + x * P.wfis[(size_t)g * G.NB + b];
    }
    P.fs[0][b] = fs;
    P.fs[1][b] = fs;
  }
}

__device__ __forceinline__ void xs_updt_items(const BoxGeom& G, int ng, const int* act, int nnod, const double* sigtr,
                                              const double* siga, const double* sigs, double* D, double* sigr,
                                              OuterCtl* C, int start, int stride) {
  const int NB = G.NB;
  for (int q = start; q < nnod * ng; q += stride) {
    const int g = q / nnod, n = q - g * nnod, b = act[n];
    const double st = sigtr[(size_t)g * NB + b];
    if (st < kF1em5) {
      set_status(C, ADP_ERR_BADXS);
      atomicCAS(&C->err_node, -1, b);
      continue;
    }
    const double d = 1.0 / (3.0 * st);
    double dum = 0.;
    for (int h = 0; h < ng; ++h)
      if (h != g) dum = dum + sigs[((size_t)g * ng + h) * NB + b];
    const double sr = siga[(size_t)g * NB + b] + dum;
    D[(size_t)g * NB + b] = d;
    sigr[(size_t)g * NB + b] = sr;
    if (d < (double)1.e-20f || sr < 0.) {
      set_status(C, ADP_ERR_BADXS);
      atomicCAS(&C->err_node, -1, b);
    }
  }
}

}  // namespace adp
