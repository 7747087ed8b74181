// Adjoint-weighted edits of the current state, from mod_trans.f90:
//   reactivity (:648-688): rho = (src - lea - rem) / fde, with
//     src = <af, (sum_{h/=g} sigs(h->g) phi_h + chi_g fs0) V>,
//     rem = <af, sigrp phi V>, lea = <af, L V> (L = the net leakage of Lxyz
//     from df, dn and the flux), fde = <af, chi fs0 V>;
//   calc_beta (:692-746): beta = sum_i <chi af, beta_i(mat) nuf.phi V> /
//     <chi af, nuf.phi V>.
// At a converged static solution the first is 1 - 1/k for any weight af.
// One thread per node forms the node's contributions; block partials are
// summed on the host in block order.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"
#include "handle.h"
#include "nodal_body.cuh"

namespace adp {

struct ReactParams {
  BoxGeom G;
  int ng, nnod;
  long long NBH;
  const int* act;
  const double* phi;     // current flux [ng][NBH]
  const double* fs;      // current fission source [NB]
  const double* af;      // weight [ng][NB]
  const double* sigrp;   // removal [ng][NB]
  const double* sigs;    // [ng][ng][NB], g -> h
  const double* chin;
  const double* nuf;
  const double* df;
  const double* dn;
  const double* ibeta;   // [nf][NB] delayed fractions of the node's material
  int nf;
};

__global__ void k_reactivity(ReactParams P, double* part) {
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};   // src, rem, lea, fde
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nnod; n += gridDim.x * blockDim.x) {
    const int b = P.act[n];
    const double v = G.vdel[b];
    for (int g = 0; g < ng; ++g) {
      double scg = 0.0;
      for (int h = 0; h < ng; ++h)
        if (h != g) scg = scg + P.sigs[((size_t)h * ng + g) * NB + b] * P.phi[(size_t)h * P.NBH + b];
      double L[3];
      net_leakage(G, P.phi + (size_t)g * P.NBH, P.df + (size_t)g * 6 * NB, P.dn + (size_t)g * 6 * NB, b, L);
      const double a = P.af[(size_t)g * NB + b], chi = P.chin[(size_t)g * NB + b];
      acc[0] = acc[0] + a * (scg + chi * P.fs[b]) * v;
      acc[1] = acc[1] + a * P.sigrp[(size_t)g * NB + b] * P.phi[(size_t)g * P.NBH + b] * v;
      acc[2] = acc[2] + a * (L[0] + L[1] + L[2]) * v;
      acc[3] = acc[3] + a * chi * P.fs[b] * v;
    }
  }
  block_partials<4, 0u>(acc, part);
}

constexpr int kMaxDelayed = 8;

__global__ void k_beta(ReactParams P, double* part) {
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  double acc[1 + kMaxDelayed];
  for (int q = 0; q <= kMaxDelayed; ++q) acc[q] = 0.0;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nnod; n += gridDim.x * blockDim.x) {
    const int b = P.act[n];
    double vdum = 0.0;
    for (int g = 0; g < ng; ++g) vdum = vdum + P.nuf[(size_t)g * NB + b] * P.phi[(size_t)g * P.NBH + b];
    double w = 0.0;
    for (int g = 0; g < ng; ++g) w = w + P.chin[(size_t)g * NB + b] * vdum * P.af[(size_t)g * NB + b];
    acc[0] = acc[0] + G.vdel[b] * w;
    for (int i = 0; i < P.nf; ++i) {
      const double bi = P.ibeta[(size_t)i * NB + b];
      double wi = 0.0;
      for (int g = 0; g < ng; ++g) wi = wi + P.chin[(size_t)g * NB + b] * bi * vdum * P.af[(size_t)g * NB + b];
      acc[1 + i] = acc[1 + i] + G.vdel[b] * wi;
    }
  }
  block_partials<1 + kMaxDelayed, 0u>(acc, part);
}

}  // namespace adp

using namespace adp;

namespace {

adp_status rfail(adp_handle* h, adp_status s, const std::string& m) {
  h->err = m;
  return s;
}

#define RCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return rfail(h, ADP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Device scratch of the weighted edits: af, sigrp, ibeta planes and the
// block partials, allocated on first use.
adp_status react_scratch(adp_handle* h, int nf, double*& af, double*& sigrp, double*& ibeta, double*& part) {
  const size_t gnb = (size_t)h->ng * h->NB * 8;
  const size_t need = 2 * gnb + (size_t)kMaxDelayed * h->NB * 8 + (size_t)(1 + kMaxDelayed) * kMaxBlocks * 8 + 8 * 256;
  if (h->react_size < need) {
    if (h->react_base) cudaFree(h->react_base);
    h->react_base = nullptr;
    h->react_size = 0;
    RCK(cudaMalloc((void**)&h->react_base, need));
    h->react_size = need;
  }
  DevArena A;
  A.base = h->react_base;
  A.size = h->react_size;
  af = (double*)A.take(gnb);
  sigrp = (double*)A.take(gnb);
  ibeta = (double*)A.take((size_t)kMaxDelayed * h->NB * 8);
  part = (double*)A.take((size_t)(1 + kMaxDelayed) * kMaxBlocks * 8);
  (void)nf;
  return ADP_OK;
}

// a node array (nnod, ncomp), node index fastest, onto the box planes [ncomp][NB]
adp_status upload_nodes(adp_handle* h, const double* src, int ncomp, double* dst) {
  std::vector<double> box((size_t)ncomp * h->NB, 0.0);
  for (int c = 0; c < ncomp; ++c)
    for (int n = 0; n < h->nnod; ++n) box[(size_t)c * h->NB + h->node2box[n]] = src[(size_t)c * h->nnod + n];
  RCK(cudaMemcpyAsync(dst, box.data(), box.size() * 8, cudaMemcpyHostToDevice, h->st));
  RCK(cudaStreamSynchronize(h->st));
  return ADP_OK;
}

ReactParams react_params(adp_handle* h, const double* af, const double* sigrp, const double* ibeta, int nf) {
  ReactParams P;
  P.G = box_geom(h);
  P.ng = h->ng;
  P.nnod = h->nnod;
  P.NBH = h->NBH;
  P.act = h->d_act;
  const int cur = h->h_ctl->cur;
  P.phi = h->d_phi[cur];
  P.fs = h->d_fs[cur];
  P.af = af;
  P.sigrp = sigrp;
  P.sigs = h->d_sigs;
  P.chin = h->d_chin;
  P.nuf = h->d_nuf;
  P.df = h->d_df;
  P.dn = h->d_dn;
  P.ibeta = ibeta;
  P.nf = nf;
  return P;
}

}  // namespace

extern "C" {

adp_status adp_reactivity(adp_handle* h, const double* af, const double* sigrp, double* rho) {
  if (!h || !af || !rho) return ADP_ERR_INPUT;
  RCK(cudaSetDevice(h->dev));
  double *d_af, *d_sr, *d_ib, *d_part;
  adp_status s = react_scratch(h, 0, d_af, d_sr, d_ib, d_part);
  if (s != ADP_OK) return s;
  if ((s = upload_nodes(h, af, h->ng, d_af)) != ADP_OK) return s;
  if (sigrp && (s = upload_nodes(h, sigrp, h->ng, d_sr)) != ADP_OK) return s;
  RCK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  RCK(cudaStreamSynchronize(h->st));
  ReactParams P = react_params(h, d_af, sigrp ? d_sr : h->d_sigr, nullptr, 0);
  const int blocks = std::max(1, std::min((h->nnod + 255) / 256, kMaxBlocks));
  k_reactivity<<<blocks, 256, 0, h->st>>>(P, d_part);
  RCK(cudaGetLastError());
  std::vector<double> part((size_t)4 * kMaxBlocks);
  RCK(cudaMemcpyAsync(part.data(), d_part, part.size() * 8, cudaMemcpyDeviceToHost, h->st));
  RCK(cudaStreamSynchronize(h->st));
  double t[4] = {0, 0, 0, 0};
  for (int q = 0; q < 4; ++q)
    for (int k = 0; k < blocks; ++k) t[q] += part[(size_t)q * kMaxBlocks + k];
  if (t[3] == 0.0) return rfail(h, ADP_ERR_INPUT, "adp_reactivity: the weighted fission source is zero");
  *rho = (t[0] - t[2] - t[1]) / t[3];
  return ADP_OK;
}

adp_status adp_core_beta(adp_handle* h, const double* af, int nmat, int nf, const double* ibeta, const int* mat,
                         double* beta) {
  if (!h || !af || !ibeta || !mat || !beta) return ADP_ERR_INPUT;
  if (nf < 1 || nf > kMaxDelayed) return rfail(h, ADP_ERR_UNSUPPORTED, "adp_core_beta: 1..8 delayed groups");
  RCK(cudaSetDevice(h->dev));
  double *d_af, *d_sr, *d_ib, *d_part;
  adp_status s = react_scratch(h, nf, d_af, d_sr, d_ib, d_part);
  if (s != ADP_OK) return s;
  if ((s = upload_nodes(h, af, h->ng, d_af)) != ADP_OK) return s;
  // the delayed fractions of each node's material, (nnod, nf)
  std::vector<double> nb((size_t)h->nnod * nf);
  for (int n = 0; n < h->nnod; ++n) {
    if (mat[n] < 1 || mat[n] > nmat) return rfail(h, ADP_ERR_INPUT, "adp_core_beta: material number out of range");
    for (int i = 0; i < nf; ++i) nb[(size_t)i * h->nnod + n] = ibeta[(mat[n] - 1) + (size_t)nmat * i];
  }
  if ((s = upload_nodes(h, nb.data(), nf, d_ib)) != ADP_OK) return s;
  RCK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  RCK(cudaStreamSynchronize(h->st));
  ReactParams P = react_params(h, d_af, h->d_sigr, d_ib, nf);
  const int blocks = std::max(1, std::min((h->nnod + 255) / 256, kMaxBlocks));
  k_beta<<<blocks, 256, 0, h->st>>>(P, d_part);
  RCK(cudaGetLastError());
  std::vector<double> part((size_t)(1 + kMaxDelayed) * kMaxBlocks);
  RCK(cudaMemcpyAsync(part.data(), d_part, part.size() * 8, cudaMemcpyDeviceToHost, h->st));
  RCK(cudaStreamSynchronize(h->st));
  double t[1 + kMaxDelayed];
  for (int q = 0; q <= nf; ++q) {
    t[q] = 0.0;
    for (int k = 0; k < blocks; ++k) t[q] += part[(size_t)q * kMaxBlocks + k];
  }
  if (t[0] == 0.0) return rfail(h, ADP_ERR_INPUT, "adp_core_beta: the weighted fission rate is zero");
  double b = 0.0;
  for (int i = 1; i <= nf; ++i) b = b + t[i] / t[0];
  *beta = b;
  return ADP_OK;
}

}  // extern "C"
