// Rod ejection transient of one handle (mod_trans.f90:17-640,
// mod_cmfd.f90:800-952), the per-node work of a time step on the device:
//   before the step's outer iterations (k_trans_prep): the frequencies of
//   the exponential transformation, the removal of the step
//   sigr + 1/(theta v dt) + omega/v (the XS_updt value kept as sigrp), the
//   previous flux and fission source, and get_exsrc: the delayed source,
//   dfis, and the theta-method terms of the previous step;
//   after them (k_trans_after): uPden, PowTot, the leakage L of Lxyz and
//   the scattering source s0 that the next step's source needs, and the
//   adjoint-weighted reactivity
//   (mod_trans.f90:648-688) with the removal sigrp.
// The outer iterations themselves are outer_tr: the FP64 persistent kernel
// in its transient mode (source (1 - tbeta + dfis) chi fs + s0 + exsrc, no
// eigenvalue update) with the nodal update in cmode 2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"
#include "handle.h"
#include "nodal_body.cuh"

namespace adp {

struct TransParams {
  BoxGeom G;
  int ng, nnod, nf, omeg_mode, after_upden;
  long long NBH;
  const int* act;
  const double* phi;     // current flux [ng][NBH] (halo offset applied)
  const double* fs;      // current fission source [NB]
  const double* chin;
  const double* sigs;    // [ng][ng][NB], g -> h
  const double* sigf;
  const double* df;
  const double* dn;
  double* sigr;
  double* c0;            // [nf][NB]
  double* omeg;          // [ng][NB]
  double* ft;            // [ng][NB]
  double* fst;           // [NB]
  double* sigrp;         // [ng][NB]
  double* Lt;            // [ng][NB]
  double* exsrc;         // [ng][NB]
  double* wtr;           // [ng][NB] (1 - tbeta + dfis) chi
  double* wnode;         // [NB] 1 - tbeta + dfis
  double* s0q;           // [NB] the last group's s0 left by the previous outer iterations
  const double* af;      // [ng][NB]
  const double* velo;    // [ng]
  double beta[8], lamb[8];
  double sth, bth, tbeta, ht;
};

// One thread per node: the step's removal, old flux, and get_exsrc.
__global__ void k_trans_prep(TransParams P) {
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nnod; n += gridDim.x * blockDim.x) {
    const int b = P.act[n];
    // omega = log(f0 / ft) / dt from the previous step (rod_eject, mod_trans.f90:124-152)
    for (int g = 0; g < ng; ++g) {
      const size_t o = (size_t)g * NB + b;
      const double f = P.phi[(size_t)g * P.NBH + b];
      P.omeg[o] = P.omeg_mode ? log(f / P.ft[o]) / P.ht : 0.0;
    }
    // the s0 the last TSrc / TSrcTr left behind (k_trans_after)
    const int gl = ng - 1;
    const double s0l = P.s0q[b];
    // sigrp = sigr; sigr = sigr + 1/(theta v dt) + omega/v; ft = f0; fst = fs0
    for (int g = 0; g < ng; ++g) {
      const size_t o = (size_t)g * NB + b;
      const double sr = P.sigr[o];
      P.sigrp[o] = sr;
      P.sigr[o] = sr + 1.0 / (P.sth * P.velo[g] * P.ht) + P.omeg[o] / P.velo[g];
      P.ft[o] = P.phi[(size_t)g * P.NBH + b];
    }
    const double fst = P.fs[b];
    P.fst[b] = fst;
    // get_exsrc (mod_cmfd.f90:925-949)
    double dfis = 0.0, dt = 0.0, dtp = 0.0;
    for (int i = 0; i < P.nf; ++i) {
      const double pxe = exp(-P.lamb[i] * P.ht);
      double a1 = (1.0 - pxe) / (P.lamb[i] * P.ht);
      const double a2 = 1.0 - a1;
      a1 = a1 - pxe;
      const double c = P.c0[(size_t)i * NB + b];
      dfis = dfis + P.beta[i] * a2;
      dt = dt + P.lamb[i] * c * pxe + P.beta[i] * a1 * fst;
      dtp = dtp + P.lamb[i] * c;
    }
    const double w = 1.0 - P.tbeta + dfis;
    P.wnode[b] = w;
    for (int g = 0; g < ng; ++g) {
      const size_t o = (size_t)g * NB + b;
      const double chi = P.chin[o];
      const double s0 = (g == gl) ? s0l : 0.0;
      const double pthet = -P.Lt[o] - P.sigrp[o] * P.ft[o] + s0 + (1.0 - P.tbeta) * chi * fst + chi * dtp;
      P.exsrc[o] = chi * dt + exp(P.omeg[o] * P.ht) * P.ft[o] / (P.sth * P.velo[g] * P.ht) + P.bth * pthet;
      P.wtr[o] = w * chi;
    }
  }
}

// One thread per node: uPden (when after_upden), PowTot, L and the
// reactivity partials; block partials [5][kMaxBlocks]: power, src, rem,
// lea, fde.
__global__ void k_trans_after(TransParams P, double* part) {
  const BoxGeom& G = P.G;
  const int NB = G.NB, ng = P.ng;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nnod; n += gridDim.x * blockDim.x) {
    const int b = P.act[n];
    const double fs = P.fs[b], v = G.vdel[b];
    if (P.after_upden) {
      // uPden (mod_trans.f90:626-637)
      for (int i = 0; i < P.nf; ++i) {
        const double pxe = exp(-P.lamb[i] * P.ht);
        double a1 = (1.0 - pxe) / (P.lamb[i] * P.ht);
        const double a2 = 1.0 - a1;
        a1 = a1 - pxe;
        double& c = P.c0[(size_t)i * NB + b];
        c = c * pxe + P.beta[i] / P.lamb[i] * (a1 * P.fst[b] + a2 * fs);
      }
    }
    // PowTot (mod_trans.f90:541-552)
    double pw = 0.0;
    for (int g = 0; g < ng; ++g) {
      double q = P.phi[(size_t)g * P.NBH + b] * P.sigf[(size_t)g * NB + b] * v;
      if (q < 0.) q = 0.;
      pw = pw + q;
    }
    acc[0] = acc[0] + pw;
    // the s0 array the next step's get_exsrc reads is the one the last
    // TSrc / TSrcTr call left: each call zero-fills every group and fills
    // the group it solves, so only the last group's column remains, formed
    // with that call's cross sections (this step's, before the rods move
    // again) and the other groups' final flux (mod_cmfd.f90:1022-1027,
    // 1084-1089)
    {
      const int gl = ng - 1;
      double s0l = 0.0;
      for (int h = 0; h < ng; ++h)
        if (h != gl)
          s0l = __dadd_rn(s0l, __dmul_rn(P.sigs[((size_t)h * ng + gl) * NB + b], P.phi[(size_t)h * P.NBH + b]));
      P.s0q[b] = s0l;
    }
    // reactivity (mod_trans.f90:660-686), with L(n,g) kept for the next step
    for (int g = 0; g < ng; ++g) {
      const size_t o = (size_t)g * NB + b;
      double scg = 0.0;
      for (int h = 0; h < ng; ++h)
        if (h != g) scg = scg + P.sigs[((size_t)h * ng + g) * NB + b] * P.phi[(size_t)h * P.NBH + b];
      double L[3];
      net_leakage(G, P.phi + (size_t)g * P.NBH, P.df + (size_t)g * 6 * NB, P.dn + (size_t)g * 6 * NB, b, L);
      const double Lg = L[0] + L[1] + L[2];
      P.Lt[o] = Lg;
      const double a = P.af[o], chi = P.chin[o];
      acc[1] = acc[1] + a * (scg + chi * fs) * v;
      acc[2] = acc[2] + a * P.sigrp[o] * P.phi[(size_t)g * P.NBH + b] * v;
      acc[3] = acc[3] + a * Lg * v;
      acc[4] = acc[4] + a * chi * fs * v;
    }
  }
  block_partials<5, 0u>(acc, part);
}

// iPden (mod_trans.f90:582-589)
__global__ void k_trans_ipden(TransParams P) {
  const int NB = P.G.NB;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nnod; n += gridDim.x * blockDim.x) {
    const int b = P.act[n];
    for (int j = 0; j < P.nf; ++j) P.c0[(size_t)j * NB + b] = P.beta[j] / P.lamb[j] * P.fs[b];
  }
}

}  // namespace adp

using namespace adp;

namespace {

adp_status tfail(adp_handle* h, adp_status s, const std::string& m) {
  h->err = m;
  return s;
}

#define TCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return tfail(h, ADP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

TransParams trans_params(adp_handle* h, double ht, int omeg_mode, int after_upden) {
  TransParams P;
  P.G = box_geom(h);
  P.ng = h->ng;
  P.nnod = h->nnod;
  P.nf = h->nf;
  P.omeg_mode = omeg_mode;
  P.after_upden = after_upden;
  P.NBH = h->NBH;
  P.act = h->d_act;
  const int cur = h->h_ctl->cur;
  P.phi = h->d_phi[cur];
  P.fs = h->d_fs[cur];
  P.chin = h->d_chin;
  P.sigs = h->d_sigs;
  P.sigf = h->d_sigf;
  P.df = h->d_df;
  P.dn = h->d_dn;
  P.sigr = h->d_sigr;
  P.c0 = h->d_c0;
  P.omeg = h->d_omeg;
  P.ft = h->d_ft;
  P.fst = h->d_fst;
  P.sigrp = h->d_sigrp;
  P.Lt = h->d_Lt;
  P.exsrc = h->d_exsrc;
  P.wtr = h->d_wtr;
  P.wnode = h->d_wnode;
  P.s0q = h->d_s0q;
  P.af = h->d_af;
  P.velo = h->d_velo;
  for (int i = 0; i < 8; ++i) {
    P.beta[i] = h->beta[i];
    P.lamb[i] = h->lamb[i];
  }
  P.sth = h->sth;
  P.bth = h->bth;
  P.tbeta = h->tbeta;
  P.ht = ht;
  return P;
}

int node_blocks(const adp_handle* h) { return std::max(1, std::min((h->nnod + 255) / 256, kMaxBlocks)); }

adp_status read_ctl(adp_handle* h) {
  TCK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  TCK(cudaStreamSynchronize(h->st));
  return ADP_OK;
}

// k_trans_after and the host sums of its block partials (block order):
// relative power and the reactivity of the state.
adp_status trans_after(adp_handle* h, double ht, int upden, adp_trans_result* r) {
  adp_status s = read_ctl(h);
  if (s != ADP_OK) return s;
  const int blocks = node_blocks(h);
  k_trans_after<<<blocks, 256, 0, h->st>>>(trans_params(h, ht, 0, upden), h->d_tpart);
  TCK(cudaGetLastError());
  std::vector<double> part((size_t)5 * kMaxBlocks);
  TCK(cudaMemcpyAsync(part.data(), h->d_tpart, part.size() * 8, cudaMemcpyDeviceToHost, h->st));
  TCK(cudaStreamSynchronize(h->st));
  double t[5] = {0, 0, 0, 0, 0};
  for (int q = 0; q < 5; ++q)
    for (int k = 0; k < blocks; ++k) t[q] += part[(size_t)q * kMaxBlocks + k];
  if (t[4] == 0.0) return tfail(h, ADP_ERR_INPUT, "transient: the weighted fission source is zero");
  r->power = t[0];
  r->rho = (t[1] - t[3] - t[2]) / t[4];
  r->rho_dollar = r->rho / h->tbeta;
  return ADP_OK;
}

}  // namespace

extern "C" {

adp_status adp_trans_init(adp_handle* h, const adp_trans_opts* o, const double* af, adp_trans_result* r) {
  if (!h || !o || !af || !r) return ADP_ERR_INPUT;
  TCK(cudaSetDevice(h->dev));
  if (!h->xs_set || (!h->started[0])) return tfail(h, ADP_ERR_STATE, "adp_trans_init: solve the steady state first");
  if (o->nf < 1 || o->nf > 8 || !o->beta || !o->lambda || !o->velo)
    return tfail(h, ADP_ERR_INPUT, "adp_trans_init: 1..8 precursor families, beta, lambda and velocities");
  if (!(o->theta >= 0.001 && o->theta <= 1.0)) return tfail(h, ADP_ERR_INPUT, "adp_trans_init: theta in [0.001, 1]");
  const size_t NB = h->NB, G = h->ng;
  if (!h->trans_base) {
    size_t bytes = 0;
    auto add = [&](size_t b) { bytes += ((b + 255) & ~(size_t)255) + 256; };
    add(8 * NB * 8);              // c0
    for (int q = 0; q < 7; ++q) add(G * NB * 8);   // omeg ft sigrp Lt exsrc wtr af
    for (int q = 0; q < 2; ++q) add(G * NB * 8);   // wtr2 exsrc2 (double-float copies, mixed path)
    add(NB * 8);                  // fst
    add(NB * 8);                  // wnode
    add(NB * 8);                  // s0q
    add(G * 8);                   // velo
    add(5 * (size_t)kMaxBlocks * 8);
    TCK(cudaMalloc((void**)&h->trans_base, bytes));
    TCK(cudaMemsetAsync(h->trans_base, 0, bytes, h->st));
    DevArena A;
    A.base = h->trans_base;
    A.size = bytes;
    h->d_c0 = (double*)A.take(8 * NB * 8);
    double** pp[7] = {&h->d_omeg, &h->d_ft, &h->d_sigrp, &h->d_Lt, &h->d_exsrc, &h->d_wtr, &h->d_af};
    for (auto p : pp) *p = (double*)A.take(G * NB * 8);
    h->d_wtr2 = (float2*)A.take(G * NB * 8);
    h->d_exsrc2 = (float2*)A.take(G * NB * 8);
    h->d_fst = (double*)A.take(NB * 8);
    h->d_wnode = (double*)A.take(NB * 8);
    h->d_s0q = (double*)A.take(NB * 8);
    h->d_velo = (double*)A.take(G * 8);
    h->d_tpart = (double*)A.take(5 * (size_t)kMaxBlocks * 8);
  }
  h->nf = o->nf;
  double tb = 0.0;
  for (int i = 0; i < 8; ++i) {
    h->beta[i] = i < o->nf ? o->beta[i] : 0.0;
    h->lamb[i] = i < o->nf ? o->lambda[i] : 1.0;
  }
  for (int i = 0; i < o->nf; ++i) tb = tb + o->beta[i];   // tbeta (mod_trans.f90:86-92)
  h->tbeta = tb;
  h->sth = o->theta;
  h->bth = (1.0 - o->theta) / o->theta;
  h->extr = o->extr;
  h->velo.assign(o->velo, o->velo + G);
  TCK(cudaMemcpyAsync(h->d_velo, h->velo.data(), G * 8, cudaMemcpyHostToDevice, h->st));
  // af (nnod, ng) onto the box planes
  std::vector<double> box(G * NB, 0.0);
  for (size_t g = 0; g < G; ++g)
    for (int n = 0; n < h->nnod; ++n) box[g * NB + h->node2box[n]] = af[g * h->nnod + n];
  TCK(cudaMemcpyAsync(h->d_af, box.data(), box.size() * 8, cudaMemcpyHostToDevice, h->st));
  // sigrp of the steady state is sigr itself
  TCK(cudaMemcpyAsync(h->d_sigrp, h->d_sigr, G * NB * 8, cudaMemcpyDeviceToDevice, h->st));
  adp_status s = read_ctl(h);
  if (s != ADP_OK) return s;
  k_trans_ipden<<<node_blocks(h), 256, 0, h->st>>>(trans_params(h, 1.0, 0, 0));
  TCK(cudaGetLastError());
  if ((s = trans_after(h, 1.0, 0, r)) != ADP_OK) return s;
  h->tpow1 = r->power;
  r->relpow = 1.0;
  r->maxi = 0;
  r->outers = 0;
  r->device_ms = 0.0;
  h->trans_ready = true;
  return ADP_OK;
}

adp_status adp_trans_step(adp_handle* h, double ht, int omeg_mode, adp_trans_result* r) {
  if (!h || !r || !(ht > 0.0)) return ADP_ERR_INPUT;
  TCK(cudaSetDevice(h->dev));
  if (!h->trans_ready) return tfail(h, ADP_ERR_STATE, "adp_trans_step: call adp_trans_init first");
  adp_status s = read_ctl(h);
  if (s != ADP_OK) return s;
  k_trans_prep<<<node_blocks(h), 256, 0, h->st>>>(trans_params(h, ht, (omeg_mode && h->extr) ? 1 : 0, 0));
  TCK(cudaGetLastError());
  if (h->o.kern == ADP_KERN_SANM) TCK(launch_sanm_consts(nodal_params(h, 2), h->st));   // sigr changed
  adp_report rep;
  std::memset(&rep, 0, sizeof rep);
  h->trans_on = true;
  s = adp_outer(h, ADP_FORWARD, 0, &rep);
  h->trans_on = false;
  if (s != ADP_OK) return s;
  if ((s = trans_after(h, ht, 1, r)) != ADP_OK) return s;
  r->relpow = r->power / h->tpow1;
  r->maxi = rep.converged ? 0 : 1;
  r->outers = rep.outers;
  r->device_ms = rep.device_ms;
  return ADP_OK;
}

}  // extern "C"
