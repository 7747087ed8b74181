// The single-core solver handle (device state of one core), shared by the
// C ABI (capi.cu) and the batch (batch.cu), which owns one handle per core.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"

namespace adp {

// Bump allocator over one device allocation (256-byte aligned pieces).
struct DevArena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  void* take(size_t bytes) {
    size_t off = (used + 255) & ~(size_t)255;
    used = off + bytes;
    return base + off;
  }
};

}  // namespace adp

struct adp_handle {
  std::string err;
  int dev = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
  // geometry
  int nxx = 0, nyy = 0, nzz = 0, nnod = 0, NB = 0, plane = 0, ng = 0;
  long long NBH = 0;
  std::vector<int> node2box;
  std::vector<unsigned char> nbm;
  std::vector<int> ysmin, ysmax, xsmin, xsmax, evbase_host;
  std::vector<double> xdel, ydel, zdel, vdel;
  int bcf[6] = {0, 0, 0, 0, 0, 0};
  adp_opts o{};
  int nmat = 0;
  // device memory
  adp::DevArena ar;
  unsigned char* d_nbm = nullptr;
  double *d_xdel = nullptr, *d_ydel = nullptr, *d_zdel = nullptr, *d_vdel = nullptr;
  int *d_act = nullptr, *d_evbase = nullptr;
  double *d_D = nullptr, *d_sigr = nullptr, *d_nuf = nullptr, *d_sigf = nullptr, *d_chin = nullptr;
  double *d_sigs = nullptr, *d_dc = nullptr, *d_sigtr = nullptr, *d_siga = nullptr;
  double *d_df = nullptr, *d_dn = nullptr, *d_A = nullptr;
  float* d_A32 = nullptr;
  double* d_phi[2] = {nullptr, nullptr};
  double* d_fs[2] = {nullptr, nullptr};
  double *d_r = nullptr, *d_rs = nullptr;
  double2* d_pv2[2] = {nullptr, nullptr};   // (p, v)
  double2* d_st2 = nullptr;                 // (s, t)
  float *d_r32 = nullptr, *d_rs32 = nullptr;
  float2* d_pv2f[2] = {nullptr, nullptr};
  float2* d_st2f = nullptr;
  double* d_red = nullptr;
  // double-float copies of the mixed path
  // ((hi, lo) pairs)
  float2* d_A2 = nullptr;
  float2* d_x2[2] = {nullptr, nullptr};
  float2* d_fs2[2] = {nullptr, nullptr};
  float2 *d_chin2 = nullptr, *d_nuf2 = nullptr, *d_sigs2 = nullptr, *d_vdel2 = nullptr;
  float2* d_AT2 = nullptr;
  adp::OuterCtl* d_ctl = nullptr;
  adp::OuterCtl* h_ctl = nullptr;   // pinned mirror
  double *d_tr_k = nullptr, *d_tr_ser = nullptr, *d_tr_fer = nullptr, *d_tr_ndmax = nullptr;
  int* d_tr_flags = nullptr;
  double *d_sanm = nullptr, *d_S = nullptr, *d_a2 = nullptr, *d_a4 = nullptr, *d_L1 = nullptr, *d_Bc = nullptr;
  double* d_ndval = nullptr;
  long long* d_ndkey = nullptr;
  int* d_ndloc = nullptr;
  double* d_pbox = nullptr;
  // device staging of the node-order transfers (one host array at a time,
  // the material numbers and tables, check flags), allocated on first use
  char* xfer_base = nullptr;
  size_t xfer_size = 0;
  // output edits (adp_edit_*), allocated on first use
  char* edit_base = nullptr;
  size_t edit_size = 0;
  // adjoint-weighted edits (adp_reactivity, adp_core_beta), allocated on first use
  char* react_base = nullptr;
  size_t react_size = 0;
  // discrete adjoint (adp_adjoint_sens), allocated on its first call
  char* adj_base = nullptr;
  double* d_AT = nullptr;
  float* d_AT32 = nullptr;
  double* d_psi[2] = {nullptr, nullptr};
  double* d_fsa[2] = {nullptr, nullptr};
  adp::OuterCtl* d_ctla = nullptr;
  double *d_sens = nullptr, *d_spart = nullptr;
  // derivative through the nodal update (adp_adjoint_sens, SANM/PNM),
  // allocated on its first call
  char* nadj_base = nullptr;
  double *d_nside = nullptr, *d_nnodeu = nullptr, *d_nLbar = nullptr, *d_ndfbar = nullptr, *d_ndnbar = nullptr;
  double *d_nphibar = nullptr, *d_lam = nullptr, *d_Kd = nullptr, *d_cG = nullptr, *d_nkpart = nullptr;
  double *d_nrpart = nullptr, *d_nscal = nullptr, *d_NS = nullptr, *d_sens_full = nullptr;
  double* d_gam[2] = {nullptr, nullptr};
  double* d_fsg[2] = {nullptr, nullptr};
  double *d_gsrc = nullptr, *d_nufk = nullptr, *d_lpart = nullptr, *d_gpart = nullptr;
  adp::OuterCtl* d_ctlg = nullptr;
  float2 *d_gsrc2 = nullptr, *d_nufk2 = nullptr;   // (hi, lo) copies for the mixed kernel
  double* d_dlam = nullptr;                        // the last change of lam (its extrapolation)
  // feedback tables of adp_fb_set, kept until the next call
  char* fb_base = nullptr;
  size_t fb_size = 0;
  bool fb_ready = false, fb_chi_neg = false;
  int fb_nmat = 0, fb_nst = 0, fb_nb = 0;
  int fb_kind[4] = {0, 0, 0, 0};
  double fb_ref[4] = {0, 0, 0, 0};
  double fb_coreh = 0.0, fb_pos0 = 0.0, fb_ssize = 0.0;
  double *d_fb_base = nullptr, *d_fb_dsig = nullptr, *d_fb_rsig = nullptr, *d_fb_tab = nullptr, *d_fb_chi = nullptr;
  int *d_fb_mat = nullptr, *d_fb_bank = nullptr;
  // rod ejection transient (trans.cu), allocated by adp_trans_init
  char* trans_base = nullptr;
  bool trans_ready = false;
  bool trans_on = false;      // the current adp_outer call is outer_tr
  int nf = 0;
  double beta[8] = {0, 0, 0, 0, 0, 0, 0, 0}, lamb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<double> velo;
  double sth = 1.0, bth = 0.0, tbeta = 0.0, tpow1 = 0.0;
  int extr = 0;
  double *d_c0 = nullptr, *d_omeg = nullptr, *d_ft = nullptr, *d_fst = nullptr, *d_sigrp = nullptr;
  double *d_Lt = nullptr, *d_exsrc = nullptr, *d_wtr = nullptr, *d_wnode = nullptr, *d_af = nullptr;
  double *d_velo = nullptr, *d_tpart = nullptr, *d_s0q = nullptr;
  float2 *d_wtr2 = nullptr, *d_exsrc2 = nullptr;   // (hi, lo) copies for the mixed path
  // planes of chi, nu*fission and sigs that are nonzero at some node
  // (after_xs); all ones until known
  unsigned chi_nz = ~0u, nuf_nz = ~0u;
  unsigned long long sigs_nz = ~0ull;
  // state
  bool xs_set = false;
  bool fwd_ok = false;        // the flux is a converged forward solution of the current XS
  bool started[2] = {false, false};
  int launch_blocks = 0, launch_threads = 0;
  unsigned long long wait_ns = 0;   // barrier wait limit of the persistent kernels (0: the default 2 s)
  int phantom = 0;                  // adp_test_missing_block
  int sms = 0;
  adp_timers tm{};
};


namespace adp {
void set_global_error(const std::string& msg);
BoxGeom box_geom(const adp_handle* h);
OuterParams outer_params(adp_handle* h, int adj);
NodalParams nodal_params(adp_handle* h, int cmode);
}  // namespace adp
