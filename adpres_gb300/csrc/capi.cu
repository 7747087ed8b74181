// Host side of the C ABI (include/adpres_gb300.h): the core handle, layout
// conversion between the reference's node order and the padded device box,
// and the driver loop that stands in for outer()/outer_ad()
// (mod_cmfd.f90:415-509, :602-699).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"
#include "handle.h"
#include "host_geom.h"

using namespace adp;

namespace {

std::mutex g_err_mu;
std::string g_create_err;


}  // namespace

namespace adp {
// Message for adp_last_error(NULL) from entry points that take no handle.
void set_global_error(const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_create_err = msg;
}
}  // namespace adp


namespace {

// NVTX range over a scope: the phases of a call (CMFD outers, nodal update,
// adjoint rounds) appear by name in a timeline profiler.  Each range ends
// after the host has synchronised with its kernels, so it spans their
// device time.  Without a profiler attached the calls cost next to nothing.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

adp_status fail(adp_handle* h, adp_status s, const std::string& msg) {
  if (h) h->err = msg;
  else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
  }
  return s;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(h, ADP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
  } while (0)


// Upload a node-major Fortran array a(nnod, ng[, m]) into the box layout
// [ng][m][NB] (or [ng][NB]); inactive box positions get 0.
template <class T>
void to_box(const adp_handle* h, const T* src, int ncomp, std::vector<T>& out) {
  const int nn = h->nnod, NB = h->NB;
  out.assign((size_t)ncomp * NB, T(0));
  for (int c = 0; c < ncomp; ++c)
    for (int n = 0; n < nn; ++n) out[(size_t)c * NB + h->node2box[n]] = src[(size_t)c * nn + n];
}

}  // namespace

namespace adp {
BoxGeom box_geom(const adp_handle* h) {
  BoxGeom G;
  G.nxx = h->nxx;
  G.nyy = h->nyy;
  G.nzz = h->nzz;
  G.NB = h->NB;
  G.plane = h->plane;
  G.ng = h->ng;
  G.nbm = h->d_nbm;
  G.xdel = h->d_xdel;
  G.ydel = h->d_ydel;
  G.zdel = h->d_zdel;
  G.vdel = h->d_vdel;
  for (int f = 0; f < 6; ++f) G.bcf[f] = h->bcf[f];
  return G;
}
}  // namespace adp

namespace adp {

static adp_status gfail(std::string& err, adp_status st, const char* msg) {
  err = msg;
  return st;
}

// Geometry of one core from the reference's sdata view (adp_geom): box
// sizes, the ragged outline from plane 1 (mod_io.f90:1071-1110), the node
// order check (misc, :1317-1330), neighbour masks, volumes and the sweep
// order of the nodal update.  Shared by adp_create and adp_batch_create.
adp_status build_geometry(const adp_geom& g, HostGeom& H, std::string& err) {
  if (g.nxx < 1 || g.nyy < 1 || g.nzz < 2 || g.nnod < 1 || !g.ix || !g.iy || !g.iz || !g.xdel || !g.ydel || !g.zdel)
    return gfail(err, ADP_ERR_INPUT, "bad geometry sizes or null arrays");
  int bcs[6] = {g.east, g.west, g.north, g.south, g.bottom, g.top};
  for (int b : bcs)
    if (b < 0 || b > 2) return gfail(err, ADP_ERR_INPUT, "boundary conditions must be 0, 1 or 2");
  long long nb64 = (long long)g.nxx * g.nyy * g.nzz;
  if (nb64 > 400000000LL) return gfail(err, ADP_ERR_INPUT, "box too large");

  H.nxx = g.nxx;
  H.nyy = g.nyy;
  H.nzz = g.nzz;
  H.nnod = g.nnod;
  H.NB = (int)nb64;
  H.plane = g.nxx * g.nyy;
  H.NBH = (long long)H.NB + 2LL * H.plane;
  // face order X+ X- Y+ Y- Z+ Z- : east west north south top bottom
  H.bcf[FXP] = g.east;
  H.bcf[FXM] = g.west;
  H.bcf[FYP] = g.north;
  H.bcf[FYM] = g.south;
  H.bcf[FZP] = g.top;
  H.bcf[FZM] = g.bottom;
  H.xdel.assign(g.xdel, g.xdel + g.nxx);
  H.ydel.assign(g.ydel, g.ydel + g.nyy);
  H.zdel.assign(g.zdel, g.zdel + g.nzz);
  for (double d : H.xdel) if (!(d > 0)) return gfail(err, ADP_ERR_INPUT, "node sizes must be > 0");
  for (double d : H.ydel) if (!(d > 0)) return gfail(err, ADP_ERR_INPUT, "node sizes must be > 0");
  for (double d : H.zdel) if (!(d > 0)) return gfail(err, ADP_ERR_INPUT, "node sizes must be > 0");

  // Outline from the plane iz == 1 (mod_io.f90:1071-1110).
  const int nxx = g.nxx, nyy = g.nyy, nzz = g.nzz;
  H.ysmin.assign(nyy, nxx);
  H.ysmax.assign(nyy, -1);
  H.xsmin.assign(nxx, nyy);
  H.xsmax.assign(nxx, -1);
  for (int n = 0; n < g.nnod; ++n) {
    int i = g.ix[n] - 1, j = g.iy[n] - 1, k = g.iz[n] - 1;
    if (i < 0 || i >= nxx || j < 0 || j >= nyy || k < 0 || k >= nzz) return gfail(err, ADP_ERR_INPUT, "node index out of the box");
    if (k == 0) {
      H.ysmin[j] = std::min(H.ysmin[j], i);
      H.ysmax[j] = std::max(H.ysmax[j], i);
      H.xsmin[i] = std::min(H.xsmin[i], j);
      H.xsmax[i] = std::max(H.xsmax[i], j);
    }
  }
  // The node order must be the reference's (misc, mod_io.f90:1317-1330).
  {
    int n = 0;
    std::vector<unsigned char> on((size_t)nxx * nyy, 0);
    for (int k = 0; k < nzz; ++k)
      for (int j = 0; j < nyy; ++j)
        for (int i = H.ysmin[j]; i <= H.ysmax[j]; ++i) {
          if (n >= g.nnod || g.ix[n] - 1 != i || g.iy[n] - 1 != j || g.iz[n] - 1 != k) return gfail(err, ADP_ERR_INPUT, "nodes are not in the reference order (k, j, i over the plane-1 outline)");
          if (k == 0) on[(size_t)j * nxx + i] = 1;
          ++n;
        }
    if (n != g.nnod) return gfail(err, ADP_ERR_INPUT, "node count does not match the outline");
    // Column and row outlines must agree (the reference's zero-material
    // check, mod_io.f90:1112-1132), and every line needs two nodes
    // (the two-node sweeps read a neighbour at every line end).
    for (int i = 0; i < nxx; ++i) {
      if (H.xsmax[i] - H.xsmin[i] < 1) return gfail(err, ADP_ERR_INPUT, "a y column holds fewer than two nodes");
      for (int j = H.xsmin[i]; j <= H.xsmax[i]; ++j)
        if (!on[(size_t)j * nxx + i]) return gfail(err, ADP_ERR_INPUT, "outline has a hole inside the core");
    }
    for (int j = 0; j < nyy; ++j)
      if (H.ysmax[j] - H.ysmin[j] < 1) return gfail(err, ADP_ERR_INPUT, "an x row holds fewer than two nodes");
  }
  H.node2box.resize(g.nnod);
  H.nbm.assign(H.NB, 0);
  H.vdel.assign(H.NB, 0.0);
  for (int n = 0; n < g.nnod; ++n) {
    int i = g.ix[n] - 1, j = g.iy[n] - 1, k = g.iz[n] - 1;
    int b = i + nxx * (j + nyy * k);
    H.node2box[n] = b;
    unsigned m = NB_ACTIVE;
    if (i != H.ysmax[j]) m |= 1u << FXP;
    if (i != H.ysmin[j]) m |= 1u << FXM;
    if (j != H.xsmax[i]) m |= 1u << FYP;
    if (j != H.xsmin[i]) m |= 1u << FYM;
    if (k != nzz - 1) m |= 1u << FZP;
    if (k != 0) m |= 1u << FZM;
    H.nbm[b] = (unsigned char)m;
    H.vdel[b] = H.xdel[i] * H.ydel[j] * H.zdel[k];
  }
  // Sweep-order index of each node's minus face, per direction
  // (mod_nodal.f90:53-125: x lines over (k,j), y lines over (k,i), z lines
  // over the plane-1 columns in node order).
  std::vector<int>& evbase = H.evbase;
  evbase.assign((size_t)3 * H.NB, 0);
  {
    std::vector<long long> prefx(nyy), prefy(nxx);
    long long Tx = 0, Ty = 0;
    for (int j = 0; j < nyy; ++j) { prefx[j] = Tx; Tx += H.ysmax[j] - H.ysmin[j] + 2; }
    for (int i = 0; i < nxx; ++i) { prefy[i] = Ty; Ty += H.xsmax[i] - H.xsmin[i] + 2; }
    long long base_y = Tx * nzz, base_z = base_y + Ty * nzz;
    std::vector<int> col((size_t)nxx * nyy, -1);
    int c = 0;
    for (int j = 0; j < nyy; ++j)
      for (int i = H.ysmin[j]; i <= H.ysmax[j]; ++i) col[(size_t)j * nxx + i] = c++;
    long long total = base_z + (long long)c * (nzz + 1);
    if (total * kMaxGroups > 0x7fffffffffffLL) return gfail(err, ADP_ERR_INPUT, "too many faces");
    if (total > 0x7fffffffLL) return gfail(err, ADP_ERR_INPUT, "too many faces");
    for (int n = 0; n < g.nnod; ++n) {
      int i = g.ix[n] - 1, j = g.iy[n] - 1, k = g.iz[n] - 1, b = H.node2box[n];
      evbase[b] = (int)(k * Tx + prefx[j] + (i - H.ysmin[j]));
      evbase[(size_t)H.NB + b] = (int)(base_y + k * Ty + prefy[i] + (j - H.xsmin[i]));
      evbase[(size_t)2 * H.NB + b] = (int)(base_z + (long long)col[(size_t)j * nxx + i] * (nzz + 1) + k);
    }
  }

  H.nnod = g.nnod;
  return ADP_OK;
}

}  // namespace adp

extern "C" {

size_t adp_last_error(const adp_handle* h, char* buf, size_t len) {
  std::string m;
  if (h) m = h->err;
  else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    m = g_create_err;
  }
  if (buf && len) {
    size_t n = std::min(len - 1, m.size());
    std::memcpy(buf, m.data(), n);
    buf[n] = 0;
  }
  return m.size();
}

adp_status adp_destroy(adp_handle* h) {
  if (!h) return ADP_OK;
  cudaSetDevice(h->dev);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->ar.base) cudaFree(h->ar.base);
  if (h->adj_base) cudaFree(h->adj_base);
  if (h->nadj_base) cudaFree(h->nadj_base);
  if (h->edit_base) cudaFree(h->edit_base);
  if (h->react_base) cudaFree(h->react_base);
  if (h->trans_base) cudaFree(h->trans_base);
  if (h->xfer_base) cudaFree(h->xfer_base);
  if (h->fb_base) cudaFree(h->fb_base);
  if (h->h_ctl) cudaFreeHost(h->h_ctl);
  for (cudaEvent_t e : {h->e0, h->e1, h->e2, h->e3})
    if (e) cudaEventDestroy(e);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return ADP_OK;
}

adp_status adp_create(const adp_geom* geom, const adp_opts* opts, adp_handle** out) {
  adp_handle* h = nullptr;
  if (!geom || !opts || !out) return fail(nullptr, ADP_ERR_INPUT, "adp_create: null argument");
  *out = nullptr;
  const adp_geom& g = *geom;
  if (g.nxx < 1 || g.nyy < 1 || g.nzz < 2 || g.nnod < 1 || !g.ix || !g.iy || !g.iz || !g.xdel || !g.ydel || !g.zdel)
    return fail(nullptr, ADP_ERR_INPUT, "adp_create: bad geometry sizes or null arrays");
  if (opts->ng < 1 || opts->ng > kMaxGroups)
    return fail(nullptr, ADP_ERR_UNSUPPORTED, "adp_create: groups must be 1..8");
  if (opts->kern < 0 || opts->kern > 2 || opts->precision < 0 || opts->precision > 1)
    return fail(nullptr, ADP_ERR_INPUT, "adp_create: bad kern or precision");
  h = new adp_handle();
  {
    adp::HostGeom H;
    std::string gerr;
    adp_status gs = adp::build_geometry(g, H, gerr);
    if (gs != ADP_OK) {
      adp_destroy(h);
      return fail(nullptr, gs, "adp_create: " + gerr);
    }
    h->nxx = H.nxx;
    h->nyy = H.nyy;
    h->nzz = H.nzz;
    h->nnod = H.nnod;
    h->NB = H.NB;
    h->plane = H.plane;
    h->NBH = H.NBH;
    for (int f = 0; f < 6; ++f) h->bcf[f] = H.bcf[f];
    h->xdel = std::move(H.xdel);
    h->ydel = std::move(H.ydel);
    h->zdel = std::move(H.zdel);
    h->vdel = std::move(H.vdel);
    h->ysmin = std::move(H.ysmin);
    h->ysmax = std::move(H.ysmax);
    h->xsmin = std::move(H.xsmin);
    h->xsmax = std::move(H.xsmax);
    h->node2box = std::move(H.node2box);
    h->nbm = std::move(H.nbm);
    h->evbase_host = std::move(H.evbase);
  }
  h->ng = opts->ng;
  const int nxx = h->nxx, nyy = h->nyy, nzz = h->nzz;
  // Options with the reference defaults.
  h->o = *opts;
  if (h->o.nin < 1) h->o.nin = 2;
  if (h->o.nout < 1) h->o.nout = 500;
  if (h->o.nac < 1) h->o.nac = 5;
  if (h->o.nupd < 1) h->o.nupd = (int)std::ceil((float)(nxx + nyy + nzz) / 2.5f);
  if (!(h->o.serc > 0)) h->o.serc = kF1em5;
  if (!(h->o.ferc > 0)) h->o.ferc = kF1em5;
  if (h->o.nout < h->o.nupd && h->o.kern != ADP_KERN_FDM) {
    adp_destroy(h);
    return fail(nullptr, ADP_ERR_INPUT, "max. number of outer iteration should be bigger than nodal update interval");
  }

  // Device resources.
  cudaError_t ce = cudaGetDevice(&h->dev);
  if (ce != cudaSuccess) { adp_destroy(h); return fail(nullptr, ADP_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(ce)); }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, h->dev);
  h->sms = prop.multiProcessorCount;
  if (!prop.cooperativeLaunch) { adp_destroy(h); return fail(nullptr, ADP_ERR_CUDA, "device lacks cooperative launch"); }
  if ((ce = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking)) != cudaSuccess ||
      (ce = cudaEventCreate(&h->e0)) != cudaSuccess || (ce = cudaEventCreate(&h->e1)) != cudaSuccess ||
      (ce = cudaEventCreate(&h->e2)) != cudaSuccess || (ce = cudaEventCreate(&h->e3)) != cudaSuccess ||
      (ce = cudaMallocHost((void**)&h->h_ctl, sizeof(OuterCtl))) != cudaSuccess) {
    adp_destroy(h);
    return fail(nullptr, ADP_ERR_CUDA, std::string("stream/event set-up: ") + cudaGetErrorString(ce));
  }
  const size_t NB = h->NB, G = h->ng, NBH = h->NBH, nn = h->nnod, nout = h->o.nout;
  const bool mixed = h->o.precision == ADP_MIXED;
  size_t bytes = 0;
  auto add = [&](size_t b) { bytes += ((b + 255) & ~(size_t)255) + 256; };
  add(NB); add(nxx * 8); add(nyy * 8); add(nzz * 8); add(NB * 8); add(nn * 4); add(3 * NB * 4);
  add(G * NB * 8 * 7);              // D sigr nuf sigf chin sigtr siga
  add(G * G * NB * 8);              // sigs
  add(G * 6 * NB * 8 * 3);          // dc df dn
  add(G * 7 * NB * 8);              // A
  if (mixed) add(G * 7 * NB * 4);   // A32
  add(G * NBH * 8 * 2);             // phi
  add(NB * 8 * 2);                  // fs
  add(NBH * 8 * 8);                 // Krylov FP64
  if (mixed) add(NBH * 4 * 8);      // Krylov FP32
  if (mixed) {                      // double-float (hi, lo) pairs: A, flux, fission source, XS copies
    add(G * 7 * NB * 8);
    for (int q = 0; q < 2; ++q) add(G * NBH * 8);
    for (int q = 0; q < 2; ++q) add(NB * 8);
    for (int q = 0; q < 2; ++q) add(G * NB * 8);
    add(G * G * NB * 8);
    add(NB * 8);
  }
  add(2 * kRedQ * kMaxBlocks * 8);
  add(sizeof(OuterCtl));
  add(nout * 8 * 4 + nout * 4);
  if (opts->kern == ADP_KERN_SANM) add(3 * 6 * G * NB * 8);
  if (opts->kern != ADP_KERN_FDM) add(3 * G * NB * 8 * 4);
  if (opts->kern != ADP_KERN_FDM) add(3 * G * G * NB * 8);
  add(kMaxBlocks * 8 * 2 + kMaxBlocks * 4);
  add(NB * 8);
  h->ar.size = bytes;
  if ((ce = cudaMalloc((void**)&h->ar.base, bytes)) != cudaSuccess) {
    adp_destroy(h);
    return fail(nullptr, ADP_ERR_CUDA, std::string("cudaMalloc of the core state: ") + cudaGetErrorString(ce));
  }
  DevArena& A = h->ar;
  h->d_nbm = (unsigned char*)A.take(NB);
  h->d_xdel = (double*)A.take(nxx * 8);
  h->d_ydel = (double*)A.take(nyy * 8);
  h->d_zdel = (double*)A.take(nzz * 8);
  h->d_vdel = (double*)A.take(NB * 8);
  h->d_act = (int*)A.take(nn * 4);
  h->d_evbase = (int*)A.take(3 * NB * 4);
  h->d_D = (double*)A.take(G * NB * 8);
  h->d_sigr = (double*)A.take(G * NB * 8);
  h->d_nuf = (double*)A.take(G * NB * 8);
  h->d_sigf = (double*)A.take(G * NB * 8);
  h->d_chin = (double*)A.take(G * NB * 8);
  h->d_sigtr = (double*)A.take(G * NB * 8);
  h->d_siga = (double*)A.take(G * NB * 8);
  h->d_sigs = (double*)A.take(G * G * NB * 8);
  h->d_dc = (double*)A.take(G * 6 * NB * 8);
  h->d_df = (double*)A.take(G * 6 * NB * 8);
  h->d_dn = (double*)A.take(G * 6 * NB * 8);
  h->d_A = (double*)A.take(G * 7 * NB * 8);
  if (mixed) h->d_A32 = (float*)A.take(G * 7 * NB * 4);
  for (int t = 0; t < 2; ++t) h->d_phi[t] = (double*)A.take(G * NBH * 8) + h->plane;
  for (int t = 0; t < 2; ++t) h->d_fs[t] = (double*)A.take(NB * 8);
  // Krylov vectors: r, rs, then the (p, v) pairs of both buffers and the
  // (s, t) pairs, each with its halo planes (the arena is zeroed below)
  double* kv = (double*)A.take(NBH * 8 * 8);
  h->d_r = kv + h->plane;
  h->d_rs = kv + NBH + h->plane;
  for (int t = 0; t < 2; ++t) h->d_pv2[t] = reinterpret_cast<double2*>(kv + (2 + 2 * t) * NBH) + h->plane;
  h->d_st2 = reinterpret_cast<double2*>(kv + 6 * NBH) + h->plane;
  if (mixed) {
    float* kf = (float*)A.take(NBH * 4 * 8);
    h->d_r32 = kf + h->plane;
    h->d_rs32 = kf + NBH + h->plane;
    for (int t = 0; t < 2; ++t) h->d_pv2f[t] = reinterpret_cast<float2*>(kf + (2 + 2 * t) * NBH) + h->plane;
    h->d_st2f = reinterpret_cast<float2*>(kf + 6 * NBH) + h->plane;
  }
  h->d_red = (double*)A.take(2 * kRedQ * kMaxBlocks * 8);
  if (mixed) {
    h->d_A2 = (float2*)A.take(G * 7 * NB * 8);
    for (int t = 0; t < 2; ++t) h->d_x2[t] = (float2*)A.take(G * NBH * 8) + h->plane;
    for (int t = 0; t < 2; ++t) h->d_fs2[t] = (float2*)A.take(NB * 8);
    h->d_chin2 = (float2*)A.take(G * NB * 8);
    h->d_nuf2 = (float2*)A.take(G * NB * 8);
    h->d_sigs2 = (float2*)A.take(G * G * NB * 8);
    h->d_vdel2 = (float2*)A.take(NB * 8);
  }
  h->d_ctl = (OuterCtl*)A.take(sizeof(OuterCtl));
  h->d_tr_k = (double*)A.take(nout * 8);
  h->d_tr_ser = (double*)A.take(nout * 8);
  h->d_tr_fer = (double*)A.take(nout * 8);
  h->d_tr_ndmax = (double*)A.take(nout * 8);
  h->d_tr_flags = (int*)A.take(nout * 4);
  if (opts->kern == ADP_KERN_SANM) h->d_sanm = (double*)A.take(3 * 6 * G * NB * 8);
  if (opts->kern != ADP_KERN_FDM) {
    h->d_S = (double*)A.take(3 * G * NB * 8);
    h->d_a2 = (double*)A.take(3 * G * NB * 8);
    h->d_a4 = (double*)A.take(3 * G * NB * 8);
    h->d_L1 = (double*)A.take(3 * G * NB * 8);
    h->d_Bc = (double*)A.take(3 * G * G * NB * 8);
  }
  h->d_ndval = (double*)A.take(kMaxBlocks * 8);
  h->d_ndkey = (long long*)A.take(kMaxBlocks * 8);
  h->d_ndloc = (int*)A.take(kMaxBlocks * 4);
  h->d_pbox = (double*)A.take(NB * 8);
  if (A.used > A.size) { adp_destroy(h); return fail(nullptr, ADP_ERR_CUDA, "internal: arena overflow"); }

  // Zero everything (halos, inactive positions, dn = 0 as coup_coef's first call).
  if ((ce = cudaMemsetAsync(A.base, 0, A.size, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_nbm, h->nbm.data(), NB, cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_xdel, h->xdel.data(), nxx * 8, cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_ydel, h->ydel.data(), nyy * 8, cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_zdel, h->zdel.data(), nzz * 8, cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_vdel, h->vdel.data(), NB * 8, cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_act, h->node2box.data(), nn * 4, cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(h->d_evbase, h->evbase_host.data(), 3 * NB * 4, cudaMemcpyHostToDevice, h->st)) != cudaSuccess) {
    adp_destroy(h);
    return fail(nullptr, ADP_ERR_CUDA, std::string("initial upload: ") + cudaGetErrorString(ce));
  }
  if (mixed && (ce = launch_split(h->d_vdel, h->d_vdel2, (long long)NB, h->st)) != cudaSuccess) {
    adp_destroy(h);
    return fail(nullptr, ADP_ERR_CUDA, std::string("initial upload: ") + cudaGetErrorString(ce));
  }
  OuterCtl c0;
  std::memset(&c0, 0, sizeof c0);
  c0.Ke = 1.0;
  c0.err_node = -1;
  *h->h_ctl = c0;
  if ((ce = cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(OuterCtl), cudaMemcpyHostToDevice, h->st)) != cudaSuccess ||
      (ce = cudaStreamSynchronize(h->st)) != cudaSuccess) {
    adp_destroy(h);
    return fail(nullptr, ADP_ERR_CUDA, std::string("initial upload: ") + cudaGetErrorString(ce));
  }
  h->launch_threads = 0;   // automatic (launch_shape)
  *out = h;
  return ADP_OK;
}

// Device staging of the node-order transfers (transfer.cu): one host array
// of up to max(ng*ng, 6*ng) components, the material numbers, the material
// tables of nmat materials and the check flags.  Grows, never shrinks.
struct Xfer {
  double* stage;
  int* mat;
  double* tab;
  int* flags;
};

static adp_status xfer_reserve(adp_handle* h, int nmat, Xfer& X) {
  const size_t nn = h->nnod, G = h->ng;
  const size_t ncomp = std::max(G * G, 6 * G);
  const size_t ntab = (5 * G + G * G) * (size_t)std::max(nmat, 1);
  size_t need = 0;
  auto add = [&](size_t b) { need += ((b + 255) & ~(size_t)255) + 256; };
  add(ncomp * nn * 8);
  add(nn * 4);
  add(ntab * 8);
  add(64);
  if (h->xfer_size < need) {
    if (h->xfer_base) CK(cudaFree(h->xfer_base));
    h->xfer_base = nullptr;
    h->xfer_size = 0;
    CK(cudaMalloc((void**)&h->xfer_base, need));
    h->xfer_size = need;
  }
  DevArena A;
  A.base = h->xfer_base;
  A.size = h->xfer_size;
  X.stage = (double*)A.take(ncomp * nn * 8);
  X.mat = (int*)A.take(nn * 4);
  X.tab = (double*)A.take(ntab * 8);
  X.flags = (int*)A.take(64);
  return ADP_OK;
}

// One host array a(nnod, A, B) (node fastest) into the box planes [A][B]
// of stride `stride`: a contiguous copy, then the scatter on the device.
static adp_status put_nodes(adp_handle* h, const Xfer& X, const double* src, int A, int B, double* dst,
                            long long stride, int chk) {
  CK(cudaMemcpyAsync(X.stage, src, (size_t)h->nnod * A * B * 8, cudaMemcpyHostToDevice, h->st));
  CK(launch_nodes_to_box(X.stage, dst, h->d_act, h->nnod, A, B, stride, chk, X.flags, h->st));
  return ADP_OK;
}

// The box planes [A][B] back into a host array a(nnod, A, B).
static adp_status get_nodes(adp_handle* h, const Xfer& X, const double* src, int A, int B, long long stride,
                            double* dst) {
  CK(launch_box_to_nodes(src, X.stage, h->d_act, h->nnod, A, B, stride, h->st));
  CK(cudaMemcpyAsync(dst, X.stage, (size_t)h->nnod * A * B * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return ADP_OK;
}

// Material numbers in range and chi >= 0 are checked on the host (nnod and
// nmat*ng values); the node tables' signs on the device.
static adp_status check_mat(adp_handle* h, int nmat, const int* mat) {
  for (int n = 0; n < h->nnod; ++n)
    if (mat[n] < 1 || mat[n] > nmat) return fail(h, ADP_ERR_INPUT, "adp_set_xs: material number out of range");
  return ADP_OK;
}

static bool chi_negative(const adp_handle* h, int nmat, const double* chi) {
  for (size_t q = 0; q < (size_t)h->ng * nmat; ++q)
    if (chi[q] < 0.) return true;
  return false;
}

// check_xs on the inputs that are not recomputed (mod_xsec.f90:90-168), in
// its order: nu*fission, chi, scattering.
static adp_status xs_flags(adp_handle* h, const Xfer& X, bool chi_neg) {
  int fl = 0;
  CK(cudaMemcpyAsync(&fl, X.flags, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (fl & 1) return fail(h, ADP_ERR_BADXS, "nu*fission xs is negative");
  if (chi_neg) return fail(h, ADP_ERR_BADXS, "fission spectrum is negative");
  if (fl & 4) return fail(h, ADP_ERR_BADXS, "scattering xs is negative");
  return ADP_OK;
}

static XsBox xs_box(adp_handle* h) {
  return XsBox{h->d_sigtr, h->d_siga, h->d_nuf, h->d_sigf, h->d_chin, h->d_sigs};
}

// ADFs dc(nnod, ng, 6) into [ng][6][NB]; 1 where the host gives none.
static adp_status put_dc(adp_handle* h, const Xfer& X, const double* dc) {
  if (dc) return put_nodes(h, X, dc, h->ng, 6, h->d_dc, h->NB, 0);
  CK(launch_fill_box(h->d_dc, h->d_act, h->nnod, h->ng * 6, h->NB, 1.0, h->st));
  return ADP_OK;
}

// nu*fission, fission, scattering and ADF node tables and chi of the node's
// material: the part of the upload that adp_set_xs and adp_xs_updt_nodes share.
static adp_status upload_xs_common(adp_handle* h, int nmat, const double* nuf, const double* sigf, const double* chi,
                                   const int* mat, const double* sigs, const double* dc, Xfer& X, bool& chi_neg) {
  const int nn = h->nnod, G = h->ng;
  h->fwd_ok = false;
  if (nmat < 1 || !nuf || !sigf || !chi || !mat || !sigs) return fail(h, ADP_ERR_INPUT, "adp_set_xs: null array");
  adp_status s = check_mat(h, nmat, mat);
  if (s != ADP_OK) return s;
  chi_neg = chi_negative(h, nmat, chi);
  if ((s = xfer_reserve(h, nmat, X)) != ADP_OK) return s;
  CK(cudaMemsetAsync(X.flags, 0, sizeof(int), h->st));
  CK(cudaMemcpyAsync(X.mat, mat, (size_t)nn * 4, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(X.tab, chi, (size_t)G * nmat * 8, cudaMemcpyHostToDevice, h->st));
  XsTables T{};
  T.chi = X.tab;
  CK(launch_base_updt(T, X.mat, h->d_act, nn, nmat, G, h->NB, xs_box(h), X.flags, h->st));
  if ((s = put_nodes(h, X, nuf, G, 1, h->d_nuf, h->NB, 1)) != ADP_OK) return s;
  if ((s = put_nodes(h, X, sigf, G, 1, h->d_sigf, h->NB, 0)) != ADP_OK) return s;
  if ((s = put_nodes(h, X, sigs, G, G, h->d_sigs, h->NB, 4)) != ADP_OK) return s;
  if ((s = put_dc(h, X, dc)) != ADP_OK) return s;
  h->nmat = nmat;
  return ADP_OK;
}

}  // extern "C"

NodalParams adp::nodal_params(adp_handle* h, int cmode) {
  NodalParams P;
  std::memset(&P, 0, sizeof P);
  P.G = box_geom(h);
  P.ng = h->ng;
  P.cmode = cmode;
  P.pnm = h->o.kern == ADP_KERN_PNM;
  P.nnod = h->nnod;
  P.nout = h->o.nout;
  P.serc = h->o.serc;
  P.ferc = h->o.ferc;
  P.NBH = h->NBH;
  P.act = h->d_act;
  P.phi[0] = h->d_phi[0];
  P.phi[1] = h->d_phi[1];
  P.D = h->d_D;
  P.sigr = h->d_sigr;
  P.nuf = h->d_nuf;
  P.chin = h->d_chin;
  P.sigs = h->d_sigs;
  P.df = h->d_df;
  P.dn = h->d_dn;
  P.dc = h->d_dc;
  P.sanm = h->d_sanm;
  P.S = h->d_S;
  P.a2 = h->d_a2;
  P.a4 = h->d_a4;
  P.L1 = h->d_L1;
  P.Bc = h->d_Bc;
  P.evbase = h->d_evbase;
  if (cmode == 2) {
    P.exsrc = h->d_exsrc;
    P.wnode = h->d_wnode;
  }
  P.nd_val = h->d_ndval;
  P.nd_key = h->d_ndkey;
  P.nd_loc = h->d_ndloc;
  P.ctl = h->d_ctl;
  P.tr_ndmax = h->d_tr_ndmax;
  P.tr_flags = h->d_tr_flags;
  return P;
}

extern "C" {

static adp_status after_xs(adp_handle* h) {
  h->chi_nz = h->nuf_nz = ~0u;
  h->sigs_nz = ~0ull;
  if (h->ng <= 8) {
    // which source planes hold a nonzero value (the outer kernel skips the
    // terms of all-zero planes: down-scatter-only cores, chi = 0 groups)
    Xfer X;
    adp_status s = xfer_reserve(h, std::max(h->nmat, 1), X);
    if (s != ADP_OK) return s;
    unsigned* m = reinterpret_cast<unsigned*>(X.flags) + 4;
    unsigned hm[4] = {0, 0, 0, 0};
    CK(cudaMemsetAsync(m, 0, sizeof hm, h->st));
    CK(launch_xs_nonzero(h->d_chin, h->d_nuf, h->d_sigs, h->d_act, h->nnod, h->ng, h->NB, m, h->st));
    CK(cudaMemcpyAsync(hm, m, sizeof hm, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->chi_nz = hm[0];
    h->nuf_nz = hm[1];
    h->sigs_nz = (unsigned long long)hm[2] | ((unsigned long long)hm[3] << 32);
  }
  if (h->o.precision == ADP_MIXED) {
    const long long gn = (long long)h->ng * h->NB;
    CK(launch_split(h->d_chin, h->d_chin2, gn, h->st));
    CK(launch_split(h->d_nuf, h->d_nuf2, gn, h->st));
    CK(launch_split(h->d_sigs, h->d_sigs2, gn * h->ng, h->st));
  }
  if (h->o.kern == ADP_KERN_SANM) {
    // get_ABEFGH depends on sigr, D and the node sizes only
    NodalParams P = nodal_params(h, 1);
    CK(launch_sanm_consts(P, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  h->xs_set = true;
  return ADP_OK;
}

adp_status adp_set_xs(adp_handle* h, int nmat, const double* D, const double* sigr, const double* nuf,
                      const double* sigf, const double* chi, const int* mat, const double* sigs, const double* dc) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!D || !sigr) return fail(h, ADP_ERR_INPUT, "adp_set_xs: null D or sigr");
  const size_t q = (size_t)h->ng * h->nnod;
  for (size_t k = 0; k < q; ++k) {
    if (D[k] < (double)1.e-20f) return fail(h, ADP_ERR_BADXS, "diffusion coef. is close to zero or negative");
    if (sigr[k] < 0.) return fail(h, ADP_ERR_BADXS, "removal xs is negative");
  }
  Xfer X;
  bool chi_neg = false;
  adp_status s = upload_xs_common(h, nmat, nuf, sigf, chi, mat, sigs, dc, X, chi_neg);
  if (s != ADP_OK) return s;
  if ((s = put_nodes(h, X, D, h->ng, 1, h->d_D, h->NB, 0)) != ADP_OK) return s;
  if ((s = put_nodes(h, X, sigr, h->ng, 1, h->d_sigr, h->NB, 0)) != ADP_OK) return s;
  if ((s = xs_flags(h, X, chi_neg)) != ADP_OK) return s;
  return after_xs(h);
}

// Dsigr_updt and check_xs on the device (mod_xsec.f90:90-168, :198-227) for
// the node tables in place, then the derived copies (after_xs).
static adp_status xs_finish(adp_handle* h) {
  h->h_ctl->status = 0;
  h->h_ctl->err_node = -1;
  CK(cudaMemcpyAsync(&h->d_ctl->status, &h->h_ctl->status, sizeof(int), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(&h->d_ctl->err_node, &h->h_ctl->err_node, sizeof(int), cudaMemcpyHostToDevice, h->st));
  CK(launch_xs_updt(box_geom(h), h->ng, h->d_act, h->nnod, h->d_sigtr, h->d_siga, h->d_sigs, h->d_D, h->d_sigr,
                    h->d_ctl, h->st));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (h->h_ctl->status != 0) {
    int code = h->h_ctl->status;
    h->h_ctl->status = 0;
    CK(cudaMemcpyAsync(&h->d_ctl->status, &h->h_ctl->status, sizeof(int), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return fail(h, (adp_status)code, "cross-section check failed (sigtr < 1e-5, D < 1e-20 or sigr < 0)");
  }
  return after_xs(h);
}

adp_status adp_xs_updt_nodes(adp_handle* h, int nmat, const double* sigtr, const double* siga, const double* nuf,
                             const double* sigf, const double* chi, const int* mat, const double* sigs,
                             const double* dc) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!sigtr || !siga) return fail(h, ADP_ERR_INPUT, "adp_xs_updt: null sigtr or siga");
  Xfer X;
  bool chi_neg = false;
  adp_status s = upload_xs_common(h, nmat, nuf, sigf, chi, mat, sigs, dc, X, chi_neg);
  if (s != ADP_OK) return s;
  if ((s = put_nodes(h, X, sigtr, h->ng, 1, h->d_sigtr, h->NB, 0)) != ADP_OK) return s;
  if ((s = put_nodes(h, X, siga, h->ng, 1, h->d_siga, h->NB, 0)) != ADP_OK) return s;
  if ((s = xs_flags(h, X, chi_neg)) != ADP_OK) return s;
  return xs_finish(h);
}

// base_updt (mod_xsec.f90:172-195) on the device: only the material tables
// and numbers (and the ADFs) cross to the GPU.
adp_status adp_xs_updt(adp_handle* h, int nmat, const double* xsigtr, const double* xsiga, const double* xnuf,
                       const double* xsigf, const double* chi, const int* mat, const double* xsigs, const double* dc) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!xsigtr || !xsiga || !xnuf || !xsigf || !xsigs || !mat || !chi)
    return fail(h, ADP_ERR_INPUT, "adp_xs_updt: null array");
  if (nmat < 1) return fail(h, ADP_ERR_INPUT, "adp_xs_updt: no materials");
  const int nn = h->nnod, G = h->ng;
  h->fwd_ok = false;
  adp_status s = check_mat(h, nmat, mat);
  if (s != ADP_OK) return s;
  const bool chi_neg = chi_negative(h, nmat, chi);
  Xfer X;
  if ((s = xfer_reserve(h, nmat, X)) != ADP_OK) return s;
  const size_t t1 = (size_t)G * nmat;
  CK(cudaMemsetAsync(X.flags, 0, sizeof(int), h->st));
  CK(cudaMemcpyAsync(X.mat, mat, (size_t)nn * 4, cudaMemcpyHostToDevice, h->st));
  const double* src[5] = {xsigtr, xsiga, xnuf, xsigf, chi};
  for (int k = 0; k < 5; ++k) CK(cudaMemcpyAsync(X.tab + k * t1, src[k], t1 * 8, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(X.tab + 5 * t1, xsigs, t1 * G * 8, cudaMemcpyHostToDevice, h->st));
  XsTables T{X.tab, X.tab + t1, X.tab + 2 * t1, X.tab + 3 * t1, X.tab + 4 * t1, X.tab + 5 * t1};
  CK(launch_base_updt(T, X.mat, h->d_act, nn, nmat, G, h->NB, xs_box(h), X.flags, h->st));
  if ((s = put_dc(h, X, dc)) != ADP_OK) return s;
  h->nmat = nmat;
  if ((s = xs_flags(h, X, chi_neg)) != ADP_OK) return s;
  return xs_finish(h);
}

// Feedback tables (mod_xsec.f90:11-46 with its state and rod cards) resident
// on the device: base set, nst change sets, the rod set, the working set,
// chi, material and bank numbers in one allocation.
adp_status adp_fb_set(adp_handle* h, const adp_fb_tables* t) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  h->fb_ready = false;
  if (!t) return fail(h, ADP_ERR_INPUT, "adp_fb_set: null tables");
  const int nn = h->nnod, G = h->ng, nmat = t->nmat;
  if (nmat < 1 || !t->xsigtr || !t->xsiga || !t->xnuf || !t->xsigf || !t->xsigs || !t->chi || !t->mat)
    return fail(h, ADP_ERR_INPUT, "adp_fb_set: null base table or no materials");
  if (t->nstate < 0 || t->nstate > ADP_FB_MAX_STATE || (t->nstate > 0 && (!t->kind || !t->ref || !t->dsig)))
    return fail(h, ADP_ERR_INPUT, "adp_fb_set: 0..4 state cards with kinds, references and change tables");
  if (t->nbank < 0 || t->nbank > ADP_FB_MAX_BANKS || (t->nbank > 0 && (!t->rsig || !t->bank)))
    return fail(h, ADP_ERR_INPUT, "adp_fb_set: 0..64 rod banks with change tables and the bank map");
  for (int s = 0; s < t->nstate; ++s) {
    if (t->kind[s] < ADP_FB_BORON || t->kind[s] > ADP_FB_COOL_DENS)
      return fail(h, ADP_ERR_INPUT, "adp_fb_set: unknown state kind");
    if (t->kind[s] == ADP_FB_FUEL_TEMP && !(t->ref[s] >= 0.0))
      return fail(h, ADP_ERR_INPUT, "adp_fb_set: negative reference fuel temperature");
    for (int q = 0; q < 5; ++q)
      if (!t->dsig[5 * s + q]) return fail(h, ADP_ERR_INPUT, "adp_fb_set: null state change table");
  }
  for (int q = 0; q < 5 && t->nbank > 0; ++q)
    if (!t->rsig[q]) return fail(h, ADP_ERR_INPUT, "adp_fb_set: null rod change table");
  adp_status s = check_mat(h, nmat, t->mat);
  if (s != ADP_OK) return s;
  if (t->nbank > 0)
    for (int n = 0; n < nn; ++n)
      if (t->bank[n] < 0 || t->bank[n] > t->nbank) return fail(h, ADP_ERR_INPUT, "adp_fb_set: bank number out of range");
  const size_t t1 = (size_t)G * nmat, tq = 4 * t1 + t1 * G;
  const size_t nsets = 2 + (size_t)t->nstate + (t->nbank > 0 ? 1 : 0);   // base, work, states, rods
  size_t need = 0;
  auto add = [&](size_t b) { need += ((b + 255) & ~(size_t)255) + 256; };
  add(nsets * tq * 8);
  add(t1 * 8);
  add((size_t)nn * 4);
  add((size_t)nn * 4);
  if (h->fb_size < need) {
    if (h->fb_base) CK(cudaFree(h->fb_base));
    h->fb_base = nullptr;
    h->fb_size = 0;
    CK(cudaMalloc((void**)&h->fb_base, need));
    h->fb_size = need;
  }
  DevArena A;
  A.base = h->fb_base;
  A.size = h->fb_size;
  double* sets = (double*)A.take(nsets * tq * 8);
  h->d_fb_base = sets;
  h->d_fb_tab = sets + tq;
  h->d_fb_dsig = sets + 2 * tq;
  h->d_fb_rsig = t->nbank > 0 ? sets + (2 + (size_t)t->nstate) * tq : nullptr;
  h->d_fb_chi = (double*)A.take(t1 * 8);
  h->d_fb_mat = (int*)A.take((size_t)nn * 4);
  h->d_fb_bank = (int*)A.take((size_t)nn * 4);
  auto put_set = [&](double* dst, const double* const* src) -> cudaError_t {
    for (int q = 0; q < 4; ++q) {
      cudaError_t e = cudaMemcpyAsync(dst + q * t1, src[q], t1 * 8, cudaMemcpyHostToDevice, h->st);
      if (e != cudaSuccess) return e;
    }
    return cudaMemcpyAsync(dst + 4 * t1, src[4], t1 * G * 8, cudaMemcpyHostToDevice, h->st);
  };
  const double* base[5] = {t->xsigtr, t->xsiga, t->xnuf, t->xsigf, t->xsigs};
  CK(put_set(h->d_fb_base, base));
  for (int k = 0; k < t->nstate; ++k) CK(put_set(h->d_fb_dsig + k * tq, t->dsig + 5 * k));
  if (t->nbank > 0) CK(put_set(h->d_fb_rsig, t->rsig));
  CK(cudaMemcpyAsync(h->d_fb_chi, t->chi, t1 * 8, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_fb_mat, t->mat, (size_t)nn * 4, cudaMemcpyHostToDevice, h->st));
  if (t->nbank > 0) CK(cudaMemcpyAsync(h->d_fb_bank, t->bank, (size_t)nn * 4, cudaMemcpyHostToDevice, h->st));
  else CK(cudaMemsetAsync(h->d_fb_bank, 0, (size_t)nn * 4, h->st));
  Xfer X;
  if ((s = xfer_reserve(h, nmat, X)) != ADP_OK) return s;
  if ((s = put_dc(h, X, t->dc)) != ADP_OK) return s;
  CK(cudaStreamSynchronize(h->st));
  h->fb_chi_neg = chi_negative(h, nmat, t->chi);
  h->fb_nmat = nmat;
  h->fb_nst = t->nstate;
  h->fb_nb = t->nbank;
  for (int k = 0; k < t->nstate; ++k) {
    h->fb_kind[k] = t->kind[k];
    h->fb_ref[k] = t->ref[k];
  }
  h->fb_coreh = t->coreh;
  h->fb_pos0 = t->pos0;
  h->fb_ssize = t->ssize;
  h->fb_ready = true;
  return ADP_OK;
}

// crod_updt (mod_xsec.f90:239-263): the rod tip of each bank, walking down
// from the top of the core; the plane holding it and its rodded fraction
// (no plane holds it: every plane of the bank's columns is fully rodded).
// The product is held apart so that it is rounded on its own, as the
// reference's is, whether or not the host compiler contracts a - b * c.
adp_status adp_fb_rod_tips(int nzz, const double* zdel, double coreh, double pos0, double ssize, int nbank,
                           const double* bpos, int* tip, double* vf) {
  if (nzz < 1 || nbank < 0 || !zdel || (nbank > 0 && (!bpos || !tip || !vf))) return ADP_ERR_INPUT;
  for (int b = 0; b < nbank; ++b) {
    volatile double step = bpos[b] * ssize;
    const double rodh = (coreh - pos0) - step;
    double dum = 0.0;
    tip[b] = -1;
    vf[b] = 0.0;
    for (int k = nzz - 1; k >= 0; --k) {
      if (rodh >= dum && rodh <= dum + zdel[k]) {
        tip[b] = k;
        vf[b] = (rodh - dum) / zdel[k];
        break;
      }
      dum = dum + zdel[k];
    }
  }
  return ADP_OK;
}

adp_status adp_fb_updt(adp_handle* h, const double* state, const double* bpos) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!h->fb_ready) return fail(h, ADP_ERR_STATE, "adp_fb_updt: no feedback tables (adp_fb_set)");
  if ((h->fb_nst > 0 && !state) || (h->fb_nb > 0 && !bpos)) return fail(h, ADP_ERR_INPUT, "adp_fb_updt: null state or bank positions");
  for (int k = 0; k < h->fb_nst; ++k) {
    if (!std::isfinite(state[k])) return fail(h, ADP_ERR_INPUT, "adp_fb_updt: non-finite state value");
    if (h->fb_kind[k] == ADP_FB_FUEL_TEMP && state[k] < 0.0)
      return fail(h, ADP_ERR_INPUT, "adp_fb_updt: negative fuel temperature");
  }
  for (int b = 0; b < h->fb_nb; ++b)
    if (!std::isfinite(bpos[b])) return fail(h, ADP_ERR_INPUT, "adp_fb_updt: non-finite bank position");
  const int G = h->ng, nmat = h->fb_nmat;
  const long long t1 = (long long)G * nmat;
  FbParams P;
  std::memset(&P, 0, sizeof P);
  P.nmat = nmat;
  P.G = G;
  P.nn = h->nnod;
  P.nst = h->fb_nst;
  P.nb = h->fb_nb;
  P.plane = h->plane;
  P.NB = h->NB;
  P.tq = 4 * t1 + t1 * G;
  for (int q = 0; q < 5; ++q) P.off[q] = q * t1;
  P.base = h->d_fb_base;
  P.dsig = h->d_fb_dsig;
  P.rsig = h->d_fb_rsig;
  P.tab = h->d_fb_tab;
  P.chi = h->d_fb_chi;
  P.mat = h->d_fb_mat;
  P.bank = h->d_fb_bank;
  P.act = h->d_act;
  // the state changes of bcon_updt, ftem_updt (square roots), mtem_updt, cden_updt
  for (int k = 0; k < h->fb_nst; ++k)
    P.dv[k] = h->fb_kind[k] == ADP_FB_FUEL_TEMP ? std::sqrt(state[k]) - std::sqrt(h->fb_ref[k]) : state[k] - h->fb_ref[k];
  if (h->fb_nb > 0)
    adp_fb_rod_tips(h->nzz, h->zdel.data(), h->fb_coreh, h->fb_pos0, h->fb_ssize, h->fb_nb, bpos, P.tip, P.vf);
  Xfer X;
  adp_status s = xfer_reserve(h, nmat, X);
  if (s != ADP_OK) return s;
  h->fwd_ok = false;
  CK(cudaMemsetAsync(X.flags, 0, sizeof(int), h->st));
  P.X = xs_box(h);
  P.flags = X.flags;
  CK(launch_fb_updt(P, h->st));
  h->nmat = nmat;
  if ((s = xs_flags(h, X, h->fb_chi_neg)) != ADP_OK) return s;
  return xs_finish(h);
}

}  // extern "C"

OuterParams adp::outer_params(adp_handle* h, int adj) {
  OuterParams P;
  std::memset(&P, 0, sizeof P);
  P.G = box_geom(h);
  P.ng = h->ng;
  P.nin = h->o.nin;
  P.nac = h->o.nac;
  P.nupd = h->o.nupd;
  P.nout = h->o.nout;
  P.adj = adj;
  P.mixed = h->o.precision == ADP_MIXED;
  P.serc = h->o.serc;
  P.ferc = h->o.ferc;
  P.NBH = h->NBH;
  P.A = h->d_A;
  P.A32 = h->d_A32;
  for (int t = 0; t < 2; ++t) {
    P.phi[t] = h->d_phi[t];
    P.fs[t] = h->d_fs[t];
    P.pv2[t] = h->d_pv2[t];
    P.pv2f[t] = h->d_pv2f[t];
  }
  P.wsrc = adj ? h->d_nuf : h->d_chin;
  P.src_nz = adj ? h->nuf_nz : h->chi_nz;
  P.sc_nz = h->sigs_nz;
  P.wfis = adj ? h->d_chin : h->d_nuf;
  P.sigs = h->d_sigs;
  P.r = h->d_r;
  P.rs = h->d_rs;
  P.st2 = h->d_st2;
  P.r32 = h->d_r32;
  P.rs32 = h->d_rs32;
  P.st2f = h->d_st2f;
  P.red = h->d_red;
  P.A2 = h->d_A2;
  for (int t = 0; t < 2; ++t) {
    P.x2[t] = h->d_x2[t];
    P.fs2[t] = h->d_fs2[t];
  }
  P.wsrc2 = adj ? h->d_nuf2 : h->d_chin2;
  P.wfis2 = adj ? h->d_chin2 : h->d_nuf2;
  P.sigs2 = h->d_sigs2;
  P.vdel2 = h->d_vdel2;
  P.ctl = h->d_ctl;
  P.tr_k = h->d_tr_k;
  P.tr_ser = h->d_tr_ser;
  P.tr_fer = h->d_tr_fer;
  P.tr_flags = h->d_tr_flags;
  P.tr_ndmax = h->d_tr_ndmax;
  return P;
}

extern "C" {

// Launch shape of the persistent kernel: at most one block per SM (more
// co-resident blocks only add barrier participants), and a block count that
// gives every thread the same number of rows, so no block waits at a grid
// barrier for blocks holding one row more.  Automatic threads per block:
// 512, or 256 when 512-thread blocks of one row per thread would leave more
// than half of the SMs idle.  A small core then spreads over twice the SMs;
// the FP64 path, bound by each SM's FP64 issue rate, gains most (on a
// 25,432-node two-group core: 98 -> 75 us per outer FP64, 55 -> 52 mixed;
// 128-thread blocks were slower again).
static void launch_shape(adp_handle* h, int& blocks, int& threads) {
  threads = h->launch_threads;
  if (threads <= 0) threads = ((long long)h->NB + 511) / 512 < h->sms / 2 ? 256 : 512;
  int occ = outer_max_blocks_per_sm(threads, h->o.precision == ADP_MIXED);
  if (occ < 1) occ = 1;
  const int cap = std::min(h->sms * occ, kMaxBlocks);
  if (h->launch_blocks > 0) {
    blocks = std::min(h->launch_blocks, cap);
    return;
  }
  const long long NB = h->NB;
  const long long full = (long long)std::min(cap, h->sms) * threads;
  const long long rows = std::max(1LL, (NB + full - 1) / full);       // rows per thread
  blocks = (int)std::max(1LL, (NB + rows * threads - 1) / (rows * threads));
  blocks = std::min(blocks, cap);
}

static adp_status ctl_error(adp_handle* h, const OuterCtl& c) {
  char buf[256];
  int b = c.err_node;
  int i = b >= 0 ? b % h->nxx + 1 : 0, j = b >= 0 ? (b / h->nxx) % h->nyy + 1 : 0, k = b >= 0 ? b / h->plane + 1 : 0;
  switch (c.status) {
    case ADP_ERR_PIVOT:
      std::snprintf(buf, sizeof buf, "error in matrix decomp: diagonal elements close to zero at I = %d, J = %d, K = %d", i, j, k);
      break;
    case ADP_ERR_DIVERGED:
      std::snprintf(buf, sizeof buf, "max. change in nodal coupling coefficient = %.1f: the two-node nonlinear iteration seems not stable", c.ndmax);
      break;
    case ADP_ERR_BREAKDOWN: std::snprintf(buf, sizeof buf, "BiCGSTAB breakdown (a zero inner product) at outer %d", c.p); break;
    case ADP_ERR_NAN: std::snprintf(buf, sizeof buf, "non-finite eigenvalue or fission source at outer %d", c.p); break;
    case ADP_ERR_TIMEOUT: std::snprintf(buf, sizeof buf, "a grid barrier wait ran out of time"); break;
    case ADP_ERR_ZEROPOWER: std::snprintf(buf, sizeof buf, "total nodes power is zero or less"); break;
    case ADP_ERR_BOUNDS:
      std::snprintf(buf, sizeof buf, "device index out of range (range-checked build) at box row %d", c.err_node);
      break;
    default: std::snprintf(buf, sizeof buf, "device error %d", c.status);
  }
  return fail(h, (adp_status)c.status, buf);
}

adp_status adp_set_launch(adp_handle* h, int blocks, int threads) {
  if (!h) return ADP_ERR_INPUT;
  if (threads != 0 && (threads < 64 || threads > 1024 || threads % 32)) return fail(h, ADP_ERR_INPUT, "threads must be 64..1024, a multiple of 32");
  if (blocks < 0 || blocks > kMaxBlocks) return fail(h, ADP_ERR_INPUT, "blocks out of range");
  h->launch_blocks = blocks;
  h->launch_threads = threads;
  return ADP_OK;
}

adp_status adp_set_wait_limit(adp_handle* h, double seconds) {
  if (!h) return ADP_ERR_INPUT;
  if (!(seconds >= 0.0) || seconds > 60.0) return fail(h, ADP_ERR_INPUT, "adp_set_wait_limit: seconds must be in [0, 60]");
  h->wait_ns = (unsigned long long)(seconds * 1e9);
  return ADP_OK;
}

adp_status adp_test_missing_block(adp_handle* h, int on) {
  if (!h) return ADP_ERR_INPUT;
  h->phantom = on ? 1 : 0;
  return ADP_OK;
}

adp_status adp_outer(adp_handle* h, int mode, int popt, adp_report* rep) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!h->xs_set) return fail(h, ADP_ERR_STATE, "adp_outer: cross sections not set");
  if (mode & ~(ADP_ADJOINT | ADP_FROZEN_DN)) return fail(h, ADP_ERR_INPUT, "adp_outer: bad mode");
  const bool frozen = (mode & ADP_FROZEN_DN) != 0;
  mode &= ADP_ADJOINT;
  const int adj = mode == ADP_ADJOINT;
  h->fwd_ok = false;
  CK(cudaEventRecord(h->e0, h->st));
  // matrix_setup(1): coupling coefficients + assembly
  AssembleParams AP;
  AP.G = box_geom(h);
  AP.ng = h->ng;
  AP.with_coupling = 1;
  AP.D = h->d_D;
  AP.sigr = h->d_sigr;
  AP.df = h->d_df;
  AP.dn = h->d_dn;
  AP.A = h->d_A;
  AP.A32 = h->d_A32;
  AP.A2 = h->d_A2;
  AP.ctl = h->d_ctl;
  CK(launch_assemble(AP, h->st));
  OuterParams P = outer_params(h, adj);
  // first-call start (mod_cmfd.f90:448-454 / :635-641)
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  OuterCtl c = *h->h_ctl;
  if (!h->started[mode] && (!adj || popt > 0)) {
    CK(launch_init_flux(P, h->st));
    c.Ke = 1.0;
    c.cur = 0;
    h->started[mode] = true;
  } else if (!h->started[0] && !h->started[1]) {
    return fail(h, ADP_ERR_STATE, "adp_outer: no flux to start from (adjoint with popt <= 0 before any solve)");
  }
  c.p = 0;
  c.status = 0;
  c.converged = 0;
  c.nodal_due = 0;
  c.max_reached = 0;
  c.need_prologue = 1;
  c.err_node = -1;
  c.bar_count = 0;
  c.wait_ns = h->wait_ns;
  if (frozen) c.ndmax = 0.0;
  const int nod0 = c.nodal_updates;
  const long outers0 = c.p_total;
  *h->h_ctl = c;
  CK(cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(OuterCtl), cudaMemcpyHostToDevice, h->st));
  const int do_nodal = !frozen && (h->o.kern != ADP_KERN_FDM) && (!adj || popt > 0);
  P.do_nodal = do_nodal;
  P.phantom = h->phantom;
  NodalParams NP = nodal_params(h, adj ? 0 : (h->trans_on ? 2 : 1));
  if (h->trans_on) {
    // outer_tr (mod_cmfd.f90:800-868): the step's source weights and
    // external source, no eigenvalue update; on the mixed path both as
    // (hi, lo) pairs for the double-float defect (the kernel of the
    // generalized adjoint's fixed-eigenvalue mode, here forward)
    P.trans = 1;
    P.wsrc = h->d_wtr;
    P.exsrc = h->d_exsrc;
    if (P.mixed) {
      const long long gn = (long long)h->ng * h->NB;
      CK(launch_split(h->d_wtr, h->d_wtr2, gn, h->st));
      CK(launch_split(h->d_exsrc, h->d_exsrc2, gn, h->st));
      P.wsrc2 = h->d_wtr2;
      P.exsrc2 = h->d_exsrc2;
    }
  }
  int blocks, threads;
  launch_shape(h, blocks, threads);
  P.smem_rows = outer_smem_rows(h->NB, blocks, threads, P.mixed);
  h->tm.grid_blocks = blocks;
  h->tm.block_threads = threads;
  adp_status result = ADP_OK;
  Range r_call(adj ? "adp_outer adjoint" : (h->trans_on ? "adp_outer transient" : "adp_outer"));
  for (int guard = 0; guard < 4 * h->o.nout + 8; ++guard) {
    Range r_cmfd("CMFD outers");
    CK(cudaMemsetAsync(&h->d_ctl->bar_count, 0, sizeof(unsigned), h->st));
    CK(cudaEventRecord(h->e2, h->st));
    CK(launch_outer(P, blocks, threads, h->st));
    CK(cudaEventRecord(h->e3, h->st));
    CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->e2, h->e3);
    h->tm.outer_kernel_ms += ms;
    h->tm.outer_kernel_launches += 1;
    c = *h->h_ctl;
    if (c.status) { result = ctl_error(h, c); break; }
    if (c.converged) break;
    if (c.max_reached) {
      // outer_tr only flags it (maxi, mod_cmfd.f90:861-865)
      if (!h->trans_on) result = fail(h, ADP_ERR_MAXOUTER, "maximum number of outer iteration is reached");
      break;
    }
    if (c.nodal_due) {
      Range r_nodal("nodal update");
      CK(cudaEventRecord(h->e2, h->st));
      CK(launch_nodal(NP, h->st));
      AssembleParams A0 = AP;
      A0.with_coupling = 0;
      CK(launch_assemble(A0, h->st));
      CK(cudaEventRecord(h->e3, h->st));
      CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      ms = 0.f;
      cudaEventElapsedTime(&ms, h->e2, h->e3);
      h->tm.nodal_ms += ms;
      h->tm.nodal_updates += 1;
      c = *h->h_ctl;
      if (c.status) { result = ctl_error(h, c); break; }
      if (c.converged) break;
      if (c.max_reached) {
        if (!h->trans_on) result = fail(h, ADP_ERR_MAXOUTER, "maximum number of outer iteration is reached");
        break;
      }
    }
  }
  CK(cudaEventRecord(h->e1, h->st));
  CK(cudaEventSynchronize(h->e1));
  float total_ms = 0.f;
  cudaEventElapsedTime(&total_ms, h->e0, h->e1);
  h->tm.outers += c.p;
  h->tm.bicg_rows += (long)c.p * h->ng * h->o.nin * (long)h->NB;
  if (rep) {
    rep->outers = c.p;
    rep->converged = c.converged;
    rep->nodal_updates = c.nodal_updates - nod0;
    rep->keff = c.Ke;
    rep->ser = c.ser;
    rep->fer = c.fer;
    rep->ndmax = c.ndmax;
    rep->im = c.im;
    rep->jm = c.jm;
    rep->km = c.km;
    rep->device_ms = total_ms;
    int n = std::min(std::min(c.p, rep->trace_cap), h->o.nout);
    if (n > 0) {
      if (rep->trace_k) CK(cudaMemcpy(rep->trace_k, h->d_tr_k, n * 8, cudaMemcpyDeviceToHost));
      if (rep->trace_ser) CK(cudaMemcpy(rep->trace_ser, h->d_tr_ser, n * 8, cudaMemcpyDeviceToHost));
      if (rep->trace_fer) CK(cudaMemcpy(rep->trace_fer, h->d_tr_fer, n * 8, cudaMemcpyDeviceToHost));
      if (rep->trace_flags) CK(cudaMemcpy(rep->trace_flags, h->d_tr_flags, n * 4, cudaMemcpyDeviceToHost));
      if (rep->trace_ndmax) CK(cudaMemcpy(rep->trace_ndmax, h->d_tr_ndmax, n * 8, cudaMemcpyDeviceToHost));
    }
  }
  (void)outers0;
  h->fwd_ok = !adj && result == ADP_OK && c.converged;
  return result;
}

adp_status adp_get_state(adp_handle* h, double* f0, double* fs0, double* keff, double* dn) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const int cur = h->h_ctl->cur, G = h->ng, NB = h->NB;
  if (keff) *keff = h->h_ctl->Ke;
  if (!f0 && !fs0 && !dn) return ADP_OK;
  Xfer X;
  adp_status s = xfer_reserve(h, h->nmat, X);
  if (s != ADP_OK) return s;
  // gathered on the device; one contiguous copy per array
  if (f0 && (s = get_nodes(h, X, h->d_phi[cur], G, 1, h->NBH, f0)) != ADP_OK) return s;
  if (fs0 && (s = get_nodes(h, X, h->d_fs[cur], 1, 1, NB, fs0)) != ADP_OK) return s;
  // dn(nnod, ng, 6): face is the slowest index
  if (dn && (s = get_nodes(h, X, h->d_dn, G, 6, NB, dn)) != ADP_OK) return s;
  return ADP_OK;
}

adp_status adp_set_state(adp_handle* h, const double* f0, const double* fs0, const double* keff, const double* dn) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const int cur = h->h_ctl->cur, nn = h->nnod, G = h->ng, NB = h->NB;
  std::vector<double> box;
  if (f0) {
    box.assign((size_t)G * h->NBH, 0.0);
    for (int g = 0; g < G; ++g)
      for (int n = 0; n < nn; ++n) box[(size_t)g * h->NBH + h->plane + h->node2box[n]] = f0[(size_t)g * nn + n];
    CK(cudaMemcpy(h->d_phi[cur] - h->plane, box.data(), box.size() * 8, cudaMemcpyHostToDevice));
  }
  if (fs0) {
    box.assign(NB, 0.0);
    for (int n = 0; n < nn; ++n) box[h->node2box[n]] = fs0[n];
    CK(cudaMemcpy(h->d_fs[cur], box.data(), (size_t)NB * 8, cudaMemcpyHostToDevice));
  }
  if (dn) {
    box.assign((size_t)G * 6 * NB, 0.0);
    for (int u = 0; u < 6; ++u)
      for (int g = 0; g < G; ++g)
        for (int n = 0; n < nn; ++n)
          box[((size_t)g * 6 + u) * NB + h->node2box[n]] = dn[((size_t)u * G + g) * nn + n];
    CK(cudaMemcpy(h->d_dn, box.data(), box.size() * 8, cudaMemcpyHostToDevice));
  }
  if (keff) {
    h->h_ctl->Ke = *keff;
    CK(cudaMemcpy(&h->d_ctl->Ke, &h->h_ctl->Ke, sizeof(double), cudaMemcpyHostToDevice));
  }
  h->started[0] = h->started[1] = true;
  h->fwd_ok = false;
  return ADP_OK;
}

adp_status adp_reset(adp_handle* h) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemsetAsync(h->d_dn, 0, (size_t)h->ng * 6 * h->NB * sizeof(double), h->st));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  OuterCtl c = *h->h_ctl;
  c.Ke = 1.0;
  c.ndmax = 0.0;
  c.im = c.jm = c.km = 0;
  c.cur = 0;
  c.status = 0;
  c.converged = c.nodal_due = c.max_reached = 0;
  c.err_node = -1;
  *h->h_ctl = c;
  CK(cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(OuterCtl), cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->started[0] = h->started[1] = false;
  h->fwd_ok = false;
  return ADP_OK;
}

adp_status adp_power(adp_handle* h, double* p) {
  if (!h || !p) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  OuterCtl c = *h->h_ctl;
  c.status = 0;
  *h->h_ctl = c;
  CK(cudaMemcpyAsync(&h->d_ctl->status, &h->h_ctl->status, sizeof(int), cudaMemcpyHostToDevice, h->st));
  CK(launch_power(box_geom(h), h->ng, h->NBH, h->d_phi[c.cur], h->d_sigf, h->d_pbox, h->d_red, h->d_ctl, h->st));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (h->h_ctl->status) return ctl_error(h, *h->h_ctl);
  Xfer X;
  adp_status s = xfer_reserve(h, h->nmat, X);
  if (s != ADP_OK) return s;
  return get_nodes(h, X, h->d_pbox, 1, 1, h->NB, p);
}

// Device state of the discrete adjoint, allocated once per handle.
static SensParams sens_params(adp_handle* h, double keff, const double* phi, const double* w) {
  SensParams S;
  S.G = box_geom(h);
  S.ng = h->ng;
  S.nnod = h->nnod;
  S.NBH = h->NBH;
  S.keff = keff;
  S.act = h->d_act;
  S.phi = phi;
  S.psi = w;
  S.D = h->d_D;
  S.nuf = h->d_nuf;
  S.chin = h->d_chin;
  return S;
}

static adp_status adj_alloc(adp_handle* h) {
  if (h->adj_base) return ADP_OK;
  const size_t NB = h->NB, G = h->ng, NBH = h->NBH, nn = h->nnod;
  const bool mixed = h->o.precision == ADP_MIXED;
  size_t bytes = 0;
  auto add = [&](size_t b) { bytes += ((b + 255) & ~(size_t)255) + 256; };
  add(G * 7 * NB * 8);
  if (mixed) {
    add(G * 7 * NB * 4);
    add(G * 7 * NB * 8);
  }
  add(G * NBH * 8 * 2);
  add(NB * 8 * 2);
  add(sizeof(OuterCtl));
  add(nn * G * (4 + G) * 8);
  add(kMaxBlocks * 8);
  DevArena A;
  A.size = bytes;
  CK(cudaMalloc((void**)&A.base, bytes));
  h->adj_base = A.base;
  h->d_AT = (double*)A.take(G * 7 * NB * 8);
  if (mixed) {
    h->d_AT32 = (float*)A.take(G * 7 * NB * 4);
    h->d_AT2 = (float2*)A.take(G * 7 * NB * 8);
  }
  for (int t = 0; t < 2; ++t) h->d_psi[t] = (double*)A.take(G * NBH * 8) + h->plane;
  for (int t = 0; t < 2; ++t) h->d_fsa[t] = (double*)A.take(NB * 8);
  h->d_ctla = (OuterCtl*)A.take(sizeof(OuterCtl));
  h->d_sens = (double*)A.take(nn * G * (4 + G) * 8);
  h->d_spart = (double*)A.take(kMaxBlocks * 8);
  if (A.used > A.size) return fail(h, ADP_ERR_CUDA, "internal: adjoint arena overflow");
  CK(cudaMemsetAsync(A.base, 0, A.size, h->st));   // halos and inactive positions stay 0
  CK(cudaStreamSynchronize(h->st));
  return ADP_OK;
}

// The adjoint eigen-solve at frozen dn and the frozen-dn derivative into
// d_sens.  fwd: the forward control block; c: the adjoint's.
static adp_status adjoint_frozen(adp_handle* h, double tol, OuterCtl& fwd, OuterCtl& c) {
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  fwd = *h->h_ctl;
  // A^T of the converged forward matrix (dn frozen)
  CK(launch_transpose(box_geom(h), h->ng, h->d_A, h->d_AT, h->d_AT32, h->d_AT2, h->st));
  OuterParams P = outer_params(h, 1);
  P.A = h->d_AT;
  P.A32 = h->d_AT32;
  P.A2 = h->d_AT2;
  for (int t = 0; t < 2; ++t) {
    P.phi[t] = h->d_psi[t];
    P.fs[t] = h->d_fsa[t];
  }
  P.ctl = h->d_ctla;
  P.do_nodal = 0;
  if (tol > 0) P.serc = P.ferc = tol;
  // Warm start: the converged forward flux and eigenvalue (A^T has the
  // eigenvalue of A, and the forward flux, positive, overlaps the
  // fundamental adjoint mode)
  P.init_phi = h->d_phi[fwd.cur];
  CK(launch_init_flux(P, h->st));
  P.init_phi = nullptr;
  std::memset(&c, 0, sizeof c);
  c.Ke = fwd.Ke;
  c.need_prologue = 1;
  c.err_node = -1;
  c.wait_ns = h->wait_ns;
  *h->h_ctl = c;
  CK(cudaMemcpyAsync(h->d_ctla, h->h_ctl, sizeof(OuterCtl), cudaMemcpyHostToDevice, h->st));
  int blocks, threads;
  launch_shape(h, blocks, threads);
  P.smem_rows = outer_smem_rows(h->NB, blocks, threads, P.mixed);
  adp_status result = ADP_OK;
  Range r_adj("adjoint eigen-solve");
  for (int guard = 0; guard < 4 * h->o.nout + 8; ++guard) {
    CK(cudaMemsetAsync(&h->d_ctla->bar_count, 0, sizeof(unsigned), h->st));
    CK(launch_outer(P, blocks, threads, h->st));
    CK(cudaMemcpyAsync(h->h_ctl, h->d_ctla, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    c = *h->h_ctl;
    if (c.status) { result = ctl_error(h, c); break; }
    if (c.converged) break;
    if (c.max_reached) {
      result = fail(h, ADP_ERR_MAXOUTER, "adp_adjoint_sens: the adjoint solve reached nout outers without convergence");
      break;
    }
  }
  if (result == ADP_OK && !c.converged)
    result = fail(h, ADP_ERR_MAXOUTER, "adp_adjoint_sens: the adjoint solve did not converge");
  if (result != ADP_OK) return result;
  SensParams S = sens_params(h, fwd.Ke, h->d_phi[fwd.cur], h->d_psi[c.cur]);
  CK(launch_sens(S, h->d_spart, h->d_sens, h->st));
  return ADP_OK;
}

static adp_status nadj_alloc(adp_handle* h) {
  if (h->nadj_base) return ADP_OK;
  const size_t NB = h->NB, G = h->ng, NBH = h->NBH, nn = h->nnod;
  const size_t face = G * 6 * NB * 8, sens = nn * G * (4 + G) * 8;
  const size_t pieces[] = {nadj_side_doubles(h->ng, h->NB) * 8, nadj_nodeu_doubles(h->ng, h->NB) * 8,
                           3 * G * NB * 8, face, face, G * NB * 8, face, face, face, kMaxBlocks * 8, kMaxBlocks * 8,
                           4 * 8, sens, sens, G * NBH * 8, G * NBH * 8, NB * 8, NB * 8, G * NB * 8, G * NB * 8,
                           2 * kMaxBlocks * 8, 2 * kMaxBlocks * 8, sizeof(OuterCtl), G * NB * 8, G * NB * 8, face};
  size_t bytes = 0;
  for (size_t b : pieces) bytes += ((b + 255) & ~(size_t)255) + 256;
  DevArena A;
  A.size = bytes;
  CK(cudaMalloc((void**)&A.base, bytes));
  h->nadj_base = A.base;
  int i = 0;
  h->d_nside = (double*)A.take(pieces[i++]);
  h->d_nnodeu = (double*)A.take(pieces[i++]);
  h->d_nLbar = (double*)A.take(pieces[i++]);
  h->d_ndfbar = (double*)A.take(pieces[i++]);
  h->d_ndnbar = (double*)A.take(pieces[i++]);
  h->d_nphibar = (double*)A.take(pieces[i++]);
  h->d_lam = (double*)A.take(pieces[i++]);
  h->d_Kd = (double*)A.take(pieces[i++]);
  h->d_cG = (double*)A.take(pieces[i++]);
  h->d_nkpart = (double*)A.take(pieces[i++]);
  h->d_nrpart = (double*)A.take(pieces[i++]);
  h->d_nscal = (double*)A.take(pieces[i++]);
  h->d_NS = (double*)A.take(pieces[i++]);
  h->d_sens_full = (double*)A.take(pieces[i++]);
  for (int t = 0; t < 2; ++t) h->d_gam[t] = (double*)A.take(pieces[i++]) + h->plane;
  for (int t = 0; t < 2; ++t) h->d_fsg[t] = (double*)A.take(pieces[i++]);
  h->d_gsrc = (double*)A.take(pieces[i++]);
  h->d_nufk = (double*)A.take(pieces[i++]);
  h->d_lpart = (double*)A.take(pieces[i++]);
  h->d_gpart = (double*)A.take(pieces[i++]);
  h->d_ctlg = (OuterCtl*)A.take(pieces[i++]);
  h->d_gsrc2 = (float2*)A.take(pieces[i++]);
  h->d_nufk2 = (float2*)A.take(pieces[i++]);
  h->d_dlam = (double*)A.take(pieces[i++]);
  if (A.used > A.size) return fail(h, ADP_ERR_CUDA, "internal: nodal adjoint arena overflow");
  CK(cudaMemsetAsync(A.base, 0, A.size, h->st));   // halos, inactive positions and non-canonical slots stay 0
  CK(cudaStreamSynchronize(h->st));
  return ADP_OK;
}

// The derivative of k at the nonlinear fixed point of the CMFD eigenproblem
// M(d) phi = (1/k) F phi and the nodal update d = N(phi, d, k):
//   dk/dSigma = KS (1 + s) + lam^T N_Sigma + Gam^T (F_Sigma / k - M_Sigma) phi,
//   lam = Kd (1 + s) + N_d^T lam - Gam^T M_d phi        (per face, canonical slots)
//   (M - F/k)^T Gam = N_phi^T lam,   Gam^T F phi = 0,   s = N_k^T lam,
// with KS, Kd the frozen-dn derivatives -k^2 psi^T (M_x - F_x/k) phi / (psi^T F phi).
// Solved like the forward problem it is the adjoint of: rounds of `K` outer
// iterations of the generalized adjoint Gam (the persistent kernel on the
// transposed stencil with the eigenvalue held, nu*fission/k as the fission
// weight and N_phi^T lam as the external source, its fundamental-mode
// component removed after every round), each followed by the update of
// lam, until lam's relative change is below tol.
static adp_status adjoint_nodal(adp_handle* h, double tol, const OuterCtl& fwd, const OuterCtl& ca, int& rounds,
                                int& gouters, double& resid, double& lrel) {
  adp_status s = nadj_alloc(h);
  if (s != ADP_OK) return s;
  const BoxGeom G = box_geom(h);
  const int ng = h->ng, nn = h->nnod;
  const double* phi = h->d_phi[fwd.cur];
  const double* psi = h->d_psi[ca.cur];
  // forward intermediates of the update at the converged state
  NodalParams NP = nodal_params(h, 1);
  CK(launch_nodal_prep(NP, h->st));
  // the generalized adjoint starts at 0 with the eigenvalue held
  const size_t gbytes = (size_t)ng * h->NBH * 8;
  for (int t = 0; t < 2; ++t) {
    CK(cudaMemsetAsync(h->d_gam[t] - h->plane, 0, gbytes, h->st));
    CK(cudaMemsetAsync(h->d_fsg[t], 0, (size_t)h->NB * 8, h->st));
  }
  // psi^T F phi (the projection of Gam = 0 changes nothing)
  CK(launch_gpt_project(G, ng, nn, h->NBH, h->d_act, h->d_chin, h->d_nuf, phi, psi, h->d_gpart, h->d_gam[0],
                        h->d_fsg[0], h->st));
  std::vector<double> part(2 * kMaxBlocks);
  CK(cudaMemcpyAsync(part.data(), h->d_gpart, part.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const int nbp = std::max(1, std::min((nn + 255) / 256, kMaxBlocks));
  double den = 0.0;
  for (int b = 0; b < nbp; ++b) den += part[kMaxBlocks + b];
  const double k = fwd.Ke;
  if (!(den != 0.0) || !std::isfinite(den)) return fail(h, ADP_ERR_NAN, "adp_adjoint_sens: psi^T F phi is zero");
  CK(launch_face_contract(G, ng, nn, h->NBH, h->d_act, phi, psi, -k * k / den, h->d_Kd, h->st));
  CK(cudaMemcpyAsync(h->d_lam, h->d_Kd, (size_t)ng * 6 * h->NB * 8, cudaMemcpyDeviceToDevice, h->st));
  CK(launch_scale_planes(h->d_nuf, 1.0 / k, h->d_nufk, (long long)ng * h->NB, h->st));
  if (h->o.precision == ADP_MIXED) CK(launch_split(h->d_nufk, h->d_nufk2, (long long)ng * h->NB, h->st));
  NadjParams Q;
  std::memset(&Q, 0, sizeof Q);
  Q.N = NP;
  Q.lam = h->d_lam;
  Q.side = h->d_nside;
  Q.nodeu = h->d_nnodeu;
  Q.Lbar = h->d_nLbar;
  Q.dfbar = h->d_ndfbar;
  Q.dnbar = h->d_ndnbar;
  Q.phibar = h->d_nphibar;
  Q.kpart = h->d_nkpart;
  Q.rpart = h->d_nrpart;
  Q.scal = h->d_nscal;
  Q.out = h->d_NS;
  OuterParams P = outer_params(h, 1);
  // a mixed-precision handle runs the generalized adjoint in the mixed
  // kernel (FP32 Krylov steps, double-float defect correction: it converges
  // to the FP64 solution), an FP64 handle in the FP64 kernel
  P.trans = 1;
  P.A = h->d_AT;
  if (P.mixed) {
    P.A32 = h->d_AT32;
    P.A2 = h->d_AT2;
    P.wsrc2 = h->d_nufk2;
    P.exsrc2 = h->d_gsrc2;
  }
  for (int t = 0; t < 2; ++t) {
    P.phi[t] = h->d_gam[t];
    P.fs[t] = h->d_fsg[t];
  }
  P.wsrc = h->d_nufk;
  P.exsrc = h->d_gsrc;
  P.ctl = h->d_ctlg;
  P.do_nodal = 1;
#ifndef ADP_GPT_OUTERS
#define ADP_GPT_OUTERS 0   // outers of Gam per round; 0: two extrapolation intervals, 2 nac
#endif
  // Measured on the 34x34x22 core (tol 1e-8): the rounds lam needs do not
  // depend on the outers per round between 12 and 72 (22 rounds either way),
  // so short rounds cost least; at 5 the rounds grow (41), at 2 they explode.
  const int K = std::min(ADP_GPT_OUTERS > 0 ? ADP_GPT_OUTERS : std::max(2 * h->o.nac, 4), std::max(h->o.nout, 1));
  P.nupd = K;
  P.serc = P.ferc = 0.0;   // rounds end on the count; convergence is lam's
  int blocks, threads;
  launch_shape(h, blocks, threads);
  P.smem_rows = 0;
  OuterCtl c;
  std::memset(&c, 0, sizeof c);
  c.Ke = k;
  c.need_prologue = 1;
  c.err_node = -1;
  c.wait_ns = h->wait_ns;
  *h->h_ctl = c;
  CK(cudaMemcpyAsync(h->d_ctlg, h->h_ctl, sizeof(OuterCtl), cudaMemcpyHostToDevice, h->st));
  const double ltol = std::max(tol > 0 ? tol : std::min(h->o.serc, h->o.ferc), 1e-13);
  const int max_rounds = std::max(4, 4 * h->o.nout / K);
  const int lblk = lam_update_blocks(ng, nn);
  std::vector<double> lp(2 * kMaxBlocks);
  double scal[2] = {0.0, 0.0};
  rounds = 0;
  gouters = 0;
  lrel = 1.0;
  bool conv = false;
  double dprev = 0.0, rprev = 0.0;
  int since = 0;
  for (int r = 0; r < max_rounds; ++r) {
    Range r_round("nodal adjoint round");
    CK(launch_nodal_adjoint(Q, h->st));
    CK(launch_gpt_source(G, ng, nn, h->NBH, h->d_act, phi, h->d_nphibar, h->d_gpart, h->d_gsrc, h->st));
    if (P.mixed) CK(launch_split(h->d_gsrc, h->d_gsrc2, (long long)ng * h->NB, h->st));
    CK(cudaMemsetAsync(&h->d_ctlg->p, 0, sizeof(int), h->st));
    CK(cudaMemsetAsync(&h->d_ctlg->nodal_due, 0, sizeof(int), h->st));
    CK(cudaMemsetAsync(&h->d_ctlg->bar_count, 0, sizeof(unsigned), h->st));
    CK(launch_outer(P, blocks, threads, h->st));
    CK(cudaMemcpyAsync(h->h_ctl, h->d_ctlg, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    c = *h->h_ctl;
    if (c.status) return ctl_error(h, c);
    gouters += c.p;
    double* gam = h->d_gam[c.cur];
    CK(launch_gpt_project(G, ng, nn, h->NBH, h->d_act, h->d_chin, h->d_nuf, phi, psi, h->d_gpart, gam,
                          h->d_fsg[c.cur], h->st));
    CK(launch_face_contract(G, ng, nn, h->NBH, h->d_act, phi, gam, 1.0, h->d_cG, h->st));
    CK(launch_lam_update(G, ng, nn, h->d_act, h->d_Kd, h->d_ndnbar, h->d_cG, h->d_nscal, h->d_lam, h->d_dlam,
                         h->d_lpart, h->st));
    CK(cudaMemcpyAsync(lp.data(), h->d_lpart, lp.size() * 8, cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(scal, h->d_nscal, 2 * 8, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    double d2 = 0.0, n2 = 0.0;
    for (int b = 0; b < lblk; ++b) {
      d2 += lp[b];
      n2 += lp[kMaxBlocks + b];
    }
    ++rounds;
    if (r == 0) resid = scal[1];
    if (!std::isfinite(d2) || !std::isfinite(n2) || !std::isfinite(scal[0]))
      return fail(h, ADP_ERR_NAN, "adp_adjoint_sens: non-finite adjoint of the nodal update");
    lrel = n2 > 0.0 ? std::sqrt(d2 / n2) : 0.0;
    if (r >= 2 && lrel < ltol) {
      conv = true;
      break;
    }
#ifndef ADP_LAM_EXTRAP
#define ADP_LAM_EXTRAP 1
#endif
    // lam converges linearly (about 0.4 per round): once two successive
    // contractions agree, extrapolate along the last change as the forward
    // iteration does its fission source (mod_cmfd.f90:308-335)
    const double dn = std::sqrt(d2);
    const double ratio = dprev > 0.0 ? dn / dprev : 0.0;
    if (ADP_LAM_EXTRAP && since >= 2 && ratio > 0.0 && ratio < 0.9 && rprev > 0.0 &&
        std::fabs(ratio - rprev) <= 0.1 * ratio) {
      CK(launch_lam_extrap(G, ng, nn, h->d_act, h->d_dlam, ratio / (1.0 - ratio), h->d_lam, h->st));
      since = 0;
      dprev = 0.0;
      rprev = 0.0;
    } else {
      ++since;
      rprev = ratio;
      dprev = dn;
    }
  }
  if (!conv) return fail(h, ADP_ERR_MAXOUTER, "adp_adjoint_sens: the adjoint of the nodal update did not converge");
  // the derivative at the final lam
  CK(launch_nodal_adjoint(Q, h->st));
  SensParams S = sens_params(h, k, phi, h->d_gam[c.cur]);
  CK(launch_sens_total(S, h->d_sens, h->d_NS, h->d_nscal, h->d_sens_full, h->st));
  return ADP_OK;
}

static adp_status adjoint_entry(adp_handle* h, double tol, bool through_nodal, double* dkdp, double* psi,
                                adp_report* rep) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!h->fwd_ok)
    return fail(h, ADP_ERR_STATE, "adp_adjoint_sens: needs a converged forward adp_outer on the current cross sections");
  through_nodal = through_nodal && h->o.kern != ADP_KERN_FDM;
  if (through_nodal && h->ng > 4)
    return fail(h, ADP_ERR_UNSUPPORTED, "adp_adjoint_sens: the derivative through the nodal update supports ng <= 4");
  adp_status s = adj_alloc(h);
  if (s != ADP_OK) return s;
  CK(cudaEventRecord(h->e0, h->st));
  OuterCtl fwd, c;
  adp_status result = adjoint_frozen(h, tol, fwd, c);
  if (rep) {
    // the trace of the adjoint eigen-solve
    int n = std::min(std::min(c.p, rep->trace_cap), h->o.nout);
    if (n > 0) {
      if (rep->trace_k) CK(cudaMemcpy(rep->trace_k, h->d_tr_k, n * 8, cudaMemcpyDeviceToHost));
      if (rep->trace_ser) CK(cudaMemcpy(rep->trace_ser, h->d_tr_ser, n * 8, cudaMemcpyDeviceToHost));
      if (rep->trace_fer) CK(cudaMemcpy(rep->trace_fer, h->d_tr_fer, n * 8, cudaMemcpyDeviceToHost));
      if (rep->trace_flags) CK(cudaMemcpy(rep->trace_flags, h->d_tr_flags, n * 4, cudaMemcpyDeviceToHost));
      if (rep->trace_ndmax) CK(cudaMemcpy(rep->trace_ndmax, h->d_tr_ndmax, n * 8, cudaMemcpyDeviceToHost));
    }
  }
  int rounds = 0, gouters = 0;
  double resid = 0.0, lrel = 0.0;
  if (result == ADP_OK && through_nodal) result = adjoint_nodal(h, tol, fwd, c, rounds, gouters, resid, lrel);
  CK(cudaEventRecord(h->e1, h->st));
  CK(cudaEventSynchronize(h->e1));
  float total_ms = 0.f;
  cudaEventElapsedTime(&total_ms, h->e0, h->e1);
  h->tm.adjoint_ms += total_ms;
  h->tm.adjoint_outers += c.p + gouters;
  if (rep) {
    rep->outers = c.p + gouters;
    rep->converged = result == ADP_OK;
    rep->nodal_updates = rounds;
    rep->keff = c.Ke;
    rep->ser = through_nodal ? lrel : c.ser;
    rep->fer = c.fer;
    rep->ndmax = resid;
    rep->im = rep->jm = rep->km = 0;
    rep->device_ms = total_ms;
  }
  if (result != ADP_OK) return result;
  const int nn = h->nnod, G = h->ng;
  const double* src = through_nodal ? h->d_sens_full : h->d_sens;
  if (dkdp) CK(cudaMemcpy(dkdp, src, (size_t)nn * G * (4 + G) * 8, cudaMemcpyDeviceToHost));
  if (psi) {
    Xfer X;
    adp_status s2 = xfer_reserve(h, h->nmat, X);
    if (s2 != ADP_OK) return s2;
    return get_nodes(h, X, h->d_psi[c.cur], G, 1, h->NBH, psi);
  }
  return ADP_OK;
}

adp_status adp_adjoint_sens(adp_handle* h, double tol, double* dkdp, double* psi, adp_report* rep) {
  return adjoint_entry(h, tol, true, dkdp, psi, rep);
}

adp_status adp_adjoint_sens_frozen(adp_handle* h, double tol, double* dkdp, double* psi, adp_report* rep) {
  return adjoint_entry(h, tol, false, dkdp, psi, rep);
}

static AssembleParams assemble_params(adp_handle* h, int with_coupling) {
  AssembleParams AP;
  AP.G = box_geom(h);
  AP.ng = h->ng;
  AP.with_coupling = with_coupling;
  AP.D = h->d_D;
  AP.sigr = h->d_sigr;
  AP.df = h->d_df;
  AP.dn = h->d_dn;
  AP.A = h->d_A;
  AP.A32 = h->d_A32;
  AP.A2 = h->d_A2;
  AP.ctl = h->d_ctl;
  return AP;
}

adp_status adp_get_matrix(adp_handle* h, double* A7) {
  if (!h || !A7) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!h->xs_set) return fail(h, ADP_ERR_STATE, "adp_get_matrix: cross sections not set");
  CK(launch_assemble(assemble_params(h, 1), h->st));
  Xfer X;
  adp_status s = xfer_reserve(h, h->nmat, X);
  if (s != ADP_OK) return s;
  return get_nodes(h, X, h->d_A, h->ng, 7, h->NB, A7);
}

adp_status adp_nodal_step(adp_handle* h, adp_report* rep) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!h->xs_set || !h->started[0])
    return fail(h, ADP_ERR_STATE, "adp_nodal_step: needs cross sections and a forward state");
  if (h->o.kern == ADP_KERN_FDM) return fail(h, ADP_ERR_INPUT, "adp_nodal_step: the FDM kernel has no nodal update");
  CK(launch_assemble(assemble_params(h, 1), h->st));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  OuterCtl c = *h->h_ctl;
  c.status = 0;
  c.err_node = -1;
  c.converged = c.max_reached = c.nodal_due = 0;
  c.p = 0;                       // no trace row is written for this update
  *h->h_ctl = c;
  CK(cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(OuterCtl), cudaMemcpyHostToDevice, h->st));
  CK(launch_nodal(nodal_params(h, 1), h->st));
  CK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  c = *h->h_ctl;
  h->fwd_ok = false;
  if (rep) {
    rep->ndmax = c.ndmax;
    rep->im = c.im;
    rep->jm = c.jm;
    rep->km = c.km;
    rep->keff = c.Ke;
    rep->nodal_updates = 1;
  }
  if (c.status) return ctl_error(h, c);
  return ADP_OK;
}

adp_status adp_get_nodal_sources(adp_handle* h, double* S) {
  if (!h || !S) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  Xfer X;
  adp_status s = xfer_reserve(h, h->nmat, X);
  if (s != ADP_OK) return s;
  // box [u][g][NB] -> host (nnod, ng, 3): one direction at a time
  std::vector<double> tmp((size_t)h->nnod * h->ng);
  for (int u = 0; u < 3; ++u) {
    if ((s = get_nodes(h, X, h->d_S + (size_t)u * h->ng * h->NB, h->ng, 1, h->NB, tmp.data())) != ADP_OK) return s;
    std::memcpy(S + (size_t)u * h->nnod * h->ng, tmp.data(), tmp.size() * 8);
  }
  return ADP_OK;
}

adp_status adp_nodal_vjp(adp_handle* h, const double* lam, double* phibar, double* dnbar, double* kbar,
                         double* sigbar, double* resid) {
  if (!h) return ADP_ERR_INPUT;
  CK(cudaSetDevice(h->dev));
  if (!lam) return fail(h, ADP_ERR_INPUT, "adp_nodal_vjp: null lam");
  if (!h->xs_set || !h->started[0])
    return fail(h, ADP_ERR_STATE, "adp_nodal_vjp: needs cross sections and a forward state");
  if (h->o.kern == ADP_KERN_FDM) return fail(h, ADP_ERR_INPUT, "adp_nodal_vjp: the FDM kernel has no nodal update");
  if (h->ng > 4) return fail(h, ADP_ERR_UNSUPPORTED, "adp_nodal_vjp: supports ng <= 4");
  adp_status s = nadj_alloc(h);
  if (s != ADP_OK) return s;
  Xfer X;
  if ((s = xfer_reserve(h, h->nmat, X)) != ADP_OK) return s;
  if ((s = put_nodes(h, X, lam, h->ng, 6, h->d_lam, h->NB, 0)) != ADP_OK) return s;
  // df of the current cross sections (matrix_setup(1), as adp_outer starts)
  AssembleParams AP;
  AP.G = box_geom(h);
  AP.ng = h->ng;
  AP.with_coupling = 1;
  AP.D = h->d_D;
  AP.sigr = h->d_sigr;
  AP.df = h->d_df;
  AP.dn = h->d_dn;
  AP.A = h->d_A;
  AP.A32 = h->d_A32;
  AP.A2 = h->d_A2;
  AP.ctl = h->d_ctl;
  CK(launch_assemble(AP, h->st));
  NodalParams NP = nodal_params(h, 1);
  CK(launch_nodal_prep(NP, h->st));
  NadjParams Q;
  std::memset(&Q, 0, sizeof Q);
  Q.N = NP;
  Q.lam = h->d_lam;
  Q.side = h->d_nside;
  Q.nodeu = h->d_nnodeu;
  Q.Lbar = h->d_nLbar;
  Q.dfbar = h->d_ndfbar;
  Q.dnbar = h->d_ndnbar;
  Q.phibar = h->d_nphibar;
  Q.kpart = h->d_nkpart;
  Q.rpart = h->d_nrpart;
  Q.scal = h->d_nscal;
  Q.out = h->d_NS;
  CK(launch_nodal_adjoint(Q, h->st));
  double scal[2];
  CK(cudaMemcpyAsync(scal, h->d_nscal, 16, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (kbar) *kbar = scal[0];
  if (resid) *resid = scal[1];
  if (phibar && (s = get_nodes(h, X, h->d_nphibar, h->ng, 1, h->NB, phibar)) != ADP_OK) return s;
  if (dnbar && (s = get_nodes(h, X, h->d_ndnbar, h->ng, 6, h->NB, dnbar)) != ADP_OK) return s;
  if (sigbar)
    CK(cudaMemcpy(sigbar, h->d_NS, (size_t)h->nnod * h->ng * (4 + h->ng) * 8, cudaMemcpyDeviceToHost));
  return ADP_OK;
}

adp_status adp_get_timers(const adp_handle* h, adp_timers* t) {
  if (!h || !t) return ADP_ERR_INPUT;
  *t = h->tm;
  return ADP_OK;
}

}  // extern "C"
