// Output edits of control::forward (mod_control.f90:33-44) on the device:
// AsmPow (mod_io.f90:3267-3403), AxiPow (:3406-3498) and AsmFlux
// (:3501-3644).  The node power (PowDis) or flux stays on the device; only
// the nx x ny assembly values (or nz axial values) are copied back.
//   k_edit_columns    : per radial node column, the axial average of a node
//                       field, weighted by zdel (AsmPow) or by the node
//                       volume xdel ydel zdel (AsmFlux), summed over k in
//                       order as the reference does
//   k_edit_assemblies : per assembly, the area-weighted average of the
//                       column values over its xdiv x ydiv columns, in the
//                       reference's (ly, lx) order
//   k_edit_planes     : per box plane, the sum of a node field and of the
//                       node volumes (AxiPow; the regions of zdiv planes and
//                       the normalisation are formed on the host)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"
#include "handle.h"

namespace adp {

__global__ void k_edit_columns(BoxGeom G, int nf, long long fstride, const double* f, int volume_weight,
                               double* fnode) {
  const int ncol = G.nxx * G.nyy;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nf * ncol; q += gridDim.x * blockDim.x) {
    const int g = q / ncol, c = q - g * ncol;
    const int i = c % G.nxx, j = c / G.nxx;
    double out = 0.0;
    if (G.nbm[c] & NB_ACTIVE) {   // the outline of plane 1 is every plane's
      const double* fg = f + (size_t)g * fstride;
      double summ = 0.0, vsumm = 0.0;
      for (int k = 0; k < G.nzz; ++k) {
        const double v = fg[c + (size_t)k * G.plane];
        // _rn operations: the same roundings as the reference's expressions
        if (volume_weight) {
          summ = __dadd_rn(summ, __dmul_rn(__dmul_rn(__dmul_rn(v, G.xdel[i]), G.ydel[j]), G.zdel[k]));
          vsumm = __dadd_rn(vsumm, __dmul_rn(__dmul_rn(G.xdel[i], G.ydel[j]), G.zdel[k]));
        } else {
          summ = __dadd_rn(summ, __dmul_rn(v, G.zdel[k]));
          vsumm = __dadd_rn(vsumm, G.zdel[k]);
        }
      }
      out = summ / vsumm;
    }
    fnode[q] = out;
  }
}

__global__ void k_edit_assemblies(BoxGeom G, int nf, int nx, int ny, const int* xs, const int* ys, const int* xdiv,
                                  const int* ydiv, const double* fnode, double* fasm) {
  const int na = nx * ny, ncol = G.nxx * G.nyy;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nf * na; q += gridDim.x * blockDim.x) {
    const int g = q / na, a = q - g * na;
    const int ia = a % nx, ja = a / nx;
    const double* fn = fnode + (size_t)g * ncol;
    double summ = 0.0, vsumm = 0.0;
    for (int ly = ys[ja]; ly < ys[ja] + ydiv[ja]; ++ly)
      for (int lx = xs[ia]; lx < xs[ia] + xdiv[ia]; ++lx) {
        summ = __dadd_rn(summ, __dmul_rn(__dmul_rn(fn[lx + (size_t)G.nxx * ly], G.xdel[lx]), G.ydel[ly]));
        vsumm = __dadd_rn(vsumm, __dmul_rn(G.xdel[lx], G.ydel[ly]));
      }
    fasm[q] = summ / vsumm;
  }
}

// partials: part[q * kMaxBlocks + k], q = 0 field sum, 1 volume sum
__global__ void k_edit_planes(BoxGeom G, const double* f, double* part) {
  const int k = blockIdx.x;
  double acc[2] = {0.0, 0.0};
  for (int c = threadIdx.x; c < G.plane; c += blockDim.x) {
    const int b = c + k * G.plane;
    acc[0] += f[b];
    acc[1] += G.vdel[b];
  }
  block_partials<2, 0u>(acc, part);
}

}  // namespace adp

using namespace adp;

namespace {

adp_status efail(adp_handle* h, adp_status s, const std::string& m) {
  h->err = m;
  return s;
}

#define ECK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return efail(h, ADP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Scratch of the edits, allocated on first use: column values, assembly
// values, plane partials and the assembly index tables.
adp_status edit_scratch(adp_handle* h, int nx, int ny) {
  const size_t need = (size_t)h->ng * h->nxx * h->nyy * 8 + (size_t)h->ng * nx * ny * 8 +
                      (size_t)2 * kMaxBlocks * 8 + (size_t)4 * (h->nxx + h->nyy + 4) * 4 + 8 * 256;
  if (h->edit_size >= need) return ADP_OK;
  if (h->edit_base) cudaFree(h->edit_base);
  h->edit_base = nullptr;
  h->edit_size = 0;
  ECK(cudaMalloc((void**)&h->edit_base, need));
  h->edit_size = need;
  return ADP_OK;
}

struct EditPtrs {
  double *fnode, *fasm, *part;
  int *xs, *ys, *xdiv, *ydiv;
};

EditPtrs edit_layout(adp_handle* h, int nx, int ny) {
  DevArena A;
  A.base = h->edit_base;
  A.size = h->edit_size;
  EditPtrs p;
  p.fnode = (double*)A.take((size_t)h->ng * h->nxx * h->nyy * 8);
  p.fasm = (double*)A.take((size_t)h->ng * nx * ny * 8);
  p.part = (double*)A.take((size_t)2 * kMaxBlocks * 8);
  p.xs = (int*)A.take(nx * 4);
  p.ys = (int*)A.take(ny * 4);
  p.xdiv = (int*)A.take(nx * 4);
  p.ydiv = (int*)A.take(ny * 4);
  return p;
}

adp_status check_divs(adp_handle* h, int n, const int* div, int total, const char* what) {
  if (n < 1 || !div) return efail(h, ADP_ERR_INPUT, std::string("edit: bad ") + what + " divisions");
  int s = 0;
  for (int i = 0; i < n; ++i) {
    if (div[i] < 1) return efail(h, ADP_ERR_INPUT, std::string("edit: ") + what + " divisions must be >= 1");
    s += div[i];
  }
  if (s != total) return efail(h, ADP_ERR_INPUT, std::string("edit: ") + what + " divisions do not sum to the node count");
  return ADP_OK;
}

// column values of nf fields then assembly averages, copied to fasm (nx, ny, nf)
adp_status assembly_average(adp_handle* h, int nf, long long fstride, const double* f, int volume_weight, int nx,
                            int ny, const int* xdiv, const int* ydiv, std::vector<double>& fasm) {
  adp_status s = edit_scratch(h, nx, ny);
  if (s != ADP_OK) return s;
  EditPtrs p = edit_layout(h, nx, ny);
  std::vector<int> xs(nx), ys(ny);
  for (int i = 0, a = 0; i < nx; a += xdiv[i], ++i) xs[i] = a;
  for (int j = 0, a = 0; j < ny; a += ydiv[j], ++j) ys[j] = a;
  ECK(cudaMemcpyAsync(p.xs, xs.data(), nx * 4, cudaMemcpyHostToDevice, h->st));
  ECK(cudaMemcpyAsync(p.ys, ys.data(), ny * 4, cudaMemcpyHostToDevice, h->st));
  ECK(cudaMemcpyAsync(p.xdiv, xdiv, nx * 4, cudaMemcpyHostToDevice, h->st));
  ECK(cudaMemcpyAsync(p.ydiv, ydiv, ny * 4, cudaMemcpyHostToDevice, h->st));
  const BoxGeom G = box_geom(h);
  const int ncol = h->nxx * h->nyy;
  int b1 = std::min((nf * ncol + 255) / 256, 4096);
  k_edit_columns<<<b1, 256, 0, h->st>>>(G, nf, fstride, f, volume_weight, p.fnode);
  ECK(cudaGetLastError());
  int b2 = std::max(1, std::min((nf * nx * ny + 127) / 128, 4096));
  k_edit_assemblies<<<b2, 128, 0, h->st>>>(G, nf, nx, ny, p.xs, p.ys, p.xdiv, p.ydiv, p.fnode, p.fasm);
  ECK(cudaGetLastError());
  fasm.resize((size_t)nf * nx * ny);
  ECK(cudaMemcpyAsync(fasm.data(), p.fasm, fasm.size() * 8, cudaMemcpyDeviceToHost, h->st));
  ECK(cudaStreamSynchronize(h->st));
  return ADP_OK;
}

// PowDis into the handle's power array (normalised node power on the box)
adp_status device_power(adp_handle* h) {
  ECK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  ECK(cudaStreamSynchronize(h->st));
  OuterCtl c = *h->h_ctl;
  c.status = 0;
  *h->h_ctl = c;
  ECK(cudaMemcpyAsync(&h->d_ctl->status, &h->h_ctl->status, sizeof(int), cudaMemcpyHostToDevice, h->st));
  ECK(launch_power(box_geom(h), h->ng, h->NBH, h->d_phi[c.cur], h->d_sigf, h->d_pbox, h->d_red, h->d_ctl, h->st));
  ECK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  ECK(cudaStreamSynchronize(h->st));
  if (h->h_ctl->status) return efail(h, (adp_status)h->h_ctl->status, "total nodes power is zero or less");
  return ADP_OK;
}

}  // namespace

extern "C" {

adp_status adp_edit_asmpow(adp_handle* h, int nx, int ny, const int* xdiv, const int* ydiv, double* fasm, int* imax,
                           int* jmax) {
  if (!h || !fasm) return ADP_ERR_INPUT;
  ECK(cudaSetDevice(h->dev));
  adp_status s;
  if ((s = check_divs(h, nx, xdiv, h->nxx, "x")) != ADP_OK || (s = check_divs(h, ny, ydiv, h->nyy, "y")) != ADP_OK)
    return s;
  if ((s = device_power(h)) != ADP_OK) return s;
  std::vector<double> fa;
  if ((s = assembly_average(h, 1, 0, h->d_pbox, 0, nx, ny, xdiv, ydiv, fa)) != ADP_OK) return s;
  // normalisation and the first maximum as mod_io.f90:3321-3344
  int nfuel = 0;
  double totp = 0.0;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      if (fa[i + (size_t)nx * j] > 0.0) {
        ++nfuel;
        totp = totp + fa[i + (size_t)nx * j];
      }
  int xm = 1, ym = 1;
  double fmax = 0.0;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      double& v = fa[i + (size_t)nx * j];
      if (totp > 0.) v = (double)(float)nfuel / totp * v;   // REAL(nfuel) is default (single) real
      if (v > fmax) {
        xm = i + 1;
        ym = j + 1;
        fmax = v;
      }
    }
  std::memcpy(fasm, fa.data(), fa.size() * 8);
  if (imax) *imax = xm;
  if (jmax) *jmax = ym;
  return ADP_OK;
}

adp_status adp_edit_axipow(adp_handle* h, int nz, const int* zdiv, double* faxi, int* kmax) {
  if (!h || !faxi) return ADP_ERR_INPUT;
  ECK(cudaSetDevice(h->dev));
  adp_status s;
  if ((s = check_divs(h, nz, zdiv, h->nzz, "z")) != ADP_OK) return s;
  if ((s = device_power(h)) != ADP_OK) return s;
  if ((s = edit_scratch(h, 1, 1)) != ADP_OK) return s;
  EditPtrs p = edit_layout(h, 1, 1);
  if (h->nzz > kMaxBlocks) return efail(h, ADP_ERR_UNSUPPORTED, "edit: more planes than partial slots");
  k_edit_planes<<<h->nzz, 256, 0, h->st>>>(box_geom(h), h->d_pbox, p.part);
  ECK(cudaGetLastError());
  std::vector<double> part(2 * kMaxBlocks);
  ECK(cudaMemcpyAsync(part.data(), p.part, part.size() * 8, cudaMemcpyDeviceToHost, h->st));
  ECK(cudaStreamSynchronize(h->st));
  // regions of zdiv planes, normalisation and the first maximum (mod_io.f90:3437-3464)
  int nfuel = 0, ztot = 0;
  double totp = 0.0;
  for (int k = 0; k < nz; ++k) {
    double summ = 0.0, vsumm = 0.0;
    for (int lz = 0; lz < zdiv[k]; ++lz, ++ztot) {
      summ = summ + part[ztot];
      vsumm = vsumm + part[kMaxBlocks + ztot];
    }
    faxi[k] = summ / vsumm;
    if (faxi[k] > 0.0) {
      ++nfuel;
      totp = totp + faxi[k];
    }
  }
  double fmax = 0.0;
  int km = 1;
  for (int k = 0; k < nz; ++k) {
    faxi[k] = (double)(float)nfuel / totp * faxi[k];
    if (faxi[k] > fmax) {
      km = k + 1;
      fmax = faxi[k];
    }
  }
  if (kmax) *kmax = km;
  return ADP_OK;
}

adp_status adp_edit_asmflux(adp_handle* h, int nx, int ny, const int* xdiv, const int* ydiv, double norm, double* fasm,
                            int* negative) {
  if (!h || !fasm) return ADP_ERR_INPUT;
  ECK(cudaSetDevice(h->dev));
  adp_status s;
  if ((s = check_divs(h, nx, xdiv, h->nxx, "x")) != ADP_OK || (s = check_divs(h, ny, ydiv, h->nyy, "y")) != ADP_OK)
    return s;
  ECK(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(OuterCtl), cudaMemcpyDeviceToHost, h->st));
  ECK(cudaStreamSynchronize(h->st));
  const int cur = h->h_ctl->cur, G = h->ng;
  std::vector<double> fa;
  if ((s = assembly_average(h, G, h->NBH, h->d_phi[cur], 1, nx, ny, xdiv, ydiv, fa)) != ADP_OK) return s;
  // totals of the positive assemblies, the negative-flux flag and the
  // scaling norm / total * norm (mod_io.f90:3574-3610)
  int neg = 0;
  for (int g = 0; g < G; ++g) {
    double totp = 0.0;
    for (int q = 0; q < nx * ny; ++q) {
      const double v = fa[q + (size_t)nx * ny * g];
      if (v > 0.0) totp = totp + v;
      if (v < 0.0) neg = 1;
    }
    if (norm > 0)
      for (int q = 0; q < nx * ny; ++q) {
        double& v = fa[q + (size_t)nx * ny * g];
        v = norm / totp * v * norm;
      }
  }
  std::memcpy(fasm, fa.data(), fa.size() * 8);
  if (negative) *negative = neg;
  return ADP_OK;
}

}  // extern "C"
