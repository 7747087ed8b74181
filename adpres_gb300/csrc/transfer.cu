// Node-order transfers between the host's arrays and the device's box
// layout.  The host hands over arrays in its own layout, a(nnod, A[, B])
// with the node index fastest (the sdata arrays of the reference); they
// cross PCIe/C2C as one contiguous copy each, and the node -> box scatter
// (with the component transpose to the device's [A][B][NB] planes) runs
// here, as do the sign checks of check_xs (mod_xsec.f90:90-168) and
// base_updt (:172-195), which expands the material tables on the device.
#include <cuda_runtime.h>

#include <algorithm>

#include "adp_kernels.h"

namespace adp {

namespace {

constexpr int kXferThreads = 256;

int xfer_blocks(long long work) {
  const long long b = (work + kXferThreads - 1) / kXferThreads;
  return (int)std::max(1LL, std::min(b, 152LL * 16));
}

// dst[(i*B + j)*dstride + act[n]] = src[(j*A + i)*nn + n]; flags |= chk if a value < 0
__global__ void k_nodes_to_box(const double* __restrict__ src, double* __restrict__ dst, const int* __restrict__ act,
                               int nn, int A, int B, long long dstride, int chk, int* flags) {
  const long long total = (long long)nn * A * B;
  int bad = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(q % nn);
    const int cs = (int)(q / nn);
    const int i = cs % A, j = cs / A;
    const double v = src[q];
    bad |= v < 0.0;
    dst[(long long)(i * B + j) * dstride + act[n]] = v;
  }
  if (chk && __syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flags, chk);
}

// dst[(j*A + i)*nn + n] = src[(i*B + j)*sstride + act[n]]
__global__ void k_box_to_nodes(const double* __restrict__ src, double* __restrict__ dst, const int* __restrict__ act,
                               int nn, int A, int B, long long sstride) {
  const long long total = (long long)nn * A * B;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(q % nn);
    const int cs = (int)(q / nn);
    const int i = cs % A, j = cs / A;
    dst[q] = src[(long long)(i * B + j) * sstride + act[n]];
  }
}

// dst[c*dstride + act[n]] = v for every component c < ncomp
__global__ void k_fill_box(double* __restrict__ dst, const int* __restrict__ act, int nn, int ncomp,
                           long long dstride, double v) {
  const long long total = (long long)nn * ncomp;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x)
    dst[(q / nn) * dstride + act[q % nn]] = v;
}

// base_updt from material tables t(nmat, G) (Fortran) and sigs(nmat, G, G):
// the node's chi always; the other tables where given (null: the node
// tables of that quantity were uploaded instead).  flags |= 1 for a
// negative nu*fission, 4 for a negative scattering entry of a node.
__global__ void k_base_updt(XsTables T, const int* __restrict__ mat, const int* __restrict__ act, int nn, int nmat,
                            int G, long long NB, XsBox X, int* flags) {
  const long long total = (long long)nn * G;
  int bad = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(q % nn), g = (int)(q / nn);
    const int m = mat[n] - 1;
    const long long b = (long long)g * NB + act[n];
    const int t = g * nmat + m;
    X.chin[b] = T.chi[t];
    if (T.sigtr) X.sigtr[b] = T.sigtr[t];
    if (T.siga) X.siga[b] = T.siga[t];
    if (T.nuf) {
      const double v = T.nuf[t];
      bad |= v < 0.0 ? 1 : 0;
      X.nuf[b] = v;
    }
    if (T.sigf) X.sigf[b] = T.sigf[t];
    if (T.sigs)
      for (int h = 0; h < G; ++h) {
        const double v = T.sigs[m + (long long)nmat * (g + (long long)G * h)];
        bad |= v < 0.0 ? 4 : 0;
        X.sigs[((long long)g * G + h) * NB + act[n]] = v;
      }
  }
  const int nuf_bad = __syncthreads_or(bad & 1);
  const int sigs_bad = __syncthreads_or(bad & 4);
  if (threadIdx.x == 0 && (nuf_bad || sigs_bad)) atomicOr(flags, (nuf_bad ? 1 : 0) | (sigs_bad ? 4 : 0));
}

// The state changes of XS_updt on the material tables (bcon_updt, ftem_updt,
// mtem_updt, cden_updt, mod_xsec.f90:394-521), one entry per thread:
// x = x + dx * dv card by card, each product and sum rounded on its own as
// the reference's separate statements are.
__global__ void k_fb_state(FbParams P) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < P.tq;
       q += (long long)gridDim.x * blockDim.x) {
    double v = P.base[q];
    for (int s = 0; s < P.nst; ++s) v = __dadd_rn(v, __dmul_rn(P.dsig[s * P.tq + q], P.dv[s]));
    P.tab[q] = v;
  }
}

// base_updt of the changed tables and crod_updt (mod_xsec.f90:172-195,
// :230-303), one (node, group) per thread.  A node of bank b in a plane
// above the rod tip takes x + dx, the plane of the tip x + w dx; in rodded
// columns negative siga, nuf, sigf and sigs become 0.  flags as
// k_base_updt: 1 a negative nu*fission, 4 a negative scattering entry.
__global__ void k_fb_nodes(FbParams P) {
  const long long total = (long long)P.nn * P.G;
  const int G = P.G, nmat = P.nmat;
  int bad = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(q % P.nn), g = (int)(q / P.nn);
    const int m = P.mat[n] - 1;
    const int a = P.act[n];
    const long long b = (long long)g * P.NB + a;
    const int bk = P.bank[n];
    int mode = 0;   // 0 no rod, 1 fully rodded, 2 the plane of the tip
    double w = 0.0;
    if (bk > 0) {
      const int z = a / P.plane, kt = P.tip[bk - 1];
      mode = z > kt ? 1 : (z == kt ? 2 : 0);
      w = P.vf[bk - 1];
    }
    auto val = [&](int tq, long long i, bool clamp) -> double {
      double v = P.tab[P.off[tq] + i];
      if (mode == 1) v = __dadd_rn(v, P.rsig[P.off[tq] + i]);
      else if (mode == 2) v = __dadd_rn(v, __dmul_rn(w, P.rsig[P.off[tq] + i]));
      if (clamp && bk > 0 && v < 0.0) v = 0.0;
      return v;
    };
    const long long t = (long long)g * nmat + m;
    P.X.chin[b] = P.chi[t];
    P.X.sigtr[b] = val(0, t, false);
    P.X.siga[b] = val(1, t, true);
    const double nf = val(2, t, true);
    bad |= nf < 0.0 ? 1 : 0;
    P.X.nuf[b] = nf;
    P.X.sigf[b] = val(3, t, true);
    for (int h = 0; h < G; ++h) {
      const double v = val(4, m + (long long)nmat * (g + (long long)G * h), true);
      bad |= v < 0.0 ? 4 : 0;
      P.X.sigs[((long long)g * G + h) * P.NB + a] = v;
    }
  }
  const int nuf_bad = __syncthreads_or(bad & 1);
  const int sigs_bad = __syncthreads_or(bad & 4);
  if (threadIdx.x == 0 && (nuf_bad || sigs_bad)) atomicOr(P.flags, (nuf_bad ? 1 : 0) | (sigs_bad ? 4 : 0));
}

// Source planes that are nonzero somewhere (launch_xs_nonzero): per thread
// the masks of its nodes, OR-reduced over the warp, one atomic per warp.
__global__ void k_xs_nonzero(const double* __restrict__ chin, const double* __restrict__ nuf,
                             const double* __restrict__ sigs, const int* __restrict__ act, int nn, int G,
                             long long NB, unsigned* out) {
  unsigned c = 0, f = 0, s0 = 0, s1 = 0;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
    const long long b = act[n];
    for (int g = 0; g < G; ++g) {
      if (chin[g * NB + b] != 0.0) c |= 1u << g;
      if (nuf[g * NB + b] != 0.0) f |= 1u << g;
      for (int h = 0; h < G; ++h) {
        const int q = g * G + h;
        if (sigs[(long long)q * NB + b] != 0.0) {
          if (q < 32) s0 |= 1u << q;
          else s1 |= 1u << (q - 32);
        }
      }
    }
  }
  c = __reduce_or_sync(0xffffffffu, c);
  f = __reduce_or_sync(0xffffffffu, f);
  s0 = __reduce_or_sync(0xffffffffu, s0);
  s1 = __reduce_or_sync(0xffffffffu, s1);
  if ((threadIdx.x & 31) == 0) {
    if (c) atomicOr(out, c);
    if (f) atomicOr(out + 1, f);
    if (s0) atomicOr(out + 2, s0);
    if (s1) atomicOr(out + 3, s1);
  }
}

}  // namespace

cudaError_t launch_xs_nonzero(const double* chin, const double* nuf, const double* sigs, const int* act, int nn,
                              int G, long long NB, unsigned* out, cudaStream_t st) {
  k_xs_nonzero<<<xfer_blocks(nn), kXferThreads, 0, st>>>(chin, nuf, sigs, act, nn, G, NB, out);
  return cudaGetLastError();
}

cudaError_t launch_fb_updt(const FbParams& P, cudaStream_t st) {
  k_fb_state<<<xfer_blocks(P.tq), kXferThreads, 0, st>>>(P);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_fb_nodes<<<xfer_blocks((long long)P.nn * P.G), kXferThreads, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_nodes_to_box(const double* src, double* dst, const int* act, int nn, int A, int B,
                                long long dstride, int chk, int* flags, cudaStream_t st) {
  k_nodes_to_box<<<xfer_blocks((long long)nn * A * B), kXferThreads, 0, st>>>(src, dst, act, nn, A, B, dstride, chk,
                                                                              flags);
  return cudaGetLastError();
}

cudaError_t launch_box_to_nodes(const double* src, double* dst, const int* act, int nn, int A, int B,
                                long long sstride, cudaStream_t st) {
  k_box_to_nodes<<<xfer_blocks((long long)nn * A * B), kXferThreads, 0, st>>>(src, dst, act, nn, A, B, sstride);
  return cudaGetLastError();
}

cudaError_t launch_fill_box(double* dst, const int* act, int nn, int ncomp, long long dstride, double v,
                            cudaStream_t st) {
  k_fill_box<<<xfer_blocks((long long)nn * ncomp), kXferThreads, 0, st>>>(dst, act, nn, ncomp, dstride, v);
  return cudaGetLastError();
}

cudaError_t launch_base_updt(const XsTables& T, const int* mat, const int* act, int nn, int nmat, int G, long long NB,
                             const XsBox& X, int* flags, cudaStream_t st) {
  k_base_updt<<<xfer_blocks((long long)nn * G), kXferThreads, 0, st>>>(T, mat, act, nn, nmat, G, NB, X, flags);
  return cudaGetLastError();
}

}  // namespace adp
