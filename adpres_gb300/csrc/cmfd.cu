// CMFD kernels: coupling coefficients and matrix assembly, the persistent
// outer-iteration kernel (group sweeps of BiCGSTAB, fission source,
// extrapolation, eigenvalue and convergence test) and the power edit.
//
// Reference routines: coup_coef / matrix_setup (mod_cmfd.f90:11-304),
// outer / outer_ad (:415-509, :602-699), FSrc/FSrcAd (:956-1002),
// TSrc/TSrcAd (:1006-1064), l2norm/Integrate/RelE/RelEg (:1100-1199),
// bicg / sp_matvec / dproduct (:1203-1286), fiss_extrp (:308-335),
// PowDis (:1290-1333).
#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"
#include "cmfd_items.cuh"
#include "outer_body.cuh"

namespace adp {

constexpr int kOuterThreads = 512;

// ---------------------------------------------------------------------------
// matrix_setup (mod_cmfd.f90:217-304) with coup_coef (:11-137) when requested.
// One thread per (node, group); inactive box positions get all-zero rows.
// Row slots in reference column order: [z-, y-, x-, diag, x+, y+, z+].
// ---------------------------------------------------------------------------
__global__ void k_assemble(AssembleParams P) {
  assemble_items(P, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

cudaError_t launch_assemble(const AssembleParams& P, cudaStream_t st) {
  long long total = (long long)P.G.NB * P.ng;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 65535 * 4) blocks = 65535 * 4;
  k_assemble<<<blocks, 256, 0, st>>>(P);
  return cudaGetLastError();
}

// First-call start of outer()/outer_ad(): f0 = 1, Ke = 1, fs0 = FSrc(f0)
// (mod_cmfd.f90:448-454, :635-641).
__global__ void k_split(const double* x, float2* out, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double v = x[q];
    const float h = (float)v;
    out[q] = make_float2(h, (float)(v - (double)h));
  }
}

cudaError_t launch_split(const double* x, float2* out, long long n, cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 65535 * 4) blocks = 65535 * 4;
  if (blocks < 1) blocks = 1;
  k_split<<<(int)blocks, 256, 0, st>>>(x, out, n);
  return cudaGetLastError();
}

__global__ void k_init_flux(OuterParams P) { init_flux_items(P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x); }

cudaError_t launch_init_flux(const OuterParams& P, cudaStream_t st) {
  int blocks = (P.G.NB + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_init_flux<<<blocks, 256, 0, st>>>(P);
  return cudaGetLastError();
}

template <bool MIXED, bool SMEMA, bool XSRC = false>
__global__ void __launch_bounds__(kOuterThreads, 1) k_outer(OuterParams P) {
  outer_body<MIXED, SMEMA, XSRC>(P, blockIdx.x, gridDim.x + P.phantom);
}

int outer_max_blocks_per_sm(int threads, int mixed) {
  int nb = 0;
  if (mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_outer<true, false>, threads, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_outer<false, false>, threads, 0);
  return nb;
}

// Shared memory of the matrix copy: at most this much (the static shared
// memory of the kernel is a few KB; 227 KB per block is the limit).
constexpr size_t kSmemMatrixMax = 200 * 1024;

int outer_smem_rows(int NB, int blocks, int threads, int mixed) {
  const long long nthr = (long long)blocks * threads;
  const long long rpt = (NB + nthr - 1) / nthr;   // rows per thread
  const long long rows = rpt * threads;
  const size_t bytes = (size_t)rows * 7 * (mixed ? sizeof(float) : sizeof(double));
  return bytes <= kSmemMatrixMax ? (int)rows : 0;
}

template <bool MIXED, bool SMEMA>
static cudaError_t launch_outer_t(const OuterParams& P, int blocks, int threads, cudaStream_t st) {
  void* args[] = {(void*)&P};
  size_t smem = 0;
  if (SMEMA) {
    smem = (size_t)P.smem_rows * 7 * (MIXED ? sizeof(float) : sizeof(double));
    cudaError_t e = cudaFuncSetAttribute((const void*)k_outer<MIXED, SMEMA>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  return cudaLaunchCooperativeKernel((const void*)k_outer<MIXED, SMEMA>, dim3(blocks), dim3(threads), args, smem, st);
}

cudaError_t launch_outer(const OuterParams& P, int blocks, int threads, cudaStream_t st) {
  if (P.mixed && P.trans) {
    // a transient step or the generalized adjoint in mixed precision: the
    // external source as (hi, lo) pairs, no shared-memory matrix copy
    void* args[] = {(void*)&P};
    return cudaLaunchCooperativeKernel((const void*)k_outer<true, false, true>, dim3(blocks), dim3(threads), args, 0,
                                       st);
  }
  if (P.smem_rows > 0)
    return P.mixed ? launch_outer_t<true, true>(P, blocks, threads, st) : launch_outer_t<false, true>(P, blocks, threads, st);
  return P.mixed ? launch_outer_t<true, false>(P, blocks, threads, st) : launch_outer_t<false, false>(P, blocks, threads, st);
}

// ---------------------------------------------------------------------------
// PowDis (mod_cmfd.f90:1290-1333): per-node power, then the total in a fixed
// order and the normalisation.
// ---------------------------------------------------------------------------
__global__ void k_power_nodes(BoxGeom G, int ng, long long NBH, const double* phi, const double* sigf, double* pbox,
                              double* part) {
  double acc[1] = {0.0};
  // 64-bit index: the stride is added after the last row, so an int could
  // wrap when NB is within one stride of 2^31
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < G.NB;
       b += (long long)gridDim.x * blockDim.x) {
    double pw = 0.0;
    for (int g = 0; g < ng; ++g) {
      double q = phi[(size_t)g * NBH + b] * sigf[(size_t)g * G.NB + b] * G.vdel[b];
      if (q < 0.) q = 0.;
      pw = pw + q;
    }
    pbox[b] = pw;
    acc[0] += pw;
  }
  block_partials<1, 0u>(acc, part);
}

__global__ void k_power_norm(BoxGeom G, double* pbox, const double* part, int nblk, OuterCtl* C) {
  double tot[1];
  grid_totals<1, 0u>(part, nblk, tot);
  const double tpow = tot[0];
  if (tpow <= 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_status(C, ADP_ERR_ZEROPOWER);
    return;
  }
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < G.NB;
       b += (long long)gridDim.x * blockDim.x)
    pbox[b] = pbox[b] / tpow;
}

cudaError_t launch_power(const BoxGeom& G, int ng, long long NBH, const double* phi, const double* sigf, double* pbox,
                         double* red, OuterCtl* ctl, cudaStream_t st) {
  int blocks = (G.NB + 255) / 256;
  if (blocks > kMaxBlocks) blocks = kMaxBlocks;
  k_power_nodes<<<blocks, 256, 0, st>>>(G, ng, NBH, phi, sigf, pbox, red);
  k_power_norm<<<blocks, 256, 0, st>>>(G, pbox, red, blocks, ctl);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dsigr_updt (mod_xsec.f90:199-226) and the node checks of check_xs
// (:90-168) on the device.
// ---------------------------------------------------------------------------
__global__ void k_xs_updt(BoxGeom G, int ng, const int* act, int nnod, const double* sigtr, const double* siga,
                          const double* sigs, double* D, double* sigr, OuterCtl* C) {
  xs_updt_items(G, ng, act, nnod, sigtr, siga, sigs, D, sigr, C, blockIdx.x * blockDim.x + threadIdx.x,
                gridDim.x * blockDim.x);
}

cudaError_t launch_xs_updt(const BoxGeom& G, int ng, const int* act, int nnod, const double* sigtr,
                           const double* siga, const double* sigs, double* D, double* sigr, OuterCtl* ctl,
                           cudaStream_t st) {
  int blocks = (nnod * ng + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_xs_updt<<<blocks, 256, 0, st>>>(G, ng, act, nnod, sigtr, siga, sigs, D, sigr, ctl);
  return cudaGetLastError();
}

}  // namespace adp
