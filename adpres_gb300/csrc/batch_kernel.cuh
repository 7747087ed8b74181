// Batched static solves: many independent cores in one persistent
// cooperative launch.  Each block walks its own task list; a task is one
// core solved by a team of co-resident blocks (one block for a small core),
// which synchronise only among themselves through the core's own barrier
// word, so cores converge, update their nodal coefficients and finish
// independently.  Per core the kernel runs the whole static path of
// control::forward (mod_control.f90:11-47): Dsigr_updt (mod_xsec.f90:199-226),
// get_ABEFGH (mod_nodal.f90:1409-1451), matrix_setup(1) (mod_cmfd.f90:217-304),
// the first-call start of outer (:448-454), outer iterations with nodal
// updates (:415-509, mod_nodal.f90:18-278) and PowDis (mod_cmfd.f90:1290-1333).
// Task lists are built on the host so that every block's list is a
// subsequence of one global order, which rules out a cycle of teams waiting
// on each other.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"
#include "cmfd_items.cuh"
#include "nodal_body.cuh"
#include "outer_body.cuh"

namespace adp {

// Everything after the cross-section update; false when a barrier wait ran
// out of time (the core's status then says ADP_ERR_TIMEOUT).
template <bool MIXED, int NG>
__device__ __forceinline__ bool solve_core(const BatchInst& I, unsigned rank, unsigned size) {
  const OuterParams& P = I.op;
  const NodalParams& N = I.np;
  OuterCtl* C = P.ctl;
  const int start = rank * blockDim.x + threadIdx.x, stride = size * blockDim.x;
  const bool lead = rank == 0 && threadIdx.x == 0;

  // XS_updt: D = 1/(3 sigtr), sigr = siga + sum_{h/=g} sigs(g->h), checks
  xs_updt_items(P.G, NG, N.act, I.nnod, I.sigtr, I.siga, P.sigs, const_cast<double*>(N.D),
                const_cast<double*>(N.sigr), C, start, stride);
  // dn = 0 as on coup_coef's first call (mod_cmfd.f90:25-33): every solve starts fresh
  {
    double* dn = const_cast<double*>(I.ap.dn);
    const long long ndn = (long long)NG * 6 * P.G.NB;
    for (long long q = start; q < ndn; q += stride) dn[q] = 0.0;
  }
  if (!team_barrier(C, size, rank)) return false;
  if (vld(&C->status)) return true;
  if (I.kern == ADP_KERN_SANM) sanm_consts_items(N, start, stride);
  assemble_items(I.ap, start, stride);
  init_flux_items(P, start, stride);
  if (!team_barrier(C, size, rank)) return false;

  for (int guard = 0; guard < 4 * P.nout + 8; ++guard) {
    outer_body<MIXED>(P, rank, size);
    if (!team_barrier(C, size, rank)) return false;
    if (vld(&C->status) || vld(&C->converged) || vld(&C->max_reached) || !vld(&C->nodal_due)) break;
    // nodal update (mod_cmfd.f90:339-383) and matrix_setup(0)
    tl_source_items(N, start, stride);
    if (!team_barrier(C, size, rank)) return false;
    node_prep_items<NG>(N, start, stride);
    if (!team_barrier(C, size, rank)) return false;
    NdBest best{0.0, 0x7fffffffffffffffLL, -1};
    interface_items<NG>(N, start, stride, best);
    nd_block_reduce(N, best, rank);
    if (!team_barrier(C, size, rank)) return false;
    if (rank == 0 && threadIdx.x < 32) nodal_finish_warp(N, size);
    if (!team_barrier(C, size, rank)) return false;
    if (vld(&C->status) || vld(&C->converged) || vld(&C->max_reached)) break;
    assemble_items(I.ap0, start, stride);
    if (!team_barrier(C, size, rank)) return false;
  }
  if (vld(&C->status) || !vld(&C->converged)) return true;

  // PowDis: p = sum_g max(0, phi sigf vdel), normalised to sum 1
  const BoxGeom& G = P.G;
  const double* phi = P.phi[vld(&C->cur)];
  double acc[1] = {0.0};
  for (int b = start; b < G.NB; b += stride) {
    double pw = 0.0;
    for (int g = 0; g < NG; ++g) {
      double q = phi[(size_t)g * P.NBH + b] * I.sigf[(size_t)g * G.NB + b] * G.vdel[b];
      if (q < 0.) q = 0.;
      pw = pw + q;
    }
    I.pbox[b] = pw;
    acc[0] += pw;
  }
  double tot[1];
  if (!grid_reduce<1, 0u>(C, size, rank, P.red, acc, tot)) return false;
  if (tot[0] <= 0.0) {
    if (lead) set_status(C, ADP_ERR_ZEROPOWER);
    return true;
  }
  for (int b = start; b < G.NB; b += stride) I.pbox[b] = I.pbox[b] / tot[0];
  return true;
}

template <bool MIXED, int NG, int THREADS>
__global__ void __launch_bounds__(THREADS, 1)
    k_batch(const BatchInst* __restrict__ insts, const BatchTask* __restrict__ tasks, const int* __restrict__ begin) {
  __shared__ __align__(16) BatchInst sI;
  const int t0 = begin[blockIdx.x], t1 = begin[blockIdx.x + 1];
  for (int t = t0; t < t1; ++t) {
    const BatchTask tk = tasks[t];
    __syncthreads();
    {
      const int* src = (const int*)(insts + tk.inst);
      int* dst = (int*)&sI;
      for (int i = threadIdx.x; i < (int)(sizeof(BatchInst) / 4); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const bool lead = tk.rank == 0 && threadIdx.x == 0;
    if (lead) sI.t_ns[0] = globaltimer_ns();
    solve_core<MIXED, NG>(sI, (unsigned)tk.rank, (unsigned)tk.size);
    if (lead) sI.t_ns[1] = globaltimer_ns();
  }
}

template <bool MIXED, int NG, int THREADS>
cudaError_t launch_batch_t(int blocks, const BatchInst* insts, const BatchTask* tasks, const int* begin,
                           cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_batch<MIXED, NG, THREADS>, insts, tasks, begin);
}

template <bool MIXED, int NG, int THREADS>
int batch_occupancy_t() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<MIXED, NG, THREADS>, THREADS, 0);
  return nb;
}

}  // namespace adp

namespace adp {

// Dispatch over the compiled group counts (1..4) and block sizes (256, 512).
template <bool MIXED>
cudaError_t batch_dispatch_launch(int ng, int threads, int blocks, const BatchInst* insts, const BatchTask* tasks,
                                  const int* begin, cudaStream_t st) {
  const bool big = threads == 512;
  switch (ng) {
    case 1: return big ? launch_batch_t<MIXED, 1, 512>(blocks, insts, tasks, begin, st)
                       : launch_batch_t<MIXED, 1, 256>(blocks, insts, tasks, begin, st);
    case 2: return big ? launch_batch_t<MIXED, 2, 512>(blocks, insts, tasks, begin, st)
                       : launch_batch_t<MIXED, 2, 256>(blocks, insts, tasks, begin, st);
    case 3: return big ? launch_batch_t<MIXED, 3, 512>(blocks, insts, tasks, begin, st)
                       : launch_batch_t<MIXED, 3, 256>(blocks, insts, tasks, begin, st);
    case 4: return big ? launch_batch_t<MIXED, 4, 512>(blocks, insts, tasks, begin, st)
                       : launch_batch_t<MIXED, 4, 256>(blocks, insts, tasks, begin, st);
    default: return cudaErrorInvalidValue;
  }
}

template <bool MIXED>
int batch_dispatch_occupancy(int ng, int threads) {
  const bool big = threads == 512;
  switch (ng) {
    case 1: return big ? batch_occupancy_t<MIXED, 1, 512>() : batch_occupancy_t<MIXED, 1, 256>();
    case 2: return big ? batch_occupancy_t<MIXED, 2, 512>() : batch_occupancy_t<MIXED, 2, 256>();
    case 3: return big ? batch_occupancy_t<MIXED, 3, 512>() : batch_occupancy_t<MIXED, 3, 256>();
    case 4: return big ? batch_occupancy_t<MIXED, 4, 512>() : batch_occupancy_t<MIXED, 4, 256>();
    default: return 0;
  }
}

}  // namespace adp
