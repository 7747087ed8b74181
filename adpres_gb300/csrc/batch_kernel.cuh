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

// The nodal update of one core (mod_cmfd.f90:339-383) and matrix_setup(0),
// by the core's team.  Not inlined: it runs once per nodal interval, and as
// a function of its own its register needs (the 2G x 2G face systems) do
// not press on the register allocation of the outer-iteration loop, which
// then fits the two-blocks-per-SM budget.  Returns: 0 go on, 1 stop (a
// status, convergence or nout), -1 a barrier wait ran out of time.
template <int NG>
__device__ __noinline__ int nodal_stage(const BatchInst& I, unsigned rank, unsigned size) {
  const NodalParams& N = I.np;
  OuterCtl* C = I.op.ctl;
  const int start = rank * blockDim.x + threadIdx.x, stride = size * blockDim.x;
  tl_source_items(N, start, stride);
  if (!team_barrier(C, size, rank)) return -1;
  node_prep_items<NG>(N, start, stride);
  if (!team_barrier(C, size, rank)) return -1;
  NdBest best{0.0, 0x7fffffffffffffffLL, -1};
  interface_items<NG>(N, start, stride, best);
  nd_block_reduce(N, best, rank);
  if (!team_barrier(C, size, rank)) return -1;
  if (rank == 0 && threadIdx.x < 32) nodal_finish_warp(N, size);
  if (!team_barrier(C, size, rank)) return -1;
  if (vld(&C->status) || vld(&C->converged) || vld(&C->max_reached)) return 1;
  assemble_items(I.ap0, start, stride);
  if (!team_barrier(C, size, rank)) return -1;
  return 0;
}

// XS_updt, dn = 0, the SANM constants, matrix_setup(1) and the first-call
// start of one core (not inlined, as the nodal stage).  Returns 0 go on,
// 1 stop (a cross-section check failed), -1 a barrier wait ran out of time.
template <int NG>
__device__ __noinline__ int setup_stage(const BatchInst& I, unsigned rank, unsigned size) {
  const OuterParams& P = I.op;
  const NodalParams& N = I.np;
  OuterCtl* C = P.ctl;
  const int start = rank * blockDim.x + threadIdx.x, stride = size * blockDim.x;
  // XS_updt: D = 1/(3 sigtr), sigr = siga + sum_{h/=g} sigs(g->h), checks
  xs_updt_items(P.G, NG, N.act, I.nnod, I.sigtr, I.siga, P.sigs, const_cast<double*>(N.D),
                const_cast<double*>(N.sigr), C, start, stride);
  // dn = 0 as on coup_coef's first call (mod_cmfd.f90:25-33): every solve starts fresh
  {
    double* dn = const_cast<double*>(I.ap.dn);
    const long long ndn = (long long)NG * 6 * P.G.NB;
    for (long long q = start; q < ndn; q += stride) dn[q] = 0.0;
  }
  if (!team_barrier(C, size, rank)) return -1;
  if (vld(&C->status)) return 1;
  if (I.kern == ADP_KERN_SANM) sanm_consts_items(N, start, stride);
  assemble_items(I.ap, start, stride);
  init_flux_items(P, start, stride);
  if (!team_barrier(C, size, rank)) return -1;
  return 0;
}

template <int NG>
__device__ __noinline__ bool power_stage(const BatchInst& I, unsigned rank, unsigned size);

// Everything after the cross-section update; false when a barrier wait ran
// out of time (the core's status then says ADP_ERR_TIMEOUT).
template <bool MIXED, int NG>
__device__ __forceinline__ bool solve_core(const BatchInst& I, unsigned rank, unsigned size) {
  const OuterParams& P = I.op;
  OuterCtl* C = P.ctl;

  const int su = setup_stage<NG>(I, rank, size);
  if (su < 0) return false;
  if (su > 0) return true;

  for (int guard = 0; guard < 4 * P.nout + 8; ++guard) {
    outer_body<MIXED>(P, rank, size);
    if (!team_barrier(C, size, rank)) return false;
    if (vld(&C->status) || vld(&C->converged) || vld(&C->max_reached) || !vld(&C->nodal_due)) break;
    const int ns = nodal_stage<NG>(I, rank, size);
    if (ns < 0) return false;
    if (ns > 0) break;
  }
  if (vld(&C->status) || !vld(&C->converged)) return true;
  return power_stage<NG>(I, rank, size);
}

// PowDis: p = sum_g max(0, phi sigf vdel), normalised to sum 1 (not
// inlined, as the nodal stage).
template <int NG>
__device__ __noinline__ bool power_stage(const BatchInst& I, unsigned rank, unsigned size) {
  const OuterParams& P = I.op;
  OuterCtl* C = P.ctl;
  const int start = rank * blockDim.x + threadIdx.x, stride = size * blockDim.x;
  const bool lead = rank == 0 && threadIdx.x == 0;
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

// MINB: blocks per SM the register budget is sized for (1, or 2 for
// 256-thread blocks: 128 registers, two cores' teams sharing an SM).
template <bool MIXED, int NG, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
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
    // The core's time runs from the arrival of the last block of its team
    // (every member raises the start to its own arrival; the time a member
    // waited for the others is not the core's work) to rank 0's end.
    if (threadIdx.x == 0) atomicMax(sI.t_ns, globaltimer_ns());
    solve_core<MIXED, NG>(sI, (unsigned)tk.rank, (unsigned)tk.size);
    if (tk.rank == 0 && threadIdx.x == 0) sI.t_ns[1] = globaltimer_ns();
  }
}

template <bool MIXED, int NG, int THREADS, int MINB>
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
  return cudaLaunchKernelEx(&cfg, k_batch<MIXED, NG, THREADS, MINB>, insts, tasks, begin);
}

template <bool MIXED, int NG, int THREADS, int MINB>
int batch_occupancy_t() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<MIXED, NG, THREADS, MINB>, THREADS, 0);
  return nb;
}

}  // namespace adp

namespace adp {

// Dispatch over the compiled group counts (1..4) and kernel shapes: 256
// threads sized for one or two blocks per SM, or 512 threads.
template <bool MIXED, int NG>
cudaError_t batch_launch_ng(int threads, int minb, int blocks, const BatchInst* insts, const BatchTask* tasks,
                            const int* begin, cudaStream_t st) {
  if (threads == 512) return launch_batch_t<MIXED, NG, 512, 1>(blocks, insts, tasks, begin, st);
  if (minb >= 2) return launch_batch_t<MIXED, NG, 256, 2>(blocks, insts, tasks, begin, st);
  return launch_batch_t<MIXED, NG, 256, 1>(blocks, insts, tasks, begin, st);
}

template <bool MIXED, int NG>
int batch_occupancy_ng(int threads, int minb) {
  if (threads == 512) return batch_occupancy_t<MIXED, NG, 512, 1>();
  if (minb >= 2) return batch_occupancy_t<MIXED, NG, 256, 2>();
  return batch_occupancy_t<MIXED, NG, 256, 1>();
}

template <bool MIXED>
cudaError_t batch_dispatch_launch(int ng, int threads, int minb, int blocks, const BatchInst* insts,
                                  const BatchTask* tasks, const int* begin, cudaStream_t st) {
  switch (ng) {
    case 1: return batch_launch_ng<MIXED, 1>(threads, minb, blocks, insts, tasks, begin, st);
    case 2: return batch_launch_ng<MIXED, 2>(threads, minb, blocks, insts, tasks, begin, st);
    case 3: return batch_launch_ng<MIXED, 3>(threads, minb, blocks, insts, tasks, begin, st);
    case 4: return batch_launch_ng<MIXED, 4>(threads, minb, blocks, insts, tasks, begin, st);
    default: return cudaErrorInvalidValue;
  }
}

template <bool MIXED>
int batch_dispatch_occupancy(int ng, int threads, int minb) {
  switch (ng) {
    case 1: return batch_occupancy_ng<MIXED, 1>(threads, minb);
    case 2: return batch_occupancy_ng<MIXED, 2>(threads, minb);
    case 3: return batch_occupancy_ng<MIXED, 3>(threads, minb);
    case 4: return batch_occupancy_ng<MIXED, 4>(threads, minb);
    default: return 0;
  }
}

}  // namespace adp
