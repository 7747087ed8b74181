// Single-core nodal kernels over the item functions of nodal_body.cuh.
#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"
#include "nodal_body.cuh"

namespace adp {

#define ADP_GRID_START (blockIdx.x * blockDim.x + threadIdx.x)
#define ADP_GRID_STRIDE (gridDim.x * blockDim.x)

__global__ void k_sanm_consts(NodalParams P) { sanm_consts_items(P, ADP_GRID_START, ADP_GRID_STRIDE); }

cudaError_t launch_sanm_consts(const NodalParams& P, cudaStream_t st) {
  int total = P.nnod * 3 * P.ng;
  int blocks = (total + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  k_sanm_consts<<<blocks, 256, 0, st>>>(P);
  return cudaGetLastError();
}

__global__ void k_tl_source(NodalParams P) { tl_source_items(P, ADP_GRID_START, ADP_GRID_STRIDE); }

template <int NG>
__global__ void __launch_bounds__(128) k_node_prep(NodalParams P) {
  node_prep_items<NG>(P, ADP_GRID_START, ADP_GRID_STRIDE);
}

template <int NG>
__global__ void __launch_bounds__(128) k_interface(NodalParams P) {
  NdBest best{0.0, 0x7fffffffffffffffLL, -1};
  interface_items<NG>(P, ADP_GRID_START, ADP_GRID_STRIDE, best);
  nd_block_reduce(P, best, blockIdx.x);
}

__global__ void k_nodal_finish(NodalParams P) {
  if (threadIdx.x >= 32 || blockIdx.x != 0) return;
  nodal_finish_warp(P, P.nd_blocks);
}

template <int NG>
static cudaError_t nodal_ng(const NodalParams& P, cudaStream_t st) {
  const int total = P.nnod * 3;
  int blocks1 = (P.nnod * NG + 255) / 256;
  if (blocks1 > 8192) blocks1 = 8192;
  k_tl_source<<<blocks1, 256, 0, st>>>(P);
  int blocks2 = (total + 127) / 128;
  if (blocks2 > 8192) blocks2 = 8192;
  k_node_prep<NG><<<blocks2, 128, 0, st>>>(P);
  NodalParams Q = P;
  int blocks3 = (total + 127) / 128;
  if (blocks3 > kMaxBlocks) blocks3 = kMaxBlocks;
  Q.nd_blocks = blocks3;
  k_interface<NG><<<blocks3, 128, 0, st>>>(Q);
  k_nodal_finish<<<1, 32, 0, st>>>(Q);
  return cudaGetLastError();
}

// The stages of the update before the faces (get_source, then per node and
// direction get_B, a2, a4, L1) at the current state, leaving dn unchanged:
// the forward quantities the derivative of the update reads.
template <int NG>
static cudaError_t nodal_prep_ng(const NodalParams& P, cudaStream_t st) {
  int blocks1 = (P.nnod * NG + 255) / 256;
  if (blocks1 > 8192) blocks1 = 8192;
  k_tl_source<<<blocks1, 256, 0, st>>>(P);
  int blocks2 = (P.nnod * 3 + 127) / 128;
  if (blocks2 > 8192) blocks2 = 8192;
  k_node_prep<NG><<<blocks2, 128, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_nodal_prep(const NodalParams& P, cudaStream_t st) {
  switch (P.ng) {
    case 1: return nodal_prep_ng<1>(P, st);
    case 2: return nodal_prep_ng<2>(P, st);
    case 3: return nodal_prep_ng<3>(P, st);
    case 4: return nodal_prep_ng<4>(P, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_nodal(const NodalParams& P, cudaStream_t st) {
  switch (P.ng) {
    case 1: return nodal_ng<1>(P, st);
    case 2: return nodal_ng<2>(P, st);
    case 3: return nodal_ng<3>(P, st);
    case 4: return nodal_ng<4>(P, st);
    case 5: return nodal_ng<5>(P, st);
    case 6: return nodal_ng<6>(P, st);
    case 7: return nodal_ng<7>(P, st);
    case 8: return nodal_ng<8>(P, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace adp
