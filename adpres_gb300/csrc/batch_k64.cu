// FP64 instances of the batched kernel (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace adp {

cudaError_t launch_batch_fp64(int ng, int threads, int minb, int blocks, const BatchInst* insts,
                              const BatchTask* tasks, const int* begin, cudaStream_t st) {
  return batch_dispatch_launch<false>(ng, threads, minb, blocks, insts, tasks, begin, st);
}

int batch_occupancy_fp64(int ng, int threads, int minb) {
  return batch_dispatch_occupancy<false>(ng, threads, minb);
}

}  // namespace adp
