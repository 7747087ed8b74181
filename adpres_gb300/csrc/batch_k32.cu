// Mixed-precision instances of the batched kernel (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace adp {

cudaError_t launch_batch_mixed(int ng, int threads, int minb, int blocks, const BatchInst* insts,
                              const BatchTask* tasks, const int* begin, cudaStream_t st) {
  return batch_dispatch_launch<true>(ng, threads, minb, blocks, insts, tasks, begin, st);
}

int batch_occupancy_mixed(int ng, int threads, int minb) {
  return batch_dispatch_occupancy<true>(ng, threads, minb);
}

}  // namespace adp
