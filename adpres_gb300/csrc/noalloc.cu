// adp_power_noalloc: the PowDis kernels (k_power_nodes / k_power_norm) run on
// device arrays owned by the caller, with their scratch -- the per-block
// partial sums of the total power and a status word -- in a fixed array of
// device memory that belongs to this library.  It allocates nothing, for
// callers that cannot call cudaMalloc: a host whose device memory is handed
// out by another allocator (a framework's caching allocator, or a budget
// fixed at start-up), or a code path where cudaMalloc/cudaFree and their
// implicit device synchronisation are not acceptable.
//
// The array below is held by every GPU that loads the library, until the
// process exits.  Every call uses the same array: two calls whose work
// overlaps on the GPU (on different streams, or from different host threads)
// race on it; serialise them.  The status word is cleared at the start of
// each call; the partial sums are fully rewritten by each call.
#include <cuda_runtime.h>

#include <climits>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"

namespace adp {
void set_global_error(const std::string& msg);
}

namespace {

using namespace adp;

// Partial sums of up to kMaxBlocks blocks, then room for the status word.
constexpr size_t kPartialsDoubles = kMaxBlocks;
constexpr size_t kStatusDoubles = 32;                       // 256 bytes
constexpr size_t kScratchDoubles = kPartialsDoubles + kStatusDoubles;  // 8,448 bytes
static_assert(sizeof(OuterCtl) <= kStatusDoubles * sizeof(double), "status area too small");

static __device__ __align__(256) double g_power_scratch[kScratchDoubles];

// Device address of g_power_scratch per device.  In host code the array's
// name is only a host-side stand-in, so the address is looked up once per
// device (with that device current) and passed to the kernels.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {};

adp_status fail(adp_status s, const std::string& msg) {
  set_global_error(msg);
  return s;
}

}  // namespace

extern "C" adp_status adp_power_noalloc(int nnod, int ng, const double* f0, const double* sigf, const double* vdel,
                                        double* p, void* stream) {
  if (nnod < 1 || ng < 1)
    return fail(ADP_ERR_INPUT, "adp_power_noalloc: nnod and ng must be at least 1");
  if (ng > kMaxGroups)
    return fail(ADP_ERR_INPUT, "adp_power_noalloc: ng is beyond the maximum of 8 groups");
  if ((long long)nnod * ng > (long long)INT_MAX)
    return fail(ADP_ERR_INPUT, "adp_power_noalloc: nnod * ng is beyond the maximum of 2^31 - 1 values");
  if (!f0 || !sigf || !vdel || !p) return fail(ADP_ERR_INPUT, "adp_power_noalloc: null array");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(ADP_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(ADP_ERR_CUDA, "adp_power_noalloc: device ordinal out of range");
  void* base = nullptr;
  {
    // First call on this device: resolve the scratch array's device address.
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_dev[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_power_scratch);
      if (e != cudaSuccess || !ptr)
        return fail(ADP_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      g_scratch_dev[dev] = ptr;
    }
    base = g_scratch_dev[dev];
  }
  double* partials = (double*)base;
  OuterCtl* status = (OuterCtl*)((double*)base + kPartialsDoubles);
  cudaStream_t st = (cudaStream_t)stream;
  // The same box description the handle's PowDis uses, with the node list as
  // the box: PowDis reads only the node count and the node volumes.
  BoxGeom G;
  std::memset(&G, 0, sizeof G);
  G.NB = nnod;
  G.ng = ng;
  G.vdel = vdel;
  e = cudaMemsetAsync(&status->status, 0, sizeof(int), st);
  if (e == cudaSuccess) e = launch_power(G, ng, (long long)nnod, f0, sigf, p, partials, status, st);
  int code = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&code, &status->status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(ADP_ERR_CUDA, std::string("adp_power_noalloc: ") + cudaGetErrorString(e));
  if (code == ADP_ERR_ZEROPOWER) return fail(ADP_ERR_ZEROPOWER, "total nodes power is zero or less");
  if (code != 0) return fail((adp_status)code, "adp_power_noalloc: device error");
  return ADP_OK;
}
