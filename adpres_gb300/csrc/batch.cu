// Batched static solves (adp_batch_*): many independent cores in one
// persistent cooperative launch, replayed from a captured CUDA graph.
//
// The reference solves one core per process (control::forward,
// mod_control.f90:11-47); a batch owns one single-core handle per core (the
// same device state and the same per-core API for results) and runs all of
// them in one launch of k_batch (batch_kernel.cuh).  The schedule assigns
// each core a team of blocks and each block an ordered task list:
//   - weights: box rows x groups until a solve has been timed, then the
//     measured block time of each core (device clock, t_ns);
//   - team size: ceil(weight * grain / (total / blocks)), at most max_team;
//   - longest-first list scheduling: a core goes to the `size` least loaded
//     blocks and starts when the last of them is free.
// Since cores are placed in one global order and appended to the chosen
// blocks' lists in that order, every block's list is a subsequence of the
// same order and no cycle of teams waiting on each other can form.
// The autotuner (adp_batch_autotune) times the whole batch over block size,
// max_team and grain with measured weights and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/adpres_gb300.h"
#include "adp_kernels.h"
#include "handle.h"

namespace adp {
cudaError_t launch_batch_fp64(int ng, int threads, int minb, int blocks, const BatchInst* insts,
                              const BatchTask* tasks, const int* begin, cudaStream_t st);
cudaError_t launch_batch_mixed(int ng, int threads, int minb, int blocks, const BatchInst* insts,
                               const BatchTask* tasks, const int* begin, cudaStream_t st);
int batch_occupancy_fp64(int ng, int threads, int minb);
int batch_occupancy_mixed(int ng, int threads, int minb);

cudaError_t launch_batch(bool mixed, int ng, int threads, int minb, int blocks, const BatchInst* insts,
                         const BatchTask* tasks, const int* task_begin, cudaStream_t st) {
  return mixed ? launch_batch_mixed(ng, threads, minb, blocks, insts, tasks, task_begin, st)
               : launch_batch_fp64(ng, threads, minb, blocks, insts, tasks, task_begin, st);
}

int batch_max_blocks_per_sm(bool mixed, int ng, int threads, int minb) {
  return mixed ? batch_occupancy_mixed(ng, threads, minb) : batch_occupancy_fp64(ng, threads, minb);
}

bool batch_supported(int ng, int threads) { return ng >= 1 && ng <= 4 && (threads == 256 || threads == 512); }

// Control block of every core at the start of a solve: the state of a fresh
// process (k = 1, first-call start, barrier word 0).
__global__ void k_batch_init(const BatchInst* insts, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    OuterCtl* C = insts[i].op.ctl;
    OuterCtl c{};
    c.Ke = 1.0;
    c.need_prologue = 1;
    c.err_node = -1;
    *C = c;
    insts[i].t_ns[0] = 0;
    insts[i].t_ns[1] = 0;
  }
}

__global__ void k_batch_gather(const BatchInst* insts, int n, OuterCtl* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = *insts[i].op.ctl;
}

cudaError_t launch_batch_init(const BatchInst* insts, int n, cudaStream_t st) {
  k_batch_init<<<(n + 127) / 128, 128, 0, st>>>(insts, n);
  return cudaGetLastError();
}

cudaError_t launch_batch_gather(const BatchInst* insts, int n, OuterCtl* out, cudaStream_t st) {
  k_batch_gather<<<(n + 127) / 128, 128, 0, st>>>(insts, n, out);
  return cudaGetLastError();
}

}  // namespace adp

using namespace adp;

struct adp_batch {
  std::string err;
  int dev = 0, sms = 0, n = 0, ng = 0, kern = 0;
  bool mixed = false;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::vector<adp_handle*> core;
  std::vector<double> rows;          // box rows x groups per core
  std::vector<double> measured;      // block-ns per core from the last solve (0: none)
  // device
  BatchInst* d_inst = nullptr;
  unsigned long long* d_tns = nullptr;
  OuterCtl* d_res = nullptr;
  BatchTask* d_tasks = nullptr;
  int* d_begin = nullptr;
  size_t tasks_cap = 0;
  int begin_cap = 0;
  // pinned host
  OuterCtl* h_res = nullptr;
  unsigned long long* h_tns = nullptr;
  // schedule
  adp_batch_config cfg{};
  int blocks = 0;
  std::vector<BatchTask> tasks;
  std::vector<int> begin;
  std::vector<int> team;             // team size per core
  bool plan_ok = false;
  cudaGraphExec_t gexec = nullptr;
  bool graph_ok = false;
  double last_ms = 0.0;
};

namespace {

adp_status bfail(adp_batch* b, adp_status s, const std::string& m) {
  if (b) b->err = m;
  else adp::set_global_error(m);
  return s;
}

#define BCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return bfail(b, ADP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));           \
  } while (0)

void drop_graph(adp_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->graph_ok = false;
}

// Longest-first list scheduling with teams (see the file comment).
void make_plan(adp_batch* b) {
  const int n = b->n, B = b->blocks;
  std::vector<double> w(n);
  bool meas = true;
  for (int i = 0; i < n; ++i) meas = meas && b->measured[i] > 0.0;
  for (int i = 0; i < n; ++i) w[i] = meas ? b->measured[i] : b->rows[i];
  const double total = std::accumulate(w.begin(), w.end(), 0.0);
  const double avg = total / B;
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return w[a] > w[c]; });
  std::vector<double> load(B, 0.0);
  std::vector<std::vector<BatchTask>> lists(B);
  std::vector<int> idx(B);
  b->team.assign(n, 1);
  const int maxteam = std::max(1, std::min(b->cfg.max_team, B));
  const double grain = b->cfg.grain > 0 ? b->cfg.grain : 1.0;
  for (int i : order) {
    int s = (int)std::ceil(w[i] * grain / avg - 1e-9);
    s = std::max(1, std::min(s, maxteam));
    std::iota(idx.begin(), idx.end(), 0);
    std::partial_sort(idx.begin(), idx.begin() + s, idx.end(), [&](int a, int c) {
      return load[a] < load[c] || (load[a] == load[c] && a < c);
    });
    std::sort(idx.begin(), idx.begin() + s);
    double t0 = 0.0;
    for (int k = 0; k < s; ++k) t0 = std::max(t0, load[idx[k]]);
    const double t1 = t0 + w[i] / s;
    for (int k = 0; k < s; ++k) {
      lists[idx[k]].push_back(BatchTask{i, k, s, 0});
      load[idx[k]] = t1;
    }
    b->team[i] = s;
  }
  b->tasks.clear();
  b->begin.assign(B + 1, 0);
  for (int c = 0; c < B; ++c) {
    b->begin[c] = (int)b->tasks.size();
    b->tasks.insert(b->tasks.end(), lists[c].begin(), lists[c].end());
  }
  b->begin[B] = (int)b->tasks.size();
}

adp_status upload_plan(adp_batch* b) {
  if (b->tasks.size() > b->tasks_cap) {
    if (b->d_tasks) cudaFree(b->d_tasks);
    b->d_tasks = nullptr;
    b->tasks_cap = std::max(b->tasks.size(), (size_t)(2 * b->n));
    BCK(cudaMalloc((void**)&b->d_tasks, b->tasks_cap * sizeof(BatchTask)));
  }
  if ((int)b->begin.size() > b->begin_cap) {
    if (b->d_begin) cudaFree(b->d_begin);
    b->d_begin = nullptr;
    b->begin_cap = (int)b->begin.size();
    BCK(cudaMalloc((void**)&b->d_begin, b->begin_cap * sizeof(int)));
  }
  BCK(cudaMemcpy(b->d_tasks, b->tasks.data(), b->tasks.size() * sizeof(BatchTask), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_begin, b->begin.data(), b->begin.size() * sizeof(int), cudaMemcpyHostToDevice));
  return ADP_OK;
}

// The work of one solve on the batch's stream.
cudaError_t enqueue_solve(adp_batch* b) {
  cudaError_t e;
  if ((e = launch_batch_init(b->d_inst, b->n, b->st)) != cudaSuccess) return e;
  if ((e = launch_batch(b->mixed, b->ng, b->cfg.threads, b->cfg.blocks_per_sm, b->blocks, b->d_inst, b->d_tasks,
                        b->d_begin, b->st)) != cudaSuccess)
    return e;
  if ((e = launch_batch_gather(b->d_inst, b->n, b->d_res, b->st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(b->h_res, b->d_res, b->n * sizeof(OuterCtl), cudaMemcpyDeviceToHost, b->st)) != cudaSuccess)
    return e;
  return cudaMemcpyAsync(b->h_tns, b->d_tns, 2 * b->n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, b->st);
}

// Plan, upload and capture the solve as a graph (when cfg.use_graph).
adp_status prepare(adp_batch* b) {
  if (b->plan_ok) return ADP_OK;
  drop_graph(b);
  const int occ = batch_max_blocks_per_sm(b->mixed, b->ng, b->cfg.threads, b->cfg.blocks_per_sm);
  if (occ < 1) return bfail(b, ADP_ERR_CUDA, "batched kernel cannot be resident with this block size");
  b->blocks = std::min(b->sms * std::min(occ, std::max(1, b->cfg.blocks_per_sm)), kMaxBlocks);
  make_plan(b);
  adp_status s = upload_plan(b);
  if (s != ADP_OK) return s;
  if (b->cfg.use_graph) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t e2 = enqueue_solve(b);
      e = cudaStreamEndCapture(b->st, &g);
      if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      drop_graph(b);
      return bfail(b, ADP_ERR_CUDA, std::string("graph capture of the batched solve failed: ") + cudaGetErrorString(e));
    }
    b->graph_ok = true;
  }
  b->plan_ok = true;
  return ADP_OK;
}

}  // namespace

extern "C" {

size_t adp_batch_last_error(const adp_batch* b, char* buf, size_t len) {
  if (!b) return adp_last_error(nullptr, buf, len);
  const std::string& m = b->err;
  if (buf && len) {
    size_t k = std::min(len - 1, m.size());
    std::memcpy(buf, m.data(), k);
    buf[k] = 0;
  }
  return m.size();
}

adp_status adp_batch_destroy(adp_batch* b) {
  if (!b) return ADP_OK;
  cudaSetDevice(b->dev);
  if (b->st) cudaStreamSynchronize(b->st);
  drop_graph(b);
  for (adp_handle* h : b->core) adp_destroy(h);
  for (void* p : {(void*)b->d_inst, (void*)b->d_tns, (void*)b->d_res, (void*)b->d_tasks, (void*)b->d_begin})
    if (p) cudaFree(p);
  if (b->h_res) cudaFreeHost(b->h_res);
  if (b->h_tns) cudaFreeHost(b->h_tns);
  for (cudaEvent_t e : {b->e0, b->e1})
    if (e) cudaEventDestroy(e);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return ADP_OK;
}

adp_status adp_batch_create(int n, const adp_geom* geoms, const adp_opts* opts, adp_batch** out) {
  adp_batch* b = nullptr;
  if (n < 1 || !geoms || !opts || !out) return bfail(nullptr, ADP_ERR_INPUT, "adp_batch_create: bad arguments");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (opts[i].ng != opts[0].ng || opts[i].kern != opts[0].kern || opts[i].precision != opts[0].precision)
      return bfail(nullptr, ADP_ERR_UNSUPPORTED, "adp_batch_create: all cores need the same ng, kern and precision");
  }
  if (opts[0].ng < 1 || opts[0].ng > 4)
    return bfail(nullptr, ADP_ERR_UNSUPPORTED, "adp_batch_create: batched solves support 1..4 groups");
  b = new adp_batch();
  b->n = n;
  b->ng = opts[0].ng;
  b->kern = opts[0].kern;
  b->mixed = opts[0].precision == ADP_MIXED;
  cudaGetDevice(&b->dev);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, b->dev);
  b->sms = prop.multiProcessorCount;
  b->core.assign(n, nullptr);
  for (int i = 0; i < n; ++i) {
    adp_status s = adp_create(&geoms[i], &opts[i], &b->core[i]);
    if (s != ADP_OK) {
      char msg[512];
      adp_last_error(nullptr, msg, sizeof msg);
      adp_batch_destroy(b);
      return bfail(nullptr, s, "adp_batch_create: core " + std::to_string(i) + ": " + msg);
    }
  }
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&b->e0)) != cudaSuccess || (e = cudaEventCreate(&b->e1)) != cudaSuccess ||
      (e = cudaMalloc((void**)&b->d_inst, n * sizeof(BatchInst))) != cudaSuccess ||
      (e = cudaMalloc((void**)&b->d_tns, 2 * n * sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc((void**)&b->d_res, n * sizeof(OuterCtl))) != cudaSuccess ||
      (e = cudaMallocHost((void**)&b->h_res, n * sizeof(OuterCtl))) != cudaSuccess ||
      (e = cudaMallocHost((void**)&b->h_tns, 2 * n * sizeof(unsigned long long))) != cudaSuccess) {
    adp_batch_destroy(b);
    return bfail(nullptr, ADP_ERR_CUDA, std::string("adp_batch_create: ") + cudaGetErrorString(e));
  }
  std::vector<BatchInst> inst(n);
  b->rows.resize(n);
  b->measured.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    adp_handle* h = b->core[i];
    BatchInst& I = inst[i];
    std::memset(&I, 0, sizeof I);
    // the kernel forms D and sigr itself; chi, nu*fission and sigs (and
    // with them the handle's masks of all-zero planes) come from the host
    I.op = adp::outer_params(h, 0);
    I.op.do_nodal = h->o.kern != ADP_KERN_FDM;
    I.np = adp::nodal_params(h, 1);
    I.np.nd_blocks = 0;
    I.ap.G = adp::box_geom(h);
    I.ap.ng = h->ng;
    I.ap.with_coupling = 1;
    I.ap.D = h->d_D;
    I.ap.sigr = h->d_sigr;
    I.ap.df = h->d_df;
    I.ap.dn = h->d_dn;
    I.ap.A = h->d_A;
    I.ap.A32 = h->d_A32;
    I.ap.A2 = h->d_A2;
    I.ap.ctl = h->d_ctl;
    I.ap0 = I.ap;
    I.ap0.with_coupling = 0;
    I.sigtr = h->d_sigtr;
    I.siga = h->d_siga;
    I.sigf = h->d_sigf;
    I.pbox = h->d_pbox;
    I.t_ns = b->d_tns + 2 * i;
    I.kern = h->o.kern;
    I.nnod = h->nnod;
    b->rows[i] = (double)h->NB * h->ng;
  }
  if ((e = cudaMemcpy(b->d_inst, inst.data(), n * sizeof(BatchInst), cudaMemcpyHostToDevice)) != cudaSuccess) {
    adp_batch_destroy(b);
    return bfail(nullptr, ADP_ERR_CUDA, std::string("adp_batch_create: ") + cudaGetErrorString(e));
  }
  b->cfg.threads = 256;
  b->cfg.max_team = 8;
  b->cfg.grain = 1.0;
  b->cfg.blocks_per_sm = 1;
  b->cfg.use_graph = 1;
  *out = b;
  return ADP_OK;
}

adp_status adp_batch_set_xs(adp_batch* b, int i, int nmat, const double* sigtr, const double* siga, const double* nuf,
                            const double* sigf, const double* chi, const int* mat, const double* sigs,
                            const double* dc) {
  if (!b) return ADP_ERR_INPUT;
  if (i < 0 || i >= b->n) return bfail(b, ADP_ERR_INPUT, "adp_batch_set_xs: core index out of range");
  BCK(cudaSetDevice(b->dev));
  adp_status s = adp_xs_updt_nodes(b->core[i], nmat, sigtr, siga, nuf, sigf, chi, mat, sigs, dc);
  if (s != ADP_OK) {
    char msg[512];
    adp_last_error(b->core[i], msg, sizeof msg);
    return bfail(b, s, "core " + std::to_string(i) + ": " + msg);
  }
  return ADP_OK;
}

adp_status adp_batch_set_config(adp_batch* b, const adp_batch_config* c) {
  if (!b || !c) return ADP_ERR_INPUT;
  if (!batch_supported(b->ng, c->threads)) return bfail(b, ADP_ERR_INPUT, "adp_batch_set_config: threads must be 256 or 512");
  if (c->max_team < 1 || c->blocks_per_sm < 1 || !(c->grain > 0))
    return bfail(b, ADP_ERR_INPUT, "adp_batch_set_config: max_team, blocks_per_sm >= 1 and grain > 0");
  b->cfg = *c;
  b->plan_ok = false;
  return ADP_OK;
}

adp_status adp_batch_get_config(const adp_batch* b, adp_batch_config* c) {
  if (!b || !c) return ADP_ERR_INPUT;
  *c = b->cfg;
  return ADP_OK;
}

adp_status adp_batch_solve(adp_batch* b, adp_batch_result* res, double* device_ms) {
  if (!b) return ADP_ERR_INPUT;
  BCK(cudaSetDevice(b->dev));
  for (int i = 0; i < b->n; ++i)
    if (!b->core[i]->xs_set) return bfail(b, ADP_ERR_STATE, "adp_batch_solve: cross sections of core " + std::to_string(i) + " not set");
  adp_status s = prepare(b);
  if (s != ADP_OK) return s;
  BCK(cudaEventRecord(b->e0, b->st));
  if (b->graph_ok) BCK(cudaGraphLaunch(b->gexec, b->st));
  else BCK(enqueue_solve(b));
  BCK(cudaEventRecord(b->e1, b->st));
  BCK(cudaStreamSynchronize(b->st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->e0, b->e1);
  b->last_ms = ms;
  if (device_ms) *device_ms = ms;
  adp_status worst = ADP_OK;
  for (int i = 0; i < b->n; ++i) {
    const OuterCtl& c = b->h_res[i];
    const unsigned long long t0 = b->h_tns[2 * i], t1 = b->h_tns[2 * i + 1];
    const double t = (t1 > t0) ? (double)(t1 - t0) : 0.0;
    b->measured[i] = t * b->team[i];
    adp_status st = (adp_status)c.status;
    if (st == ADP_OK && !c.converged) st = ADP_ERR_MAXOUTER;
    if (st != ADP_OK && worst == ADP_OK) worst = st;
    if (res) {
      adp_batch_result& r = res[i];
      r.status = st;
      r.converged = c.converged;
      r.outers = c.p;
      r.nodal_updates = c.nodal_updates;
      r.keff = c.Ke;
      r.ser = c.ser;
      r.fer = c.fer;
      r.ndmax = c.ndmax;
      r.device_ms = t * 1e-6;
      r.team = b->team[i];
    }
    // the core's handle now holds a solved state
    adp_handle* h = b->core[i];
    h->started[0] = true;
    h->fwd_ok = st == ADP_OK;
  }
  if (worst != ADP_OK) return bfail(b, worst, "adp_batch_solve: at least one core failed (see the per-core status)");
  return ADP_OK;
}

adp_status adp_batch_autotune(adp_batch* b, adp_batch_config* best_out, double* best_ms) {
  if (!b) return ADP_ERR_INPUT;
  const adp_batch_config base = b->cfg;
  // measured weights from one solve with the current settings
  adp_status s = adp_batch_solve(b, nullptr, nullptr);
  if (s != ADP_OK) return s;
  adp_batch_config best = base;
  double best_t = 1e300;
  // kernel shapes: (threads, blocks per SM) = (256, 1), (256, 2), (512, 1)
  const int shapes[3][2] = {{256, 1}, {256, 2}, {512, 1}};
  const int teams[3] = {2, 8, 32};
  const double grains[2] = {1.0, 4.0};
  const std::vector<double> meas = b->measured;
  for (const auto& sh : shapes) {
    if (batch_max_blocks_per_sm(b->mixed, b->ng, sh[0], sh[1]) < sh[1]) continue;
    for (int mt : teams)
      for (double gr : grains) {
        adp_batch_config c = base;
        c.threads = sh[0];
        c.max_team = mt;
        c.grain = gr;
        c.blocks_per_sm = sh[1];
        s = adp_batch_set_config(b, &c);
        if (s != ADP_OK) return s;
        b->measured = meas;   // every candidate plans from the same measurement
        double ms = 0.0;
        s = adp_batch_solve(b, nullptr, &ms);
        if (s != ADP_OK) return s;
        if (ms < best_t) {
          best_t = ms;
          best = c;
        }
      }
  }
  b->measured = meas;
  s = adp_batch_set_config(b, &best);
  if (s != ADP_OK) return s;
  if (best_out) *best_out = best;
  if (best_ms) *best_ms = best_t;
  return ADP_OK;
}

adp_status adp_batch_core(adp_batch* b, int i, adp_handle** h) {
  if (!b || !h) return ADP_ERR_INPUT;
  if (i < 0 || i >= b->n) return bfail(b, ADP_ERR_INPUT, "adp_batch_core: core index out of range");
  *h = b->core[i];
  return ADP_OK;
}

int adp_batch_trace(adp_batch* b, int i, int cap, double* k, double* ser, double* fer, int* flags, double* ndmax) {
  if (!b || i < 0 || i >= b->n || cap < 0) return -1;
  if (cudaSetDevice(b->dev) != cudaSuccess) return -1;
  adp_handle* h = b->core[i];
  const int n = std::min(std::min(b->h_res[i].p, cap), h->o.nout);
  if (n <= 0) return 0;
  if ((k && cudaMemcpy(k, h->d_tr_k, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (ser && cudaMemcpy(ser, h->d_tr_ser, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (fer && cudaMemcpy(fer, h->d_tr_fer, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (flags && cudaMemcpy(flags, h->d_tr_flags, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (ndmax && cudaMemcpy(ndmax, h->d_tr_ndmax, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess))
    return -1;
  return n;
}

adp_status adp_batch_power(adp_batch* b, int i, double* p) {
  if (!b || !p) return ADP_ERR_INPUT;
  if (i < 0 || i >= b->n) return bfail(b, ADP_ERR_INPUT, "adp_batch_power: core index out of range");
  BCK(cudaSetDevice(b->dev));
  adp_handle* h = b->core[i];
  std::vector<double> box(h->NB);
  BCK(cudaMemcpy(box.data(), h->d_pbox, (size_t)h->NB * 8, cudaMemcpyDeviceToHost));
  for (int n = 0; n < h->nnod; ++n) p[n] = box[h->node2box[n]];
  return ADP_OK;
}

}  // extern "C"
