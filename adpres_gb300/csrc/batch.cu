// Batched static solves (adp_batch_*): many independent cores in one
// persistent cooperative launch, replayed from a captured CUDA graph.
//
// The reference solves one core per process (control::forward,
// mod_control.f90:11-47); a batch owns one single-core handle per core (the
// same device state and the same per-core API for results) and runs all of
// them in one launch of k_batch (batch_kernel.cuh).  The schedule assigns
// each core a team of blocks and each block an ordered task list, by
// longest-first list scheduling: a core goes to the `size` least loaded
// blocks and starts when the last of them is free.
//   - Before any solve is timed: weights box rows x groups, team size
//     ceil(weight * grain / (total / blocks)), at most max_team.
//   - Once timed: every core's time at each (kernel shape, team size) it
//     ran at is kept (device clock, t_ns: from the arrival of the last
//     block of its team to its end).  Its duration on s blocks is that time,
//     or the time at the nearest size scaled by the model
//     t(s) = A (1/s + kappa), kappa fitted to all cores timed at two sizes.
//     For a target end T each core (longest first) takes the smallest team,
//     at most max_team, that ends by T on the least loaded blocks (else the
//     one that ends earliest); T is scanned over [1, 1.3] x a lower bound
//     (the least block-time of all cores over the blocks, the longest core
//     at max_team) and the plan with the earliest predicted end is kept.
// Since cores are placed in one global order and appended to the chosen
// blocks' lists in that order, every block's list is a subsequence of the
// same order and no cycle of teams waiting on each other can form.
// The autotuner (adp_batch_autotune) times the whole batch over kernel
// shape and max_team and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
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
  // per core: ns of its solves by kernel shape and team size (shape_key)
  std::vector<std::map<int, double>> took;
  std::vector<double> last_t;        // per core: ns of the last solve (0: none) ...
  std::vector<int> last_team;        // ... on a team of this size
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
  bool keep_tasks = false;           // re-capture without re-planning
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

// Key of a time in adp_batch::took: kernel shape and team size.
int shape_key(const adp_batch_config& c, int s) { return ((c.threads / 256) * 8 + c.blocks_per_sm) * 65536 + s; }

// Times of core i in the current kernel shape: team size -> ns.
std::map<int, double> times_here(const adp_batch* b, int i) {
  std::map<int, double> m;
  const int lo = shape_key(b->cfg, 0), hi = shape_key(b->cfg, 65535);
  for (auto it = b->took[i].lower_bound(lo); it != b->took[i].end() && it->first <= hi; ++it)
    m[it->first - lo] = it->second;
  return m;
}

// Team overhead kappa of the duration model t(s) = A (1/s + kappa): least
// squares over every pair of team sizes some core was timed at (kappa in
// [0, 0.3] by steps of 0.002); kDefaultKappa when no core has two sizes.
constexpr double kDefaultKappa = 0.03;

double fit_kappa(const adp_batch* b) {
  std::vector<double> r, q0, q1;   // t(s1)/t(s0) with 1/s0, 1/s1
  for (int i = 0; i < b->n; ++i) {
    const std::map<int, double> m = times_here(b, i);
    for (auto a = m.begin(); a != m.end(); ++a)
      for (auto c = std::next(a); c != m.end(); ++c) {
        r.push_back(c->second / a->second);
        q0.push_back(1.0 / a->first);
        q1.push_back(1.0 / c->first);
      }
  }
  if (r.empty()) return kDefaultKappa;
  double best = kDefaultKappa, err_best = 1e300;
  for (int j = 0; j <= 150; ++j) {
    const double k = 0.002 * j;
    double e = 0.0;
    for (size_t p = 0; p < r.size(); ++p) {
      const double d = r[p] - (q1[p] + k) / (q0[p] + k);
      e += d * d;
    }
    if (e < err_best) {
      err_best = e;
      best = k;
    }
  }
  return best;
}

// Predicted duration of core i on a team of s blocks: its time at s when
// timed in this kernel shape, else the time at the nearest size timed (or
// of the last solve, in any shape) scaled by (1/s + kappa) / (1/s0 + kappa).
double duration(const adp_batch* b, int i, int s, double kappa) {
  const std::map<int, double> m = times_here(b, i);
  auto it = m.find(s);
  if (it != m.end()) return it->second;
  int s0 = b->last_team[i];
  double t0 = b->last_t[i];
  double gap = 1e300;
  for (const auto& e : m) {
    const double g = std::fabs(std::log((double)e.first / s));
    if (g < gap) {
      gap = g;
      s0 = e.first;
      t0 = e.second;
    }
  }
  return t0 * (1.0 / s + kappa) / (1.0 / s0 + kappa);
}

struct Plan {
  std::vector<std::vector<BatchTask>> lists;
  std::vector<int> team;
  double makespan = 0.0;
};

// One list schedule: cores longest first, each on the `size` least loaded
// blocks (ties to the lower index), starting when the last of them is free.
// size(i, sorted loads) picks the team size.
template <class SizeRule>
Plan list_schedule(int n, int B, const std::vector<int>& order, SizeRule size,
                   const std::function<double(int, int)>& dur) {
  Plan P;
  P.lists.assign(B, {});
  P.team.assign(n, 1);
  std::vector<double> load(B, 0.0);
  std::vector<int> idx(B);
  for (int i : order) {
    std::iota(idx.begin(), idx.end(), 0);
    const int smax = size.cap;
    std::partial_sort(idx.begin(), idx.begin() + smax, idx.end(), [&](int a, int c) {
      return load[a] < load[c] || (load[a] == load[c] && a < c);
    });
    const int s = size(i, load, idx);
    std::sort(idx.begin(), idx.begin() + s);
    double t0 = 0.0;
    for (int k = 0; k < s; ++k) t0 = std::max(t0, load[idx[k]]);
    const double t1 = t0 + dur(i, s);
    for (int k = 0; k < s; ++k) {
      P.lists[idx[k]].push_back(BatchTask{i, k, s, 0});
      load[idx[k]] = t1;
    }
    P.team[i] = s;
  }
  P.makespan = *std::max_element(load.begin(), load.end());
  return P;
}

// Longest-first list scheduling with teams (see the file comment), on the
// host alone: n cores on B blocks, teams of at most max_team.  Untimed
// (dur empty): weights `rows`, team size from the grain.  Timed: dur(i, s)
// is core i's duration on s blocks.
Plan plan_schedule(int n, int B, int max_team, double grain_cfg, const std::vector<double>& rows,
                   const std::function<double(int, int)>& dur_model) {
  const int maxteam = std::max(1, std::min(max_team, B));
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  Plan P;
  if (!dur_model) {
    // before any solve is timed: weights box rows x groups, team size from
    // the grain
    const std::vector<double>& w = rows;
    const double avg = std::accumulate(w.begin(), w.end(), 0.0) / B;
    const double grain = grain_cfg > 0 ? grain_cfg : 1.0;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return w[a] > w[c]; });
    struct Grain {
      int cap;
      const std::vector<double>& w;
      double avg, grain;
      int operator()(int i, const std::vector<double>&, const std::vector<int>&) const {
        return std::max(1, std::min((int)std::ceil(w[i] * grain / avg - 1e-9), cap));
      }
    } rule{maxteam, w, avg, grain};
    return list_schedule(n, B, order, rule, [&](int i, int s) { return w[i] / s; });
  }
  // timed: for a target end T each core takes the smallest team that ends
  // by T on the least loaded blocks (else the team that ends earliest); T
  // runs over [lower bound, 1.3 x lower bound] and the plan with the
  // earliest predicted end is kept.  Durations per core and team size are
  // formed once.
  std::vector<double> dt((size_t)n * (maxteam + 1));
  for (int i = 0; i < n; ++i)
    for (int s = 1; s <= maxteam; ++s) dt[(size_t)i * (maxteam + 1) + s] = dur_model(i, s);
  std::function<double(int, int)> dur = [&](int i, int s) { return dt[(size_t)i * (maxteam + 1) + s]; };
  double work = 0.0, longest = 0.0;
  for (int i = 0; i < n; ++i) {
    double wmin = 1e300;
    for (int s = 1; s <= maxteam; ++s) wmin = std::min(wmin, s * dur(i, s));
    work += wmin;
    longest = std::max(longest, dur(i, maxteam));
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return dur(a, 1) > dur(c, 1); });
  const double lb = std::max(work / B, longest);
  struct Fill {
    int cap;
    double T;
    const std::function<double(int, int)>& dur;
    int operator()(int i, const std::vector<double>& load, const std::vector<int>& idx) const {
      int best = 1;
      double fbest = 1e300;
      for (int s = 1; s <= cap; ++s) {
        const double f = load[idx[s - 1]] + dur(i, s);
        if (f <= T) return s;
        if (f < fbest) {
          fbest = f;
          best = s;
        }
      }
      return best;
    }
  };
  // 61 targets 0.5% apart; fewer (at least 9, over the same range) when
  // cores x blocks is large, to bound the host time of a plan
  const int nt = std::max(9, std::min(61, (int)(2.0e7 / ((double)n * B))));
  bool have = false;
  for (int j = 0; j < nt; ++j) {
    Plan Q = list_schedule(n, B, order, Fill{maxteam, lb * (1.0 + 0.3 * j / (nt - 1)), dur}, dur);
    if (!have || Q.makespan < P.makespan) {
      P = std::move(Q);
      have = true;
    }
  }
  return P;
}

// The batch's schedule from its cores' times (see the file comment).
void make_plan(adp_batch* b) {
  const int n = b->n, B = b->blocks;
  bool meas = true;
  for (int i = 0; i < n; ++i) meas = meas && b->last_t[i] > 0.0;
  std::function<double(int, int)> dur;
  double kappa = 0.0;
  if (meas) {
    kappa = fit_kappa(b);
    dur = [b, &kappa](int i, int s) { return duration(b, i, s, kappa); };
  }
  const Plan P = plan_schedule(n, B, b->cfg.max_team, b->cfg.grain, b->rows, dur);
  b->team = P.team;
  b->tasks.clear();
  b->begin.assign(B + 1, 0);
  for (int c = 0; c < B; ++c) {
    b->begin[c] = (int)b->tasks.size();
    b->tasks.insert(b->tasks.end(), P.lists[c].begin(), P.lists[c].end());
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
  if (!b->keep_tasks) make_plan(b);
  b->keep_tasks = false;
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
  b->took.assign(n, {});
  b->last_t.assign(n, 0.0);
  b->last_team.assign(n, 1);
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
  // a change of use_graph alone keeps the schedule (the same tasks, so the
  // same results to the bit); any other call re-plans from the latest times
  b->keep_tasks = c->threads == b->cfg.threads && c->max_team == b->cfg.max_team && c->grain == b->cfg.grain &&
                  c->blocks_per_sm == b->cfg.blocks_per_sm && c->use_graph != b->cfg.use_graph &&
                  !b->tasks.empty();
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
    if (t > 0.0) {
      b->last_t[i] = t;
      b->last_team[i] = b->team[i];
      b->took[i][shape_key(b->cfg, b->team[i])] = t;
    }
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
  // per-core times from one solve with the current settings
  adp_status s = adp_batch_solve(b, nullptr, nullptr);
  if (s != ADP_OK) return s;
  adp_batch_config best = base;
  double best_t = 1e300;
  // kernel shapes: (threads, blocks per SM) = (256, 1), (256, 2), (512, 1);
  // each candidate is solved twice, the second time planned with the
  // times of its own team sizes from the first
  const int shapes[3][2] = {{256, 1}, {256, 2}, {512, 1}};
  const int teams[4] = {4, 8, 16, 32};
  for (const auto& sh : shapes) {
    if (batch_max_blocks_per_sm(b->mixed, b->ng, sh[0], sh[1]) < sh[1]) continue;
    for (int mt : teams) {
      adp_batch_config c = base;
      c.threads = sh[0];
      c.max_team = mt;
      c.blocks_per_sm = sh[1];
      double ms = 0.0;
      for (int rep = 0; rep < 2; ++rep) {
        s = adp_batch_set_config(b, &c);
        if (s != ADP_OK) return s;
        s = adp_batch_solve(b, nullptr, &ms);
        if (s != ADP_OK) return s;
      }
      if (ms < best_t) {
        best_t = ms;
        best = c;
      }
    }
  }
  s = adp_batch_set_config(b, &best);
  if (s != ADP_OK) return s;
  if (best_out) *best_out = best;
  if (best_ms) *best_ms = best_t;
  return ADP_OK;
}

adp_status adp_batch_plan_preview(int n, const double* rows, const double* t_ns, const int* t_team, int blocks,
                                  const adp_batch_config* c, int cap, int* team, int* begin, int* task_core,
                                  int* task_rank, double* makespan) {
  if (n < 1 || blocks < 1 || !c || !rows || !team || !begin || !task_core || !task_rank || cap < 0 ||
      (t_ns && !t_team) || c->max_team < 1 || !(c->grain > 0))
    return bfail(nullptr, ADP_ERR_INPUT, "adp_batch_plan_preview: bad arguments");
  for (int i = 0; i < n; ++i)
    if (!(rows[i] > 0) || (t_ns && (!(t_ns[i] > 0) || t_team[i] < 1)))
      return bfail(nullptr, ADP_ERR_INPUT, "adp_batch_plan_preview: weights and times must be positive");
  std::vector<double> w(rows, rows + n);
  std::function<double(int, int)> dur;
  if (t_ns)
    dur = [&](int i, int s) {
      return t_ns[i] * (1.0 / s + kDefaultKappa) / (1.0 / t_team[i] + kDefaultKappa);
    };
  const Plan P = plan_schedule(n, blocks, c->max_team, c->grain, w, dur);
  size_t total = 0;
  for (const auto& l : P.lists) total += l.size();
  if (total > (size_t)cap) return bfail(nullptr, ADP_ERR_INPUT, "adp_batch_plan_preview: task capacity too small");
  size_t k = 0;
  for (int b = 0; b < blocks; ++b) {
    begin[b] = (int)k;
    for (const BatchTask& t : P.lists[b]) {
      task_core[k] = t.inst;
      task_rank[k] = t.rank;
      ++k;
    }
  }
  begin[blocks] = (int)k;
  for (int i = 0; i < n; ++i) team[i] = P.team[i];
  if (makespan) *makespan = P.makespan;
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
