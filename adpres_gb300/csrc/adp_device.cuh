// Device-side building blocks of the GB300 solver: box geometry, the
// control block that carries the outer-iteration scalars between launches,
// a grid barrier with a time limit, and deterministic FP64 reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/adpres_gb300.h"
#include "ff.cuh"

namespace adp {

// Face order of df/dn/dc: X+, X-, Y+, Y-, Z+, Z- (mod_data.f90:59-60).
enum { FXP = 0, FXM = 1, FYP = 2, FYM = 3, FZP = 4, FZM = 5 };

// Neighbour-mask bits: bit f set when the face f of the node has a node
// across it (the reference's ystag/xstag/k tests, mod_cmfd.f90:255-298).
// Bit 6 marks an active node of the padded box.
enum { NB_ACTIVE = 64 };

constexpr int kMaxGroups = 8;     // nodal kernels are instantiated for 1..8 groups
constexpr int kMaxBlocks = 1024;  // persistent-grid size limit (reduction partial slots)
constexpr int kRedQ = 4;          // reduction quantities per phase

// Scalars of the outer iteration that live on the device between launches
// (the locals of outer()/outer_ad() in mod_cmfd.f90:431-440 plus Ke, ndmax).
struct OuterCtl {
  double Ke;          // current eigenvalue
  double f;           // integrated fission source of the latest fs0
  double e1;          // L2 norm of the previous fission-source change
  double ser, fer;    // errors of the latest outer
  double ndmax;       // last maximum change of dn (persists, mod_cmfd.f90:495)
  int p;              // outers done by the current adp_outer call
  int p_total;        // outers done over the life of the handle
  int cur;            // buffer holding the latest flux / fission source
  int status;         // first device-side error (adp_status), 0 if none
  int converged;
  int nodal_due;      // the latest outer needs a nodal update before its test
  int max_reached;
  int need_prologue;  // recompute f and e1 at the start of an outer() call
  int im, jm, km;     // location of ndmax (1-based)
  int nodal_updates;
  int err_node;       // box index attached to a device error, -1 if none
  int pad0;
  unsigned bar_count; // grid barrier state
  unsigned bar_gen;
  unsigned long long wait_ns;  // time limit of a barrier wait; 0: kBarrierTimeoutNs
  unsigned pad1[12];
};

// Box geometry shared by all kernels.  Box index b = i + nxx*(j + nyy*k),
// 0-based.  Vectors that are read at neighbours carry one halo plane on
// each side: pointer + b is valid for b in [-plane, NB + plane).
struct BoxGeom {
  int nxx, nyy, nzz;
  int NB, plane;
  int ng;
  const unsigned char* nbm;    // [NB]
  const double* xdel;          // [nxx]
  const double* ydel;          // [nyy]
  const double* zdel;          // [nzz]
  const double* vdel;          // [NB], 0 outside the core
  int bcf[6];                  // boundary condition of each face direction
};

__device__ __forceinline__ int face_off(const BoxGeom& G, int f) {
  switch (f) {
    case FXP: return 1;
    case FXM: return -1;
    case FYP: return G.nxx;
    case FYM: return -G.nxx;
    case FZP: return G.plane;
    default: return -G.plane;
  }
}

__device__ __forceinline__ double hdir(const BoxGeom& G, int u, int b) {
  // u = 0 x, 1 y, 2 z
  if (u == 0) return G.xdel[b % G.nxx];
  if (u == 1) return G.ydel[(b / G.nxx) % G.nyy];
  return G.zdel[b / G.plane];
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned atom_add_acqrel_gpu(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void set_status(OuterCtl* C, int code) {
  atomicCAS(&C->status, 0, code);
}

// Barrier of a team of co-resident blocks (the whole grid of a cooperative
// launch, or the blocks that share one core of a batch).  One 32-bit word
// per team: the block of rank 0 adds 2^31 - (nblocks - 1), every other
// block adds 1, so the top bit flips exactly when the last block arrives
// and the low bits return to zero; each block waits until the top bit
// differs from the value its own add returned.  The word must be 0 when the
// team first uses it.  The wait is bounded: after C->wait_ns (when 0,
// kBarrierTimeoutNs) the block records ADP_ERR_TIMEOUT and returns false, so
// a fault elsewhere can never leave the kernel spinning.  Called by lane 0
// of one warp.
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

// The arrival is an acquire-release add (it publishes this block's writes,
// which the block's other threads ordered before it with __syncthreads,
// and the last arrival acquires everyone else's) and the wait an acquire
// load; the add's read-modify-write chain carries every arriving block's
// release to the acquire that sees the flip, so no separate fence is
// needed.  A block that gave up never arrives again, so every later wait
// of the team runs out of time too and the kernel ends.
__device__ __forceinline__ int team_arrive_wait(OuterCtl* C, unsigned nblocks, unsigned rank) {
  int ok = 1;
  const unsigned long long lim0 = *(const volatile unsigned long long*)&C->wait_ns;
  const unsigned long long lim = lim0 ? lim0 : kBarrierTimeoutNs;
  const unsigned add = (rank == 0) ? (0x80000000u - (nblocks - 1u)) : 1u;
  const unsigned old = atom_add_acqrel_gpu(&C->bar_count, add);
  if (!(((old + add) ^ old) & 0x80000000u)) {
    unsigned long long t0 = 0;
    unsigned spins = 0;
    while (!((ld_acquire_gpu(&C->bar_count) ^ old) & 0x80000000u)) {
#if defined(ADP_BAR_SLEEP_NS) && ADP_BAR_SLEEP_NS > 0
      __nanosleep(ADP_BAR_SLEEP_NS);
#endif
      if ((++spins & 63u) == 0) {
        const unsigned long long t = globaltimer_ns();
        if (t0 == 0) t0 = t;
        else if (t - t0 > lim) {
          set_status(C, ADP_ERR_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
  }
  return ok;
}

__device__ __forceinline__ bool team_barrier(OuterCtl* C, unsigned nblocks, unsigned rank) {
  __shared__ int s_ok;
  __syncthreads();
  if (nblocks == 1) return true;
  if (threadIdx.x == 0) s_ok = team_arrive_wait(C, nblocks, rank);
  __syncthreads();
  return s_ok != 0;
}

// ---- range checks of device indices (bounds-checked build) ---------------
// Compiled in with -DADP_BOUNDS, a separate build of the library for tests:
// an index outside the box, or a neighbour index that is not an active
// node, records ADP_ERR_BOUNDS (first one wins, its index in err_node) and
// the item that computed it is skipped -- nothing traps.  In the product
// build the checks are constant true and compile to nothing.  The outer
// kernel's rows are in [0, NB) by their loop bounds and its stencil reads
// b +- plane stay inside the vectors' halo planes, so it needs none.
#ifdef ADP_BOUNDS
__device__ __forceinline__ bool adp_bounds_fail(OuterCtl* C, long long b) {
  if (C && atomicCAS(&C->status, 0, ADP_ERR_BOUNDS) == 0)
    C->err_node = (b >= -2147483647LL && b <= 2147483647LL) ? (int)b : -2;
  return false;
}
#define ADP_IN_BOX(C, b, NB) (((long long)(b) >= 0 && (long long)(b) < (long long)(NB)) ? true : adp::adp_bounds_fail((C), (b)))
#define ADP_NB_OK(C, G, bm) \
  ((ADP_IN_BOX(C, bm, (G).NB) && ((G).nbm[(bm)] & adp::NB_ACTIVE)) ? true : adp::adp_bounds_fail((C), (bm)))
#else
#define ADP_IN_BOX(C, b, NB) true
#define ADP_NB_OK(C, G, bm) true
#endif

// An item's node b and its neighbours across the faces its mask opens.
__device__ __forceinline__ bool node_ok(OuterCtl* C, const BoxGeom& G, long long b) {
#ifdef ADP_BOUNDS
  if (!ADP_IN_BOX(C, b, G.NB)) return false;
  const unsigned m = G.nbm[b];
  if (!(m & NB_ACTIVE)) return adp_bounds_fail(C, b);
  for (int f = 0; f < 6; ++f)
    if (m & (1u << f)) {
      const long long bm = b + face_off(G, f);
      if (!ADP_NB_OK(C, G, bm)) return false;
    }
  return true;
#else
  (void)C; (void)G; (void)b;
  return true;
#endif
}

// ---- deterministic reductions ------------------------------------------
// Sums use a fixed tree (xor-butterfly inside warps, warp results in order),
// so every block that reduces the same partials gets bit-identical totals.

template <bool MAX>
__device__ __forceinline__ double warp_all(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = MAX ? fmax(v, w) : v + w;
  }
  return v;
}

// Reduce NQ per-thread values over the block; thread 0 writes them to
// out[q * kMaxBlocks + blockIdx.x].  MAXMASK bit q selects max instead of sum.
template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ void block_partials(const double (&v)[NQ], double* out) {
  __shared__ double sw[NQ][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double x = ((MAXMASK >> q) & 1u) ? warp_all<true>(v[q]) : warp_all<false>(v[q]);
    if (lane == 0) sw[q][w] = x;
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const bool mx = (MAXMASK >> q) & 1u;
      double x = lane < nw ? sw[q][lane] : 0.0;   // sums and maxima of |.| start at 0
      x = mx ? warp_all<true>(x) : warp_all<false>(x);
      if (lane == 0) out[q * kMaxBlocks + blockIdx.x] = x;
    }
  }
  __syncthreads();
}

// Totals of NQ quantities from the partials of nblk blocks, identical in
// every block; every thread of the block receives them.  Warp q reduces
// quantity q; each lane issues its loads eight at a time before adding, so
// the partials cost one L2 round trip per 256 blocks instead of one per
// loop step.  The summation order is fixed by (lane, k), hence the same in
// every block.
template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ void grid_totals(const double* in, int nblk, double (&tot)[NQ]) {
  __shared__ double st[NQ];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (w < NQ) {
    const bool mx = (MAXMASK >> w) & 1u;
    const double* src = in + w * kMaxBlocks;
    double x = 0.0;
    for (int base = 0; base < nblk; base += 256) {
      double v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int i = base + lane + 32 * k;
        v[k] = (i < nblk) ? __ldcg(src + i) : 0.0;   // L2: partials were written by other SMs
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) x = mx ? fmax(x, v[k]) : x + v[k];
    }
    x = mx ? warp_all<true>(x) : warp_all<false>(x);
    if (lane == 0) st[w] = x;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) tot[q] = st[q];
  __syncthreads();
}

// xor-butterfly over a warp for NQ independent values at once (the steps of
// the different quantities are interleaved, so their latencies overlap).
template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ void warp_all_n(double (&x)[NQ]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double y[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) y[q] = __shfl_xor_sync(0xffffffffu, x[q], o);
#pragma unroll
    for (int q = 0; q < NQ; ++q) x[q] = ((MAXMASK >> q) & 1u) ? fmax(x[q], y[q]) : x[q] + y[q];
  }
}

// Block reduction, team barrier and totals in one step, with two block-wide
// synchronisations: every warp reduces its values; after the first
// __syncthreads warp 0 forms the block partials, lane 0 publishes them in
// slot[q * kMaxBlocks + rank] and waits at the team barrier, and warp 0
// then sums every block's partials (same order in every block) into shared
// memory for the whole block.  Returns false when the barrier wait ran out
// of time.
template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ bool grid_reduce(OuterCtl* C, unsigned nblocks, unsigned rank, double* slot,
                                            const double (&v)[NQ], double (&tot)[NQ]) {
  __shared__ double sw[NQ][32];
  __shared__ double st[NQ];
  __shared__ int s_ok;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  double x[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) x[q] = v[q];
  warp_all_n<NQ, MAXMASK>(x);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) sw[q][w] = x[q];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) x[q] = lane < nw ? sw[q][lane] : 0.0;   // sums and maxima of |.| start at 0
    warp_all_n<NQ, MAXMASK>(x);
    int ok = 1;
    if (nblocks == 1) {
      // a team of one block: its partials are the totals (the same values
      // the general path below would form from one partial)
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) st[q] = x[q];
      }
    } else {
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) slot[q * kMaxBlocks + rank] = x[q];
      }
      if (lane == 0) ok = team_arrive_wait(C, nblocks, rank);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
    }
    if (ok && nblocks > 1) {
      const int nblk = (int)nblocks;
#pragma unroll
      for (int q = 0; q < NQ; ++q) x[q] = 0.0;
      for (int base = 0; base < nblk; base += 256) {
        double y[NQ][8];
#pragma unroll
        for (int q = 0; q < NQ; ++q)
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int i = base + lane + 32 * k;
            y[q][k] = (i < nblk) ? __ldcg(slot + q * kMaxBlocks + i) : 0.0;   // L2: written by other SMs
          }
#pragma unroll
        for (int k = 0; k < 8; ++k)
#pragma unroll
          for (int q = 0; q < NQ; ++q) x[q] = ((MAXMASK >> q) & 1u) ? fmax(x[q], y[q][k]) : x[q] + y[q][k];
      }
      warp_all_n<NQ, MAXMASK>(x);
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) st[q] = x[q];
      }
    }
    if (lane == 0) s_ok = ok;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) tot[q] = st[q];
  return s_ok != 0;
}

// The same fused block reduction, team barrier and totals in double-float
// arithmetic (FP32 pairs, error-free sums) for the mixed path: the values,
// the warp and block sums and the partials in memory are double-floats, so
// no FP64 instruction runs except the final conversion of each total.
// The partial slots of `slot` hold one (hi, lo) pair per block.  MAXMASK
// quantities are maxima of non-negative values carried in hi.
template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ void warp_all_ff(ff (&x)[NQ]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const ff y{__shfl_xor_sync(0xffffffffu, x[q].hi, o), __shfl_xor_sync(0xffffffffu, x[q].lo, o)};
      x[q] = ((MAXMASK >> q) & 1u) ? (y.hi > x[q].hi ? y : x[q]) : ff_add(x[q], y);
    }
  }
}

// The butterfly of warp_all_ff over the lanes below 2 * o0 (o0 a power of
// two, the lanes above it ignored), leaving the totals in lane 0 only, with
// the quantities scattered over the lanes: at each of the first log2(NQ)
// levels a lane keeps half of its quantities and hands the partner the
// other half, so the next levels carry one quantity per lane, and lane 0
// collects the NQ totals at the end.  Every total is formed from the same
// pairs in the same order as in warp_all_ff (the sum of a lane and its
// partner at each level; the sums are commutative), so the totals are the
// same to the bit; a level of warp_all_ff that only adds lanes holding
// exact zeros is left out.  With fewer levels than quantities it runs
// warp_all_ff.
template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ void warp_reduce_lane0_ff(ff (&x)[NQ], int o0) {
  static_assert(NQ == 1 || NQ == 2 || NQ == 4, "1, 2 or 4 quantities");
  constexpr int L = NQ == 4 ? 2 : (NQ == 2 ? 1 : 0);
  if ((o0 >> (L > 0 ? L - 1 : 0)) < 1 && L > 0) {
    warp_all_ff<NQ, MAXMASK>(x);
    return;
  }
  const int lane = threadIdx.x & 31;
  int o = o0, q0 = 0;
  ff v[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = x[q];
#pragma unroll
  for (int m = NQ; m > 1; m >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < m / 2; ++j) {
      const ff give = up ? v[j] : v[j + m / 2];
      const ff keep = up ? v[j + m / 2] : v[j];
      const ff y{__shfl_xor_sync(0xffffffffu, give.hi, o), __shfl_xor_sync(0xffffffffu, give.lo, o)};
      const int q = q0 + (up ? m / 2 : 0) + j;
      v[j] = ((MAXMASK >> q) & 1u) ? (y.hi > keep.hi ? y : keep) : ff_add(keep, y);
    }
    if (up) q0 += m / 2;
    o >>= 1;
  }
  for (; o > 0; o >>= 1) {
    const ff y{__shfl_xor_sync(0xffffffffu, v[0].hi, o), __shfl_xor_sync(0xffffffffu, v[0].lo, o)};
    v[0] = ((MAXMASK >> q0) & 1u) ? (y.hi > v[0].hi ? y : v[0]) : ff_add(v[0], y);
  }
  // quantity q sits in the lanes whose scatter bits spell q: the lowest is
  // the sum of the scatter offsets of q's bits
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    int src = 0;
#pragma unroll
    for (int i = 0; i < L; ++i) src += ((q >> (L - 1 - i)) & 1) * (o0 >> i);
    x[q] = ff{__shfl_sync(0xffffffffu, v[0].hi, src), __shfl_sync(0xffffffffu, v[0].lo, src)};
  }
}

template <int NQ, unsigned MAXMASK>
__device__ __forceinline__ bool grid_reduce_ff(OuterCtl* C, unsigned nblocks, unsigned rank, double* slot_d,
                                               const ff (&v)[NQ], double (&tot)[NQ]) {
  __shared__ ff sw[NQ][32];
  __shared__ double st[NQ];
  __shared__ int s_ok;
  float2* slot = reinterpret_cast<float2*>(slot_d);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  ff x[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) x[q] = v[q];
  warp_reduce_lane0_ff<NQ, MAXMASK>(x, 16);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) sw[q][w] = x[q];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) x[q] = lane < nw ? sw[q][lane] : ff{0.f, 0.f};
    // the levels that reach the nw lanes holding a warp's sum
    int o0 = 16;
    while (o0 > 1 && o0 >= nw) o0 >>= 1;
    if (nw > 1) warp_reduce_lane0_ff<NQ, MAXMASK>(x, o0);
    int ok = 1;
    if (nblocks > 1) {
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) slot[q * kMaxBlocks + rank] = make_float2(x[q].hi, x[q].lo);
        ok = team_arrive_wait(C, nblocks, rank);
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
      if (ok) {
        const int nblk = (int)nblocks;
#pragma unroll
        for (int q = 0; q < NQ; ++q) x[q] = ff{0.f, 0.f};
        for (int base = 0; base < nblk; base += 256) {
          // partials past the last block would add exact zeros: left out
          const int kmax = min(8, (nblk - base + 31) >> 5);
          float2 y[NQ][8];
#pragma unroll
          for (int q = 0; q < NQ; ++q)
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int i = base + lane + 32 * k;
              y[q][k] = (k < kmax && i < nblk) ? __ldcg(slot + q * kMaxBlocks + i) : make_float2(0.f, 0.f);
            }
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (k < kmax) {
#pragma unroll
              for (int q = 0; q < NQ; ++q) {
                const ff yy{y[q][k].x, y[q][k].y};
                x[q] = ((MAXMASK >> q) & 1u) ? (yy.hi > x[q].hi ? yy : x[q]) : ff_add(x[q], yy);
              }
            }
        }
        warp_reduce_lane0_ff<NQ, MAXMASK>(x, 16);
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) st[q] = ff_to_double(x[q]);
      s_ok = ok;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) tot[q] = st[q];
  return s_ok != 0;
}

}  // namespace adp
