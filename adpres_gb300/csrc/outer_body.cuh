// The outer-iteration loop of outer / outer_ad (mod_cmfd.f90:415-699) as a
// device function run by a team of co-resident blocks: the whole grid of
// the single-core cooperative kernel k_outer, or the blocks that share one
// core of a batch.  Block `rank` of `nteam` owns the box rows
// rank * blockDim.x + threadIdx.x + k * nteam * blockDim.x.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "adp_kernels.h"
#include "ff.cuh"

namespace adp {

__device__ __forceinline__ double fmav(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmav(float a, float b, float c) { return fmaf(a, b, c); }

// Load that bypasses L1: control words written by other blocks of the team.
template <class T>
__device__ __forceinline__ T vld(const T* p) {
  return *(const volatile T*)p;
}

// The rows b, b + nthr, b + 2 nthr, ... of one thread, R at a time: `ld`
// computes a row's results from loads only, `ex` stores them and adds to
// the thread's partial sums, in the original row order.  Issuing the loads
// of R rows before any store lets them overlap (a store may alias a later
// row's loads for all the compiler knows), without changing any value or
// the order of any sum.
template <int R, class Ld, class Ex>
__device__ __forceinline__ void rows_batched(int b, int nthr, int NB, Ld&& ld, Ex&& ex) {
  using Row = decltype(ld(0));
  for (; b + (R - 1) * nthr < NB; b += R * nthr) {
    Row v[R];
#pragma unroll
    for (int u = 0; u < R; ++u) v[u] = ld(b + u * nthr);
#pragma unroll
    for (int u = 0; u < R; ++u) ex(b + u * nthr, v[u]);
  }
  for (; b < NB; b += nthr) ex(b, ld(b));
}

// Team reduction of per-thread partials: in double-float for the mixed
// path (no FP64 instruction per warp), in FP64 for the FP64 path.
template <bool MIXED, int NQ, unsigned MASK>
__device__ __forceinline__ bool team_reduce(OuterCtl* C, unsigned nblk, unsigned rank, double* slot,
                                            const double (&vd)[NQ], const ff (&vf)[NQ], double (&tot)[NQ]) {
  if constexpr (MIXED) return grid_reduce_ff<NQ, MASK>(C, nblk, rank, slot, vf, tot);
  else return grid_reduce<NQ, MASK>(C, nblk, rank, slot, vd, tot);
}

// Rows in flight per thread in the row loops (compile-time tunable).
#ifndef ADP_ROWS_FP64
#define ADP_ROWS_FP64 2
#endif
#ifndef ADP_ROWS_MIXED
#define ADP_ROWS_MIXED 2
#endif
template <bool MIXED>
struct RowsInFlight { static constexpr int R = ADP_ROWS_FP64; };
template <>
struct RowsInFlight<true> { static constexpr int R = ADP_ROWS_MIXED; };

// ---------------------------------------------------------------------------
// The persistent outer-iteration loop.
//
// One team runs outer iterations until one needs a nodal
// update (p mod nupd == 0), converges, reaches nout, or fails.  Every block
// owns the box rows tid, tid + nthreads, ... in every phase, so values a
// thread wrote in one phase are read back by the same thread without a
// barrier; neighbour reads and global dot products are separated by
// a team barrier.  Per group solve (bicg, mod_cmfd.f90:1203-1243):
//   P0: b = TSrc, r = b - A x, rs = r, partial (rs,r)              | barrier
//   per step i = 1..nin:
//   A : (i > 1: the previous step's x += alpha p + omega s and
//       r = s - omega t, r recomputed at neighbours), beta,
//       p = r + beta (p - omega v) (neighbours recomputed), v = A p,
//       partial (rs,v)                                               | barrier
//   B : alpha, s = r - alpha v (neighbours recomputed), t = A s,
//       partials (t,t), (t,s) and, before another step, (rs,s), (rs,t),
//       whence (rs, r_next) = (rs,s) - omega (rs,t)                  | barrier
//   C (last step only, no barrier): x += alpha p + omega s, RelEg.
// Two grid barriers per BiCGSTAB step instead of three: the (rs,r)
// reduction of bicg (mod_cmfd.f90:1230) is formed algebraically from
// phase-B partials, so the r/x update joins the next step's phase A.
// After the last group: FSrc, |fs - fs0c|^2, Integrate, RelE, RelEg
// (barrier), extrapolation every nac outers (barrier), k update and the
// convergence test, all in the same order as mod_cmfd.f90:479-495.
//
// MIXED: P0 forms the defect of the current flux in double-float (a
// compensated dot product over the FP64 matrix as (A32, A - A32) and the
// flux and sources as (hi, lo) pairs, each pair one float2); the nin Krylov steps for the correction run
// with the FP32 matrix copy and FP32 vectors; the reductions are
// double-float and the flux x, held as hi + lo, receives the FP32
// increments.  Both forms avoid FP64 division in per-row work (the source
// uses 1/k computed once per outer; RelE/RelEg divide only when a candidate
// beats the running maximum).
//
// P0 leaves out the source terms of planes that are zero at every node
// (P.src_nz, P.sc_nz: the up-scatter planes of a down-scatter-only core,
// the chi = 0 groups): for finite fluxes a zero term adds an exact zero to
// sums that are never -0, so the results are the same to the bit and only
// the loads go.
//
// The Krylov vectors read at neighbours are stored in pairs: (p, v), double
// buffered, and (s, t), so a neighbour's recomputed p or r costs two loads
// instead of four.
// ---------------------------------------------------------------------------
template <bool MIXED>
struct KV { using T = double; using T2 = double2; };
template <>
struct KV<true> { using T = float; using T2 = float2; };
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }

// SMEMA: the block keeps its own rows' matrix coefficients of the group
// being solved in dynamic shared memory (P.smem_rows rows per coefficient,
// row k * nthreads + tid of the block at index k * blockDim.x + tid): P0
// reads them from memory anyway and stores them, the 2 nin Krylov phases
// that follow read them from there instead of L2 or HBM.
// XSRC (mixed path only): the group source also carries the external source
// P.exsrc2 as (hi, lo) pairs -- the transient step (outer_tr) and the
// fixed-eigenvalue mode of the generalized adjoint of adp_adjoint_sens.
// The forward and adjoint eigenvalue solves are the XSRC = false
// instantiation.
template <bool MIXED, bool SMEMA = false, bool XSRC = false>
__device__ __forceinline__ void outer_body(const OuterParams& P, unsigned rank, unsigned nteam) {
  using T = typename KV<MIXED>::T;
  using T2 = typename KV<MIXED>::T2;
  extern __shared__ __align__(16) unsigned char adp_dyn_smem[];
  T* const sA = reinterpret_cast<T*>(adp_dyn_smem);
  const int SR = P.smem_rows;
  OuterCtl* C = P.ctl;
  const BoxGeom& G = P.G;
  const int NB = G.NB, nxx = G.nxx, plane = G.plane, ng = P.ng;
  const int nthr = nteam * blockDim.x;
  const int tid0 = rank * blockDim.x + threadIdx.x;
  const unsigned nblk = nteam;
  const long long NBH = P.NBH;
  // shared-memory index of one of this thread's rows
  auto jrow = [&](int b) -> int { return ((b - tid0) / nthr) * (int)blockDim.x + (int)threadIdx.x; };

  __shared__ int s_stop;
  if (threadIdx.x == 0)
    s_stop = (vld(&C->status) || vld(&C->converged) || vld(&C->max_reached) || vld(&C->nodal_due)) ? 1 : 0;
  __syncthreads();
  if (s_stop) return;

  // Scalars shared by the whole block (alpha, beta, omega, k, ...) are formed
  // by one thread and broadcast: on GB300 an FP64 instruction of a warp
  // occupies the FP64 pipe for tens of cycles, so forming them in every
  // warp would cost several microseconds per BiCGSTAB step.
  // Slots: step start s_d[0..1], s_f[0..2], s_ib; after phase A s_d[0],
  // s_f[0], s_ia; after phase B s_d[2..3], s_f[3], s_io (its readers may
  // still be reading when the next step's start writes, hence its own
  // slots); end of outer s_d[0..2], s_f[0..1].  Every other reuse of a slot
  // is separated from its last read by a block-wide barrier.
  __shared__ double s_d[4];
  __shared__ float s_f[4];
  __shared__ int s_ib, s_ia, s_io;
  double Ke = vld(&C->Ke), f = vld(&C->f), e1 = vld(&C->e1);
  const double ndmax = vld(&C->ndmax);
  int p = vld(&C->p), ptot = vld(&C->p_total), cur = vld(&C->cur);
  int epoch = 0;
  const bool lead = (rank == 0 && threadIdx.x == 0);
#define RED(e) (P.red + ((e) & 1) * kRedQ * kMaxBlocks)

  const T* Ab = MIXED ? (const T*)P.A32 : (const T*)P.A;
  T* r = MIXED ? (T*)P.r32 : (T*)P.r;
  T* rs = MIXED ? (T*)P.rs32 : (T*)P.rs;
  T2* st = MIXED ? (T2*)P.st2f : (T2*)P.st2;   // (s, t)
  T2* pv[2] = {MIXED ? (T2*)P.pv2f[0] : (T2*)P.pv2[0], MIXED ? (T2*)P.pv2f[1] : (T2*)P.pv2[1]};   // (p, v)

  if (vld(&C->need_prologue)) {
    // f = Integrate(fs0); errn = 1; e1 = Integrate(errn)  (mod_cmfd.f90:457-459)
    double acc[2] = {0.0, 0.0};
    const double* fsc = P.fs[cur];
    for (int b = tid0; b < NB; b += nthr) {
      acc[0] = fma(G.vdel[b], fsc[b], acc[0]);
      acc[1] += G.vdel[b];
    }
    double tot[2];
    if (!grid_reduce<2, 0u>(C, nblk, rank, RED(epoch), acc, tot)) return;
    ++epoch;
    f = tot[0];
    e1 = tot[1];
  }

  if constexpr (MIXED) {
    // The FP64 flux and fission source are authoritative between launches;
    // split the current ones into double-floats (own rows), then wait for
    // the neighbours' rows before the first stencil.
    const double* ph = P.phi[cur];
    for (int b = tid0; b < NB; b += nthr) {
      for (int g = 0; g < ng; ++g) st_ff(&P.x2[cur][(size_t)g * NBH + b], ff_from_double(ph[(size_t)g * NBH + b]));
      st_ff(&P.fs2[cur][b], ff_from_double(P.fs[cur][b]));
    }
    if (!team_barrier(C, nblk, rank)) return;
  }

  while (true) {
    ++p;
    ++ptot;
    const int old = cur, nw = cur ^ 1;
    const double* phiO = P.phi[old];
    double* phiN = P.phi[nw];
    const double* fsO = P.fs[old];
    double* fsN = P.fs[nw];
    if (threadIdx.x == 0) {
      const double ik = P.trans ? 1.0 : 1.0 / Ke;   // the transient source has no 1/k
      const ff ikf = ff_from_double(ik);
      s_d[0] = ik;
      s_f[0] = ikf.hi;
      s_f[1] = ikf.lo;
    }
    __syncthreads();
    const double invKe = s_d[0];
    const ff invKe_ff{s_f[0], s_f[1]};
    double fer_acc = 0.0;
    float fer_f = 0.f;

    for (int gi = 0; gi < ng; ++gi) {
      const int g = P.adj ? ng - 1 - gi : gi;
      const T* Ag = Ab + (size_t)g * 7 * NB;
      const double* A64 = P.A + (size_t)g * 7 * NB;
      const double* xO = phiO + (size_t)g * NBH;
      double* xN = phiN + (size_t)g * NBH;
      const double* wsrc = P.wsrc + (size_t)g * NB;

      // ---- P0: source and initial residual (TSrc + r = b - A x) --------
      double tot1[1];
      if constexpr (MIXED) {
        // (XSRC adds the external source: the transient step's, or the
        // generalized adjoint's)
        // Defect of the current flux in double-float: one compensated dot
        // product over the source and the seven matrix terms (A = A32 + lo).
        const float2* xO2 = P.x2[old] + (size_t)g * NBH;
        const float2* A2g = P.A2 + (size_t)g * 7 * NB;
        T accT = T(0);
        rows_batched<RowsInFlight<MIXED>::R>(
            tid0, nthr, NB,
            [&](int b) -> T {
              Dot2 d;
              if ((P.src_nz >> g) & 1u)
                d.add(ff_mul(ld_ff(&P.wsrc2[(size_t)g * NB + b]), ld_ff(&P.fs2[old][b])), invKe_ff);
              if constexpr (XSRC) d.add(ld_ff(&P.exsrc2[(size_t)g * NB + b]), ff{1.f, 0.f});
              for (int h = 0; h < ng; ++h) {
                if (h == g) continue;
                const int q = P.adj ? g * ng + h : h * ng + g;
                if (!((P.sc_nz >> q) & 1ull)) continue;   // an all-zero scattering plane
                const bool solved = P.adj ? (h > g) : (h < g);
                const int buf = solved ? nw : old;
                const size_t ix = (size_t)h * NBH + b;
                const size_t is = (size_t)q * NB + b;
                d.add(ld_ff(&P.sigs2[is]), ld_ff(&P.x2[buf][ix]));
              }
              const int off[7] = {-plane, -nxx, -1, 0, 1, nxx, plane};
              const int j = SMEMA ? jrow(b) : 0;
#pragma unroll
              for (int c = 0; c < 7; ++c) {
                const ff a = ld_ff(&A2g[(size_t)c * NB + b]);   // a.hi is the A32 coefficient
                if constexpr (SMEMA) sA[(size_t)c * SR + j] = a.hi;
                d.sub(a, ld_ff(&xO2[b + off[c]]));
              }
              return d.value().hi;
            },
            [&](int b, T rt) {
              r[b] = rt;
              rs[b] = rt;
              accT = fmav(rt, rt, accT);
            });
        ff acc[1] = {ff{(float)accT, 0.f}};
        if (!grid_reduce_ff<1, 0u>(C, nblk, rank, RED(epoch), acc, tot1)) return;
      } else {
        T accT = T(0);
        rows_batched<RowsInFlight<MIXED>::R>(
            tid0, nthr, NB,
            [&](int b) -> T {
              double s0 = 0.0;
              for (int h = 0; h < ng; ++h) {
                if (h == g) continue;
                const int q = P.adj ? g * ng + h : h * ng + g;
                if (!((P.sc_nz >> q) & 1ull)) continue;   // an all-zero scattering plane
                const bool solved = P.adj ? (h > g) : (h < g);
                const double ph = (solved ? phiN : phiO)[(size_t)h * NBH + b];
                s0 = fma(P.sigs[(size_t)q * NB + b], ph, s0);
              }
              double bs = ((P.src_nz >> g) & 1u) ? wsrc[b] * fsO[b] * invKe + s0 : s0;
              if (P.trans) bs = bs + P.exsrc[(size_t)g * NB + b];   // TSrcTr (mod_cmfd.f90:1091-1093)
              double a64[7];
#pragma unroll
              for (int c = 0; c < 7; ++c) a64[c] = A64[(size_t)c * NB + b];
              if constexpr (SMEMA) {
                const int j = jrow(b);
#pragma unroll
                for (int c = 0; c < 7; ++c) sA[(size_t)c * SR + j] = (T)a64[c];
              }
              double ax = a64[0] * xO[b - plane];
              ax = fma(a64[1], xO[b - nxx], ax);
              ax = fma(a64[2], xO[b - 1], ax);
              ax = fma(a64[3], xO[b], ax);
              ax = fma(a64[4], xO[b + 1], ax);
              ax = fma(a64[5], xO[b + nxx], ax);
              ax = fma(a64[6], xO[b + plane], ax);
              const double rr = bs - ax;
              return (T)rr;
            },
            [&](int b, T rt) {
              r[b] = rt;
              rs[b] = rt;
              accT = fmav(rt, rt, accT);
            });
        double acc[1] = {(double)accT};
        if (!grid_reduce<1, 0u>(C, nblk, rank, RED(epoch), acc, tot1)) return;
      }
      ++epoch;
      double rsr = tot1[0];
      double rho = 1.0, alpha = 1.0, omega = 1.0;

      for (int it = 0; it < P.nin; ++it) {
        const bool last = (it == P.nin - 1);
        if (threadIdx.x == 0) {
          const double rho_prev = rho, rho_n = rsr;
          const int brk = (rho_n == 0.0 || omega == 0.0);
          const double bt = brk ? 0.0 : (rho_n / rho_prev) * (alpha / omega);
          s_d[0] = rho_n;
          s_d[1] = bt;
          s_f[0] = (float)bt;
          s_f[1] = (float)omega;
          s_f[2] = (float)alpha;
          s_ib = brk;
        }
        __syncthreads();
        rho = s_d[0];
        const double beta = s_d[1];
        if (s_ib) {
          if (lead) set_status(C, ADP_ERR_BREAKDOWN);
          return;
        }
        T2* pvN = pv[it & 1];
        const T2* pvO = pv[(it & 1) ^ 1];
        const T tb = MIXED ? (T)s_f[0] : (T)beta, tom = MIXED ? (T)s_f[1] : (T)omega,
                tap = MIXED ? (T)s_f[2] : (T)alpha;
        // ---- phase A: (previous step's x and r), p and v = A p -----------
        {
          T accT = T(0);
          if (it == 0) {
            struct RowA0 { T pb, v, rsb; };
            rows_batched<RowsInFlight<MIXED>::R>(
                tid0, nthr, NB,
                [&](int b) -> RowA0 {
                  const T pb = r[b];
                  const int j = SMEMA ? jrow(b) : 0;
                  auto AC = [&](int c) -> T { return SMEMA ? sA[(size_t)c * SR + j] : Ag[(size_t)c * NB + b]; };
                  T v = AC(0) * r[b - plane];
                  v = fmav(AC(1), r[b - nxx], v);
                  v = fmav(AC(2), r[b - 1], v);
                  v = fmav(AC(3), pb, v);
                  v = fmav(AC(4), r[b + 1], v);
                  v = fmav(AC(5), r[b + nxx], v);
                  v = fmav(AC(6), r[b + plane], v);
                  return RowA0{pb, v, rs[b]};
                },
                [&](int b, const RowA0& q) {
                  pvN[b] = mk2(q.pb, q.v);
                  accT = fmav(q.rsb, q.v, accT);
                });
          } else {
            const double* xc = (it == 1) ? xO : xN;
            const float2* xc2 = MIXED ? ((it == 1) ? P.x2[old] : P.x2[nw]) + (size_t)g * NBH : nullptr;
            float2* xN2 = MIXED ? P.x2[nw] + (size_t)g * NBH : nullptr;
            struct RowA { T rb, pb, v, rsb; double xn; ff xf; };
            rows_batched<RowsInFlight<MIXED>::R>(
                tid0, nthr, NB,
                [&](int b) -> RowA {
                  auto rf = [&](int m) -> T {
                    const T2 q = st[m];
                    return fmav(-tom, q.y, q.x);
                  };
                  auto pf = [&](int m) -> T {
                    const T2 o = pvO[m];
                    return fmav(tb, fmav(-tom, o.y, o.x), rf(m));
                  };
                  const T2 stb = st[b], pvb = pvO[b];
                  const T rb = fmav(-tom, stb.y, stb.x);
                  double xn = 0.0;
                  ff xf{0.f, 0.f};
                  if constexpr (MIXED) {
                    // FP32 increment of the correction, added to the double-float flux
                    const T dx = fmav(tom, stb.x, tap * pvb.x);
                    xf = ff_add_f(ld_ff(&xc2[b]), dx);
                  } else {
                    xn = fma(omega, (double)stb.x, fma(alpha, (double)pvb.x, xc[b]));
                  }
                  const T pb = fmav(tb, fmav(-tom, pvb.y, pvb.x), rb);
                  const int j = SMEMA ? jrow(b) : 0;
                  auto AC = [&](int c) -> T { return SMEMA ? sA[(size_t)c * SR + j] : Ag[(size_t)c * NB + b]; };
                  T v = AC(0) * pf(b - plane);
                  v = fmav(AC(1), pf(b - nxx), v);
                  v = fmav(AC(2), pf(b - 1), v);
                  v = fmav(AC(3), pb, v);
                  v = fmav(AC(4), pf(b + 1), v);
                  v = fmav(AC(5), pf(b + nxx), v);
                  v = fmav(AC(6), pf(b + plane), v);
                  return RowA{rb, pb, v, rs[b], xn, xf};
                },
                [&](int b, const RowA& q) {
                  r[b] = q.rb;
                  if constexpr (MIXED) {
                    st_ff(&xN2[b], q.xf);
                  } else {
                    xN[b] = q.xn;
                  }
                  pvN[b] = mk2(q.pb, q.v);
                  accT = fmav(q.rsb, q.v, accT);
                });
          }
          const double accd[1] = {(double)accT};
          const ff accf[1] = {ff{(float)accT, 0.f}};
          if (!team_reduce<MIXED, 1, 0u>(C, nblk, rank, RED(epoch), accd, accf, tot1)) return;
        }
        ++epoch;
        if (threadIdx.x == 0) {
          const int brk = tot1[0] == 0.0;
          const double al = brk ? 0.0 : rho / tot1[0];
          s_d[0] = al;
          s_f[0] = (float)al;
          s_ia = brk;
        }
        __syncthreads();
        if (s_ia) {
          if (lead) set_status(C, ADP_ERR_BREAKDOWN);
          return;
        }
        alpha = s_d[0];
        const T ta = MIXED ? (T)s_f[0] : (T)alpha;
        // ---- phase B: s and t = A s; (t,t), (t,s) and, for the next step,
        //      (rs,s), (rs,t): (rs, s - omega t) = (rs,s) - omega (rs,t) ------
        double tot4[4];
        {
          T acc0 = T(0), acc1 = T(0), acc2 = T(0), acc3 = T(0);
          struct RowB { T sb, tt, rsb; };
          rows_batched<RowsInFlight<MIXED>::R>(
              tid0, nthr, NB,
              [&](int b) -> RowB {
                auto sf = [&](int m) -> T { return fmav(-ta, pvN[m].y, r[m]); };
                const T sb = sf(b);
                const int j = SMEMA ? jrow(b) : 0;
                auto AC = [&](int c) -> T { return SMEMA ? sA[(size_t)c * SR + j] : Ag[(size_t)c * NB + b]; };
                T tt = AC(0) * sf(b - plane);
                tt = fmav(AC(1), sf(b - nxx), tt);
                tt = fmav(AC(2), sf(b - 1), tt);
                tt = fmav(AC(3), sb, tt);
                tt = fmav(AC(4), sf(b + 1), tt);
                tt = fmav(AC(5), sf(b + nxx), tt);
                tt = fmav(AC(6), sf(b + plane), tt);
                return RowB{sb, tt, last ? T(0) : rs[b]};
              },
              [&](int b, const RowB& q) {
                st[b] = mk2(q.sb, q.tt);
                acc0 = fmav(q.tt, q.tt, acc0);
                acc1 = fmav(q.tt, q.sb, acc1);
                if (!last) {
                  acc2 = fmav(q.rsb, q.sb, acc2);
                  acc3 = fmav(q.rsb, q.tt, acc3);
                }
              });
          if (last) {
            const double accd[2] = {(double)acc0, (double)acc1};
            const ff accf[2] = {ff{(float)acc0, 0.f}, ff{(float)acc1, 0.f}};
            double tot2[2];
            if (!team_reduce<MIXED, 2, 0u>(C, nblk, rank, RED(epoch), accd, accf, tot2)) return;
            tot4[0] = tot2[0];
            tot4[1] = tot2[1];
          } else {
            const double accd[4] = {(double)acc0, (double)acc1, (double)acc2, (double)acc3};
            const ff accf[4] = {ff{(float)acc0, 0.f}, ff{(float)acc1, 0.f}, ff{(float)acc2, 0.f},
                                ff{(float)acc3, 0.f}};
            if (!team_reduce<MIXED, 4, 0u>(C, nblk, rank, RED(epoch), accd, accf, tot4)) return;
          }
        }
        ++epoch;
        if (threadIdx.x == 0) {
          const int brk = tot4[0] == 0.0;
          const double om = brk ? 0.0 : tot4[1] / tot4[0];
          s_d[2] = om;
          s_d[3] = last ? 0.0 : tot4[2] - om * tot4[3];
          s_f[3] = (float)om;
          s_io = brk;
        }
        __syncthreads();
        if (s_io) {
          if (lead) set_status(C, ADP_ERR_BREAKDOWN);
          return;
        }
        omega = s_d[2];
        if (!last) {
          rsr = s_d[3];
        } else {
          // ---- phase C of the last step: x, and RelEg's running maximum.
          // No barrier follows: the next group's P0 (or the fission source)
          // reads only this thread's own rows of x.
          const T to = MIXED ? (T)s_f[3] : (T)omega;
          const double* xc = (it == 0) ? xO : xN;
          if constexpr (MIXED) {
            const float2* xc2 = ((it == 0) ? P.x2[old] : P.x2[nw]) + (size_t)g * NBH;
            const float2* xO2 = P.x2[old] + (size_t)g * NBH;
            float2* xN2 = P.x2[nw] + (size_t)g * NBH;
            struct RowCm { ff xn; float d; };
            rows_batched<RowsInFlight<MIXED>::R>(
                tid0, nthr, NB,
                [&](int b) -> RowCm {
                  // FP32 increment of the correction, added to the double-float flux
                  const T dx = fmav(to, st[b].x, ta * pvN[b].x);
                  const ff xn = ff_add_f(ld_ff(&xc2[b]), dx);
                  return RowCm{xn, ff_diff(xn, ld_ff(&xO2[b]))};
                },
                [&](int b, const RowCm& q) {
                  st_ff(&xN2[b], q.xn);
                  // RelEg (mod_cmfd.f90:1172-1199): max |x - x0| / |x| over |x| > 1e-10
                  const float ax = fabsf(q.xn.hi), d = fabsf(q.d);
                  if (ax > 1.e-10f && d > fer_f * ax) fer_f = fmaxf(fer_f, d / ax);
                });
          } else {
          struct RowC { double xn, xo; };
          rows_batched<RowsInFlight<MIXED>::R>(
              tid0, nthr, NB,
              [&](int b) -> RowC {
                const double xn = fma(omega, (double)st[b].x, fma(alpha, (double)pvN[b].x, xc[b]));
                return RowC{xn, xO[b]};
              },
              [&](int b, const RowC& q) {
                xN[b] = q.xn;
                // RelEg (mod_cmfd.f90:1172-1199): max |x - x0| / |x| over |x| > 1e-10
                const double ax = fabs(q.xn), d = fabs(q.xn - q.xo);
                if (ax > 1.e-10 && d > fer_acc * ax) fer_acc = fmax(fer_acc, d / ax);
              });
          }
        }
      }
    }

    // ---- fission source, norms and eigenvalue ------------------------------
    const bool extrap = (p % P.nac) == 0;
    double tot4[4];
    if constexpr (MIXED) {
      // fission source in double-float (Dot2 over the groups), Integrate
      // as a compensated per-thread sum, norms of the change in FP32
      float e2f = 0.f, serf = 0.f;
      Dot2 dint;
      struct RowFm { ff fs, fo, vd; };
      rows_batched<RowsInFlight<MIXED>::R>(
          tid0, nthr, NB,
          [&](int b) -> RowFm {
            Dot2 d;
            for (int g = 0; g < ng; ++g)
              d.add(ld_ff(&P.x2[nw][(size_t)g * NBH + b]), ld_ff(&P.wfis2[(size_t)g * NB + b]));
            return RowFm{d.value(), ld_ff(&P.fs2[old][b]), ld_ff(&P.vdel2[b])};
          },
          [&](int b, const RowFm& q) {
            st_ff(&P.fs2[nw][b], q.fs);
            const float en = ff_diff(q.fs, q.fo);
            e2f = fmaf(en, en, e2f);
            if (!extrap) {
              dint.add(q.vd, q.fs);
              // RelE (mod_cmfd.f90:1143-1168)
              const float af = fabsf(q.fs.hi), d = fabsf(en);
              if (af > 1.e-10f && d > serf * af) serf = fmaxf(serf, d / af);
            }
          });
      const ff acc[4] = {ff{e2f, 0.f}, dint.value(), ff{serf, 0.f}, ff{fer_f, 0.f}};
      if (!grid_reduce_ff<4, 0xCu>(C, nblk, rank, RED(epoch), acc, tot4)) return;
      ++epoch;
    } else {
      double acc[4] = {0.0, 0.0, 0.0, fer_acc};
      struct RowF { double fs, fo, vd; };
      rows_batched<RowsInFlight<MIXED>::R>(
          tid0, nthr, NB,
          [&](int b) -> RowF {
            double fs = 0.0;
            for (int g = 0; g < ng; ++g) fs = fma(phiN[(size_t)g * NBH + b], P.wfis[(size_t)g * NB + b], fs);
            return RowF{fs, fsO[b], G.vdel[b]};
          },
          [&](int b, const RowF& q) {
            fsN[b] = q.fs;
            const double en = q.fs - q.fo;
            acc[0] = fma(en, en, acc[0]);
            if (!extrap) {
              acc[1] = fma(q.vd, q.fs, acc[1]);
              // RelE (mod_cmfd.f90:1143-1168)
              const double af = fabs(q.fs), d = fabs(en);
              if (af > 1.e-10 && d > acc[2] * af) acc[2] = fmax(acc[2], d / af);
            }
          });
      if (!grid_reduce<4, 0xCu>(C, nblk, rank, RED(epoch), acc, tot4)) return;
      ++epoch;
    }
    if (threadIdx.x == 0) {
      const double e2n = sqrt(tot4[0]);
      s_d[0] = e2n;
      if (extrap) {
        // fiss_extrp (mod_cmfd.f90:308-335)
        const double domiR = e2n / e1;
        const double cn = domiR / (1.0 - domiR);
        const ff cnf = ff_from_double(cn);
        s_d[1] = cn;
        s_f[0] = cnf.hi;
        s_f[1] = cnf.lo;
      }
    }
    __syncthreads();
    const double e2 = s_d[0];
    double fsum = tot4[1], ser = tot4[2];
    const double fer = tot4[3];
    if (extrap) {
      const double c = s_d[1];
      double acc[2] = {0.0, 0.0};
      ff accf[2] = {ff{0.f, 0.f}, ff{0.f, 0.f}};
      if constexpr (MIXED) {
        const ff cf{s_f[0], s_f[1]};
        float serf = 0.f;
        Dot2 dint;
        for (int b = tid0; b < NB; b += nthr) {
          const ff fo = ld_ff(&P.fs2[old][b]);
          ff fs = ld_ff(&P.fs2[nw][b]);
          fs = ff_add(fs, ff_mul(cf, ff_add(fs, ff{-fo.hi, -fo.lo})));
          st_ff(&P.fs2[nw][b], fs);
          dint.add(ld_ff(&P.vdel2[b]), fs);
          const float af = fabsf(fs.hi), d = fabsf(ff_diff(fs, fo));
          if (af > 1.e-10f && d > serf * af) serf = fmaxf(serf, d / af);
        }
        accf[0] = dint.value();
        accf[1] = ff{serf, 0.f};
      } else
      for (int b = tid0; b < NB; b += nthr) {
        const double fo = fsO[b];
        double fs = fsN[b];
        fs = fma(c, fs - fo, fs);
        fsN[b] = fs;
        acc[0] = fma(G.vdel[b], fs, acc[0]);
        const double af = fabs(fs), d = fabs(fs - fo);
        if (af > 1.e-10 && d > acc[1] * af) acc[1] = fmax(acc[1], d / af);
      }
      double tot[2];
      if (!team_reduce<MIXED, 2, 0x2u>(C, nblk, rank, RED(epoch), acc, accf, tot)) return;
      ++epoch;
      fsum = tot[0];
      ser = tot[1];
    }
    e1 = e2;
    if (threadIdx.x == 0) s_d[2] = P.trans ? Ke : Ke * fsum / f;
    __syncthreads();
    Ke = s_d[2];
    f = fsum;
    cur = nw;

    const bool nodal = P.do_nodal && (p % P.nupd) == 0;
    const bool bad = !isfinite(Ke) || !isfinite(fsum);
    const bool conv = !nodal && ser < P.serc && fer < P.ferc && ndmax < kF1em2;
    const bool maxr = !nodal && !conv && p >= P.nout;
    if (lead) {
      const int q = p - 1;
      if (q < P.nout) {
        P.tr_k[q] = Ke;
        P.tr_ser[q] = ser;
        P.tr_fer[q] = fer;
        P.tr_flags[q] = extrap ? 1 : 0;
        P.tr_ndmax[q] = ndmax;
      }
    }
    if (bad || nodal || conv || maxr) {
      if constexpr (MIXED) {
        // back to the FP64 flux and fission source for the host and the nodal update
        for (int b = tid0; b < NB; b += nthr) {
          for (int g = 0; g < ng; ++g)
            P.phi[cur][(size_t)g * NBH + b] = ff_to_double(ld_ff(&P.x2[cur][(size_t)g * NBH + b]));
          P.fs[cur][b] = ff_to_double(ld_ff(&P.fs2[cur][b]));
        }
      }
      if (lead) {
        C->Ke = Ke;
        C->f = f;
        C->e1 = e1;
        C->ser = ser;
        C->fer = fer;
        C->p = p;
        C->p_total = ptot;
        C->cur = cur;
        C->nodal_due = nodal ? 1 : 0;
        C->converged = conv ? 1 : 0;
        C->max_reached = maxr ? 1 : 0;
        C->need_prologue = 0;
        if (bad) set_status(C, ADP_ERR_NAN);
        __threadfence();
      }
      return;
    }
  }
#undef RED
}


}  // namespace adp
