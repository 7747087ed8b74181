// Kernel parameter blocks and launchers shared by the host side (capi.cu)
// and the kernel translation units (cmfd.cu, nodal.cu).
#pragma once

#include <cuda_runtime.h>

#include "adp_device.cuh"

namespace adp {

// Single-precision default literals of the reference promoted to double.
constexpr double kF1em2 = (double)1.e-2f;   // mod_cmfd.f90:495
constexpr double kF1em4 = (double)10e-5f;   // mod_nodal.f90:856
constexpr double kF1em5 = (double)1.e-5f;   // mod_data.f90:78-79

// Persistent outer-iteration kernel (outer / outer_ad, mod_cmfd.f90:415-699).
struct OuterParams {
  BoxGeom G;
  int ng, nin, nac, nupd, nout, adj, do_nodal, mixed;
  int smem_rows;              // > 0: rows per block of the matrix copy in shared memory
  int trans;                  // 1: outer_tr (mod_cmfd.f90:800-868): source wsrc fs + s0 + exsrc, no k update
  int phantom;                // team members counted by the barriers beyond the launched blocks (0; 1 makes
                              // every barrier wait run out: the host-side test of ADP_ERR_TIMEOUT)
  // Source planes that hold a nonzero value at some node: bit g of src_nz
  // for wsrc of group g, bit a*ng + c of sc_nz for sigs plane [a][c].  P0
  // skips the terms of all-zero planes (adding an exact zero changes no
  // bit of the sum); all ones when unknown.
  unsigned src_nz;
  unsigned long long sc_nz;
  const double* exsrc;        // [ng][NB] external source of the transient step (trans only)
  const float2* exsrc2;       // [ng][NB] external source as (hi, lo) pairs (mixed trans: the generalized adjoint)
  double serc, ferc;
  long long NBH;              // group stride of halo'd arrays
  const double* A;            // [ng][7][NB] FP64 CMFD matrix
  const float* A32;           // [ng][7][NB] FP32 copy (mixed storage)
  double* phi[2];             // [ng][NBH] flux double buffer (halo offset applied)
  double* fs[2];              // [NB] fission source double buffer
  const double* wsrc;         // weight of fs0 in the group source: chi (fwd) / nuf (adj), [ng][NB]
  const double* wfis;         // weight of the flux in the fission source: nuf (fwd) / chi (adj)
  const double* init_phi;     // k_init_flux: start from this flux ([ng][NBH], halo offset applied), else 1
  const double* sigs;         // [ng(from)][ng(to)][NB]
  double* r;                  // Krylov vectors, halo'd [NBH]
  double* rs;
  double2* pv2[2];            // (p, v) pairs, halo'd [NBH], double buffered
  double2* st2;               // (s, t) pairs, halo'd [NBH]
  float* r32;                 // FP32 Krylov vectors (mixed), halo'd [NBH]
  float* rs32;
  float2* pv2f[2];            // FP32 (p, v) and (s, t) pairs (mixed)
  float2* st2f;
  double* red;                // [2][kRedQ][kMaxBlocks]
  // Double-float (hi + lo FP32 pairs) state of the mixed path: the defect
  // correction and the flux and fission-source updates run on these.
  // Each array holds (hi, lo) pairs.
  const float2* A2;           // [ng][7][NB] the FP64 matrix as (A32, A - A32)
  float2* x2[2];              // flux [ng][NBH] (halo offset applied)
  float2* fs2[2];             // fission source [NB]
  const float2* wsrc2;        // [ng][NB]
  const float2* wfis2;
  const float2* sigs2;        // [ng][ng][NB]
  const float2* vdel2;        // [NB]
  OuterCtl* ctl;
  double* tr_k;
  double* tr_ser;
  double* tr_fer;
  int* tr_flags;
  double* tr_ndmax;
};

// Nodal update (mod_nodal.f90) and matrix set-up (mod_cmfd.f90:11-304).
struct NodalParams {
  BoxGeom G;
  int ng, cmode, pnm, nnod, nout;
  double serc, ferc;
  long long NBH;
  const int* act;             // [nnod] box index of each node in reference order
  const double* phi[2];
  const double* D;            // [ng][NB]
  const double* sigr;
  const double* nuf;
  const double* chin;         // chi of the node's material, [ng][NB]
  const double* sigs;         // [ng][ng][NB]
  const double* df;           // [ng][6][NB]
  double* dn;                 // [ng][6][NB]
  const double* dc;           // [ng][6][NB]
  const double* sanm;         // [3][6][ng][NB] SANM constants A,B,E,F,G,H per direction
  double* S;                  // [3][ng][NB] zeroth-order transverse-leakage sources S1..S3
  double* a2;                 // [3][ng][NB]
  double* a4;
  double* L1;
  double* Bc;                 // [3][ng][ng][NB] buckling matrix per node and direction
  const int* evbase;          // [3][NB] sweep-order index of a node's minus face
  double* nd_val;             // [kMaxBlocks] ndmax partials
  long long* nd_key;
  int* nd_loc;
  int nd_blocks;
  const double* exsrc;        // cmode 2: [ng][NB] external source of the transient step
  const double* wnode;        // cmode 2: [NB] 1 - tbeta + dfis of the node
  OuterCtl* ctl;
  double* tr_ndmax;
  int* tr_flags;
};

struct AssembleParams {
  BoxGeom G;
  int ng;
  int with_coupling;          // 1: recompute df first (matrix_setup(1))
  const double* D;
  const double* sigr;
  double* df;
  const double* dn;
  double* A;
  float* A32;
  float2* A2;                 // (A32, A - A32) pairs (mixed path), may be null
  OuterCtl* ctl;              // where the range-checked build reports a bad index (may be null)
};

// Contraction of forward and adjoint fluxes into dk/dSigma (adjoint.cu).
struct SensParams {
  BoxGeom G;
  int ng, nnod;
  long long NBH;
  double keff;                // forward eigenvalue
  const int* act;             // [nnod] box index of each node
  const double* phi;          // forward flux [ng][NBH] (halo offset applied)
  const double* psi;          // discrete adjoint flux, same layout
  const double* D;            // [ng][NB]
  const double* nuf;
  const double* chin;
};

// Reverse-mode derivative of the nodal update (nodal_adj.cu).  Face arrays
// use the [g][6][NB] layout at canonical slots (the minus face of every
// node, the plus face of a node ending its line).
struct NadjParams {
  NodalParams N;              // the forward state being differentiated (cmode 1)
  const double* lam;          // adjoint of the new coupling coefficients
  double* side;               // [2][3][9G + G^2][NB] per-side adjoints of the face stage
  double* nodeu;              // [3][7G + G^2][NB] per-direction adjoints of the node stage
  double* Lbar;               // [3][G][NB] adjoints of the leakages L1..L3
  double* dfbar;              // adjoint of df
  double* dnbar;              // out: lam^T dN/dd
  double* phibar;             // out: lam^T dN/dphi, [G][NB]
  double* kpart;              // [kMaxBlocks] partials of lam^T dN/dk
  double* rpart;              // [kMaxBlocks] partial maxima of |N(state) - d|
  double* scal;               // out: [0] lam^T dN/dk, [1] max |N(state) - d|
  double* out;                // out: lam^T dN/dSigma in the dkdp layout (nnod, G, 4 + G)
};

// One core of a batch (batch.cu): the parameter blocks of its handle plus the
// inputs of the in-kernel cross-section update and power edit.
struct BatchInst {
  OuterParams op;
  NodalParams np;
  AssembleParams ap;          // with_coupling = 1 (start of the solve)
  AssembleParams ap0;         // with_coupling = 0 (after a nodal update)
  const double* sigtr;        // [ng][NB]
  const double* siga;
  const double* sigf;
  double* pbox;               // [NB] normalised node power
  unsigned long long* t_ns;   // [2] globaltimer at the start and the end of the solve
  int kern;                   // adp_kern
  int nnod;
};

// One entry of a block's task list: core `inst`, solved by a team of `size`
// blocks in which this block has rank `rank`.
struct BatchTask {
  int inst, rank, size, pad;
};

// Material tables of base_updt (mod_xsec.f90:172-195), Fortran (nmat, ng)
// and sigs (nmat, ng, ng); null members are not expanded.
struct XsTables {
  const double* sigtr;
  const double* siga;
  const double* nuf;
  const double* sigf;
  const double* chi;
  const double* sigs;
};

// The handle's box planes that base_updt writes: [ng][NB], sigs [ng][ng][NB].
struct XsBox {
  double* sigtr;
  double* siga;
  double* nuf;
  double* sigf;
  double* chin;
  double* sigs;
};

// Feedback update of XS_updt on the device (transfer.cu).  A table set is
// sigtr, siga, nuf, sigf (nmat, G) and sigs (nmat, G, G), Fortran order,
// packed one after another: `tq` doubles per set, table q at off[q].
constexpr int kFbMaxState = 4;
constexpr int kFbMaxBanks = 64;
struct FbParams {
  int nmat, G, nn, nst, nb, plane;
  long long NB;
  long long tq;             // doubles in one table set
  long long off[5];         // start of each table in a set
  const double* base;       // the material tables
  const double* dsig;       // [nst] change sets
  const double* rsig;       // rod change set (nb > 0)
  double* tab;              // the material tables after the state changes
  const double* chi;        // (nmat, G)
  const int* mat;           // (nn) 1-based
  const int* bank;          // (nn) 0 = unrodded column
  const int* act;           // (nn) box index
  double dv[kFbMaxState];   // state change of each card
  int tip[kFbMaxBanks];     // plane of the rod tip (-1: none holds it)
  double vf[kFbMaxBanks];   // rodded fraction of that plane
  XsBox X;
  int* flags;
};

// Launchers (return the launch error, if any)
cudaError_t launch_fb_updt(const FbParams& P, cudaStream_t st);
cudaError_t launch_assemble(const AssembleParams& P, cudaStream_t st);
cudaError_t launch_init_flux(const OuterParams& P, cudaStream_t st);
cudaError_t launch_outer(const OuterParams& P, int blocks, int threads, cudaStream_t st);
// Rows per block of the shared-memory matrix copy for this launch shape
// (0 when it does not fit).
int outer_smem_rows(int NB, int blocks, int threads, int mixed);
int outer_max_blocks_per_sm(int threads, int mixed);
cudaError_t launch_power(const BoxGeom& G, int ng, long long NBH, const double* phi, const double* sigf,
                         double* pbox, double* red, OuterCtl* ctl, cudaStream_t st);
cudaError_t launch_sanm_consts(const NodalParams& P, cudaStream_t st);
cudaError_t launch_nodal(const NodalParams& P, cudaStream_t st);
cudaError_t launch_nodal_prep(const NodalParams& P, cudaStream_t st);   // G <= 4
cudaError_t launch_xs_updt(const BoxGeom& G, int ng, const int* act, int nnod, const double* sigtr,
                           const double* siga, const double* sigs, double* D, double* sigr, OuterCtl* ctl,
                           cudaStream_t st);
cudaError_t launch_transpose(const BoxGeom& G, int ng, const double* A, double* AT, float* AT32, float2* AT2,
                             cudaStream_t st);
// out = (hi, lo) with hi = (float)x, lo = (float)(x - hi) (double-float copies of the mixed path)
cudaError_t launch_split(const double* x, float2* out, long long n, cudaStream_t st);
cudaError_t launch_sens(const SensParams& P, double* part, double* out, cudaStream_t st);
// out = KS (1 + scal[0]) + NS + P.psi^T (lambda dF/dp - dM/dp) phi
cudaError_t launch_sens_total(const SensParams& P, const double* KS, const double* NS, const double* scal,
                              double* out, cudaStream_t st);
// derivative through the nodal update (nodal_adj.cu); G <= 4
cudaError_t launch_nodal_adjoint(const NadjParams& Q, cudaStream_t st);
size_t nadj_side_doubles(int ng, long long NB);
size_t nadj_nodeu_doubles(int ng, long long NB);
cudaError_t launch_face_contract(const BoxGeom& G, int ng, int nnod, long long NBH, const int* act,
                                 const double* phi, const double* w, double scale, double* out, cudaStream_t st);
cudaError_t launch_lam_update(const BoxGeom& G, int ng, int nnod, const int* act, const double* Kd,
                              const double* dnbar, const double* cG, const double* scal, double* lam, double* dlam,
                              double* part, cudaStream_t st);
cudaError_t launch_lam_extrap(const BoxGeom& G, int ng, int nnod, const int* act, const double* dlam, double c,
                              double* lam, cudaStream_t st);
int lam_update_blocks(int ng, int nnod);
cudaError_t launch_gpt_source(const BoxGeom& G, int ng, int nnod, long long NBH, const int* act, const double* phi,
                              const double* v, double* part, double* src, cudaStream_t st);
cudaError_t launch_gpt_project(const BoxGeom& G, int ng, int nnod, long long NBH, const int* act,
                               const double* chin, const double* nuf, const double* phi, const double* psi,
                               double* part, double* gam, double* fsg, cudaStream_t st);
cudaError_t launch_scale_planes(const double* in, double s, double* out, long long n, cudaStream_t st);
// node-order <-> box transfers (transfer.cu): host layout a(nn, A, B), node
// fastest; device planes [A][B] of stride `stride` indexed by act[n]
cudaError_t launch_nodes_to_box(const double* src, double* dst, const int* act, int nn, int A, int B,
                                long long dstride, int chk, int* flags, cudaStream_t st);
cudaError_t launch_box_to_nodes(const double* src, double* dst, const int* act, int nn, int A, int B,
                                long long sstride, cudaStream_t st);
cudaError_t launch_fill_box(double* dst, const int* act, int nn, int ncomp, long long dstride, double v,
                            cudaStream_t st);
// Planes of chi, nu*fission and sigs that hold a nonzero value at some
// active node: out[0] bit g (chi), out[1] bit g (nuf), out[2] | out[3] << 32
// bit g*G + h (sigs g -> h).  G <= 8; out must be zero on entry.
cudaError_t launch_xs_nonzero(const double* chin, const double* nuf, const double* sigs, const int* act, int nn,
                              int G, long long NB, unsigned* out, cudaStream_t st);
cudaError_t launch_base_updt(const XsTables& T, const int* mat, const int* act, int nn, int nmat, int G, long long NB,
                             const XsBox& X, int* flags, cudaStream_t st);
// batched solve (batch_k_*.cu): a cooperative launch of `blocks` blocks
// minb: blocks per SM the kernel's registers are sized for (1, or 2 with 256 threads)
cudaError_t launch_batch(bool mixed, int ng, int threads, int minb, int blocks, const BatchInst* insts,
                         const BatchTask* tasks, const int* task_begin, cudaStream_t st);
int batch_max_blocks_per_sm(bool mixed, int ng, int threads, int minb);
bool batch_supported(int ng, int threads);
cudaError_t launch_batch_init(const BatchInst* insts, int n, cudaStream_t st);
cudaError_t launch_batch_gather(const BatchInst* insts, int n, OuterCtl* out, cudaStream_t st);

}  // namespace adp
