/*
 * adpres_gb300.h -- C ABI of the GB300 (sm_103a) static k-eigenvalue solver.
 *
 * This ABI replaces ADPRES's module procedures `outer(popt)` and
 * `outer_ad(popt)` (src/mod_cmfd.f90:415 and :602) together with the state
 * they read and write through MODULE sdata (src/mod_data.f90), `PowDis`
 * (src/mod_cmfd.f90:1290) and the static part of `XS_updt`
 * (src/mod_xsec.f90:11-46).  The reference has no FFI of its own: its seam
 * is those procedures plus the sdata globals, so every entry point below
 * names the routine or globals it stands in for.
 *
 * Conventions
 *  - Plain C types only; host pointers are borrowed for the duration of the
 *    call and copied to or from device memory owned by the handle.
 *  - Arrays use the reference's Fortran column-major layouts with the node
 *    index fastest: f0(nnod,ng), dn(nnod,ng,6), sigs(nnod,ng,ng) with
 *    sigs(n,g,h) the g -> h scattering, dc(nnod,ng,6), chi(nmat,ng).
 *    Face order of df/dn/dc is X+, X-, Y+, Y-, Z+, Z- (mod_data.f90:59-60).
 *  - Node indices ix/iy/iz and material numbers mat are 1-based, in the
 *    reference node order (mod_io.f90:1317-1330).
 *  - Every call returns an adp_status; 0 is success.  Where the reference
 *    STOPs the process, the ABI returns a status and the handle stays usable
 *    (its solver state after an error is unspecified).
 *  - A handle is not thread-safe; calls on one handle must be serialised.
 *    Each handle owns one CUDA stream on the device current at adp_create.
 */
#ifndef ADPRES_GB300_H
#define ADPRES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum adp_status {
  ADP_OK = 0,
  ADP_ERR_INPUT = 1,        /* invalid geometry, options or arguments          */
  ADP_ERR_BADXS = 2,        /* check_xs / Dsigr_updt failures (mod_xsec.f90:90-226) */
  ADP_ERR_PIVOT = 3,        /* LU diagonal below 1e-4 (mod_nodal.f90:856-862)  */
  ADP_ERR_DIVERGED = 4,     /* nodal ndmax > 1e3 (mod_nodal.f90:131-142)       */
  ADP_ERR_MAXOUTER = 5,     /* nout outers without convergence (mod_cmfd.f90:498-505) */
  ADP_ERR_ZEROPOWER = 6,    /* total power <= 0 (mod_cmfd.f90:1322-1326)       */
  ADP_ERR_UNSUPPORTED = 7,  /* outside the static k-eigenvalue path           */
  ADP_ERR_CUDA = 8,         /* a CUDA runtime call failed                      */
  ADP_ERR_NAN = 9,          /* non-finite eigenvalue or fission source         */
  ADP_ERR_BREAKDOWN = 10,   /* BiCGSTAB rho, (rs,v) or (t,t) exactly zero      */
  ADP_ERR_TIMEOUT = 11,     /* a device-side wait ran out of its time limit   */
  ADP_ERR_STATE = 12,       /* call made in the wrong order                    */
  ADP_ERR_BOUNDS = 13       /* a device index out of range (only in the range-checked test build) */
} adp_status;

/* ADP_FROZEN_DN may be or-ed into the mode of adp_outer: the outers then
 * keep the nodal coupling coefficients dn at their current values (no nodal
 * update, ndmax taken as 0).  It has no counterpart in the reference; it
 * gives the CMFD eigenvalue at fixed dn that adp_adjoint_sens differentiates. */
typedef enum adp_mode { ADP_FORWARD = 0, ADP_ADJOINT = 1, ADP_FROZEN_DN = 4 } adp_mode;
typedef enum adp_kern { ADP_KERN_FDM = 0, ADP_KERN_PNM = 1, ADP_KERN_SANM = 2 } adp_kern;
typedef enum adp_precision { ADP_FP64 = 0, ADP_MIXED = 1 } adp_precision;

typedef struct adp_handle adp_handle;

/* Geometry: the sdata globals nxx, nyy, nzz, nnod, ix, iy, iz, xdel, ydel,
 * zdel and the boundary conditions xeast..ztop (mod_data.f90:35-43).  The
 * ragged outline (ystag/xstag) is derived from the plane iz == 1 exactly as
 * mod_io.f90:1071-1110 derives it. */
typedef struct adp_geom {
  int nxx, nyy, nzz;
  int nnod;
  const int* ix;            /* [nnod], 1-based */
  const int* iy;            /* [nnod], 1-based */
  const int* iz;            /* [nnod], 1-based */
  const double* xdel;       /* [nxx] */
  const double* ydel;       /* [nyy] */
  const double* zdel;       /* [nzz] */
  int east, west, north, south, bottom, top;   /* 0 zero flux, 1 zero incoming current, 2 reflective */
} adp_geom;

/* Iteration control (%ITER, mod_data.f90:78-86; %KERN, mod_data.f90:200). */
typedef struct adp_opts {
  int ng;                   /* energy groups                                   */
  int nin;                  /* BiCGSTAB iterations per group solve (default 2) */
  int nout;                 /* maximum outer iterations (default 500)          */
  int nac;                  /* fission-source extrapolation interval (5)       */
  int nupd;                 /* nodal update interval; <= 0 selects
                               ceiling((nxx+nyy+nzz)/2.5) (mod_io.f90:1363)    */
  double serc;              /* fission-source criterion; <= 0 selects the
                               reference default (double)1.e-5f               */
  double ferc;              /* flux criterion; <= 0 selects (double)1.e-5f     */
  int kern;                 /* adp_kern                                        */
  int precision;            /* adp_precision                                   */
} adp_opts;

/* Outcome of one adp_outer call.  The trace arrays are optional (NULL or
 * trace_cap == 0); when given, entry t holds outer t+1 of this call, i.e. the
 * values ADPRES prints per outer (mod_cmfd.f90:492). */
typedef struct adp_report {
  int outers;               /* outer iterations performed by this call         */
  int converged;            /* 1 when ser<serc, fer<ferc and ndmax<1e-2        */
  int nodal_updates;
  double keff, ser, fer, ndmax;
  int im, jm, km;           /* node of the last ndmax (mod_nodal.f90:333-337)  */
  int trace_cap;
  double* trace_k;
  double* trace_ser;
  double* trace_fer;
  int* trace_flags;         /* bit 0: source extrapolated, bit 1: nodal update */
  double* trace_ndmax;
  double device_ms;         /* device time of the call (CUDA events)           */
} adp_report;

/* Device timers accumulated over the life of a handle (CUDA events on the
 * handle's stream). */
typedef struct adp_timers {
  double outer_kernel_ms;   /* persistent CMFD kernel                          */
  long outer_kernel_launches;
  double nodal_ms;          /* nodal update kernels + matrix re-assembly       */
  long nodal_updates;
  double other_ms;
  long outers;              /* outer iterations performed                      */
  long bicg_rows;           /* BiCGSTAB row-iterations (rows x nin x groups x outers) */
  int grid_blocks, block_threads;
  double adjoint_ms;        /* adp_adjoint_sens: transpose, adjoint solve, contraction */
  long adjoint_outers;
} adp_timers;

/* -- handle life cycle ---------------------------------------------------- */

/* Allocate the device state for one core (the allocations ADPRES makes on
 * the first calls of outer/matrix_setup/coup_coef, mod_cmfd.f90:25-33,
 * :232-241, :448-454). */
adp_status adp_create(const adp_geom* geom, const adp_opts* opts, adp_handle** out);
adp_status adp_destroy(adp_handle* h);

/* Copy of the last error message of the handle (or of the last failed
 * adp_create when h is NULL) into buf; returns the full message length. */
size_t adp_last_error(const adp_handle* h, char* buf, size_t len);

/* -- cross sections ------------------------------------------------------- */

/* Node-wise cross sections as outer() reads them from sdata: D, sigr, nuf,
 * sigf (nnod,ng), chi (nmat,ng) with mat (nnod), sigs (nnod,ng,ng) and the
 * ADFs dc (nnod,ng,6; NULL means all 1, mod_io.f90:307-312).  Resets the
 * nodal constants that depend on them. */
adp_status adp_set_xs(adp_handle* h, int nmat, const double* D, const double* sigr, const double* nuf,
                      const double* sigf, const double* chi, const int* mat, const double* sigs,
                      const double* dc);

/* XS_updt on the device (mod_xsec.f90:11-46, static path): node cross
 * sections from the material tables through mat (base_updt :172-195), then
 * D = 1/(3 sigtr) and sigr = siga + sum_{h/=g} sigs(g->h) (Dsigr_updt
 * :199-226) and the checks of check_xs (:90-168).  Material tables are
 * (nmat,ng) and (nmat,ng,ng). */
adp_status adp_xs_updt(adp_handle* h, int nmat, const double* xsigtr, const double* xsiga, const double* xnuf,
                       const double* xsigf, const double* chi, const int* mat, const double* xsigs,
                       const double* dc);

/* The same from node-wise tables (nnod,ng) and (nnod,ng,ng), for perturbed
 * cores whose nodes no longer share material values. */
adp_status adp_xs_updt_nodes(adp_handle* h, int nmat, const double* sigtr, const double* siga, const double* nuf,
                             const double* sigf, const double* chi, const int* mat, const double* sigs,
                             const double* dc);

/* The feedback tables of XS_updt (mod_xsec.f90:11-46) kept on the device,
 * so that a boron search or a transient step hands over a few numbers
 * instead of node tables.  Per state variable a change table set for
 * bcon_updt, ftem_updt, mtem_updt, cden_updt (:394-521) and one for the
 * control rods (crod_updt, :230-303).  Every table set is sigtr, siga, nuf,
 * sigf (nmat,ng) and sigs (nmat,ng,ng), in that order. */
#define ADP_FB_MAX_STATE 4
#define ADP_FB_MAX_BANKS 64
typedef enum adp_fb_kind {
  ADP_FB_BORON = 0,           /* x += dx (bcon - rbcon)                        */
  ADP_FB_FUEL_TEMP = 1,       /* x += dx (sqrt(ftem) - sqrt(rftem))            */
  ADP_FB_MOD_TEMP = 2,        /* x += dx (mtem - rmtem)                        */
  ADP_FB_COOL_DENS = 3        /* x += dx (cden - rcden)                        */
} adp_fb_kind;

typedef struct adp_fb_tables {
  int nmat;
  const double* xsigtr;       /* base material tables (the %XSEC values)      */
  const double* xsiga;
  const double* xnuf;
  const double* xsigf;
  const double* xsigs;
  const double* chi;          /* (nmat,ng)                                     */
  const int* mat;             /* (nnod), 1-based                               */
  const double* dc;           /* ADFs (nnod,ng,6) or NULL (all 1)              */
  int nstate;                 /* 0..ADP_FB_MAX_STATE state cards, applied in
                                 this order (the reference's: boron, fuel
                                 temperature, moderator temperature, coolant
                                 density)                                      */
  const int* kind;            /* [nstate] adp_fb_kind                          */
  const double* ref;          /* [nstate] reference values                     */
  const double* const* dsig;  /* [5 * nstate]: state s, table q at 5 s + q     */
  int nbank;                  /* 0 (no %CROD) .. ADP_FB_MAX_BANKS              */
  const double* const* rsig;  /* [5] rod change tables                         */
  const int* bank;            /* (nnod) bank of the node's column, 0 unrodded  */
  double coreh, pos0, ssize;  /* core height, zero-step position, step size    */
} adp_fb_tables;

/* Uploads the tables; they stay until the next adp_fb_set or adp_destroy. */
adp_status adp_fb_set(adp_handle* h, const adp_fb_tables* t);

/* XS_updt at state values state[nstate] (bcon, ftem, ... as the tables'
 * kinds) and bank positions bpos[nbank] (steps), on the device: the state
 * changes on the material tables in card order, base_updt, the rods (a
 * node above the rod tip gets x + dx, the node holding the tip x + w dx
 * with w its rodded fraction, then negative siga, nuf, sigf and sigs of
 * rodded columns become 0), then D, sigr and the checks as adp_xs_updt. */
adp_status adp_fb_updt(adp_handle* h, const double* state, const double* bpos);

/* The rod tips adp_fb_updt uses (crod_updt, mod_xsec.f90:239-263): for each
 * bank position bpos[b] (steps), the plane (0-based, bottom up) holding the
 * rod tip, walking down from the top of the core, or -1 when none holds it
 * (every plane of the bank's columns is then fully rodded), and the rodded
 * fraction vf[b] of that plane.  Host arithmetic only; no device call. */
adp_status adp_fb_rod_tips(int nzz, const double* zdel, double coreh, double pos0, double ssize, int nbank,
                           const double* bpos, int* tip, double* vf);

/* -- solver --------------------------------------------------------------- */

/* Time limit of every grid-barrier wait of the persistent kernels of this
 * handle, in seconds (0: the default, 2 s; at most 60).  A wait that runs
 * out records ADP_ERR_TIMEOUT, the kernel returns and the call returns that
 * status; the handle stays usable.  No counterpart in the reference. */
adp_status adp_set_wait_limit(adp_handle* h, double seconds);

/* Failure injection for tests, on the host side: with on != 0 the forward
 * adp_outer launches count one block more than they launch, so no grid
 * barrier can complete and every wait runs out after the wait limit
 * (ADP_ERR_TIMEOUT) -- the way to exercise the timeout path without a GPU
 * fault.  on = 0 restores normal launches.  No counterpart in the
 * reference. */
adp_status adp_test_missing_block(adp_handle* h, int on);

/* One call of outer(popt) (mode ADP_FORWARD) or outer_ad(popt) (ADP_ADJOINT)
 * on the state held by the handle: matrix_setup(1), the first-call start
 * f0 = 1, k = 1 (mod_cmfd.f90:448-454, :635-641), then outer iterations with
 * nin BiCGSTAB steps per group, fission-source extrapolation every nac
 * outers, the SANM/PNM nodal update every nupd outers and the reference's
 * convergence test.  popt only matters for the adjoint (mod_cmfd.f90:635,680). */
adp_status adp_outer(adp_handle* h, int mode, int popt, adp_report* report);

/* The in/out sdata state of outer(): f0(nnod,ng), fs0(nnod), Ke and
 * nod%dn (nnod,ng,6).  Any pointer may be NULL.  adp_set_state marks the
 * handle as started, so the next adp_outer warm-starts from it as ADPRES
 * does when outer() is called again (mod_th.f90:774-795). */
adp_status adp_get_state(adp_handle* h, double* f0, double* fs0, double* keff, double* dn);
adp_status adp_set_state(adp_handle* h, const double* f0, const double* fs0, const double* keff,
                         const double* dn);

/* Return the solver state to that of a fresh ADPRES process (dn = 0 as on
 * coup_coef's first call, mod_cmfd.f90:25-33; the next adp_outer of either
 * mode starts from f0 = 1, k = 1; ndmax = 0).  Cross sections are kept.
 * Device-side only: no host copies. */
adp_status adp_reset(adp_handle* h);

/* PowDis (mod_cmfd.f90:1290-1333): p(n) = sum_g max(0, f0 sigf vdel),
 * normalised to sum 1.  p has nnod entries. */
adp_status adp_power(adp_handle* h, double* p);

/* PowDis without a handle and without allocating: no counterpart in the
 * reference.  For callers that cannot call cudaMalloc -- a host whose device
 * memory belongs to another allocator (a framework's caching allocator, or a
 * budget fixed at start-up), or a path where cudaMalloc/cudaFree and their
 * implicit device synchronisation are not acceptable.  f0 (nnod,ng) and
 * sigf (nnod,ng) (node index fastest), vdel (nnod) and the output p (nnod)
 * are device pointers owned by the caller; stream is a cudaStream_t (NULL
 * for the default stream); the call returns when p is written.  Limits:
 * 1 <= ng <= 8 and nnod * ng <= 2^31 - 1; larger sizes return
 * ADP_ERR_INPUT.  Its scratch (block partial sums and a status word) is a
 * fixed 8,448-byte array of device memory inside the library, held on every
 * GPU that loads the library until the process exits.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress), so
 * make the first call on each device before any stream capture; the
 * address is kept for the life of the process, so a cudaDeviceReset (or
 * any re-creation of the device's primary context) between calls is not
 * supported.  All calls share the array: calls that overlap on the GPU
 * race; serialise them.  On an error the contents of p are unspecified (on
 * ADP_ERR_ZEROPOWER it holds the unnormalised per-node powers).  Errors:
 * message through adp_last_error(NULL). */
adp_status adp_power_noalloc(int nnod, int ng, const double* f0, const double* sigf, const double* vdel, double* p,
                             void* stream);

/* Discrete adjoint and dk/dSigma; no counterpart in the reference (its
 * outer_ad, mod_cmfd.f90:602-699, solves the physical adjoint with its own
 * adjoint nodal update and the untransposed matrix).  Needs a converged
 * forward adp_outer on the current cross sections.
 *
 * The converged state is the fixed point of the CMFD eigenproblem
 * M(d) phi = (1/k) F phi (matrix_setup + TSrc, mod_cmfd.f90:217-304,
 * :1006-1033) and of the nodal update d = N(phi, d, k) of the faces'
 * coupling coefficients (nodal_update, mod_nodal.f90:18-278).  This call
 * returns the derivative of k at that fixed point:
 *   dk/dp = KS_p (1 + s) + lam^T dN/dp + Gam^T ((1/k) dF/dp - dM/dp) phi,
 * where KS_p = k^2 psi^T ((1/k) dF/dp - dM/dp) phi / (psi^T F phi) is the
 * derivative at frozen d with psi the adjoint of M^T psi = (1/k) F^T psi
 * (solved with the persistent kernel on the transposed stencil, source
 * weights and group sweep of outer_ad, from psi = 1 until ser < tol and
 * fer < tol; tol <= 0: the handle's serc and ferc), lam the adjoint of the
 * face coefficients, s = lam^T dN/dk, and Gam the generalized adjoint of
 * the flux: (M - F/k)^T Gam = lam^T dN/dphi with Gam^T F phi = 0.  lam and
 * Gam are iterated together as the forward iteration is (rounds of
 * 2 nac outers of Gam, each followed by the reverse-mode
 * derivative of the nodal update at the converged state and an update of
 * lam) until lam's relative change is below tol (at least 1e-13).  For the
 * FDM kernel (d = 0) the frozen-d derivative is the whole derivative.  The
 * result is the derivative of the fixed point the forward state sits at:
 * converge the forward solve tightly (small serc, ferc) for a tight result.
 * report->ndmax is the fixed-point residual max |N(phi, d, k) - d| at the
 * state, report->nodal_updates the rounds, report->ser lam's last relative
 * change.  Needs ng <= 4 for SANM/PNM (ADP_ERR_UNSUPPORTED otherwise).
 *
 * dkdp (nnod, ng, 4 + ng), node index fastest:
 * [:,g,1] dk/dD_g, [:,g,2] dk/dsiga_g, [:,g,3] dk/dnuf_g, [:,g,4]
 * dk/dsigtr_g (= -3 D_g^2 dk/dD_g, the chain rule of D = 1/(3 sigtr)),
 * [:,g,4+h] dk/dsigs(g->h) (through sigr and the scattering source; 0 for
 * h = g).  psi (nnod, ng) receives the adjoint flux (unnormalised); either
 * output may be NULL.  report (may be NULL) describes the adjoint solve
 * (keff is its eigenvalue; outers count the adjoint and Gam outers).  The
 * forward state is left unchanged. */
adp_status adp_adjoint_sens(adp_handle* h, double tol, double* dkdp, double* psi, adp_report* report);

/* The derivative with the faces' coupling coefficients d held at the
 * forward solution (KS_p above): the derivative of the CMFD eigenvalue at
 * fixed d, which adp_outer(ADP_FORWARD | ADP_FROZEN_DN) solves for.  Same
 * arguments and outputs as adp_adjoint_sens.  No counterpart in the
 * reference. */
adp_status adp_adjoint_sens_frozen(adp_handle* h, double tol, double* dkdp, double* psi, adp_report* report);

/* -- single stages, for per-stage parity checks ---------------------------- */

/* The CMFD matrix of matrix_setup(1) (mod_cmfd.f90:217-304; coup_coef
 * first, :11-137) at the current cross sections and dn: A7 (nnod, ng, 7),
 * node index fastest, columns in the reference's order z-, y-, x-,
 * diagonal, x+, y+, z+ (0 where a node has no neighbour).  No counterpart
 * in the reference (its A is module state). */
adp_status adp_get_matrix(adp_handle* h, double* A7);

/* One nodal update (nodal_upd with the static cal_mode 1: nodal_update or
 * nodal_update_pnm, mod_nodal.f90:18-278) at the current flux, k and dn,
 * which it overwrites with the new coupling coefficients; report->ndmax and
 * im, jm, km give the maximum change and its location (first maximum in
 * the reference's sweep order).  Statuses as adp_outer's (PIVOT,
 * DIVERGED).  Clears the converged flag that adp_adjoint_sens needs. */
adp_status adp_nodal_step(adp_handle* h, adp_report* report);

/* The zeroth-order transverse-leakage sources S1, S2, S3 of the last nodal
 * update (get_source, mod_nodal.f90:1009-1043): S (nnod, ng, 3). */
adp_status adp_get_nodal_sources(adp_handle* h, double* S);

/* Reverse-mode derivative of one nodal update (nodal_update /
 * nodal_update_pnm, mod_nodal.f90:18-278, static form) at the handle's
 * current state (flux, coupling coefficients dn, eigenvalue, cross
 * sections): the update is a function N(phi, d, k; Sigma) of the flux, the
 * faces' coupling coefficients d, k and the cross sections, and for an
 * adjoint lam of its new coefficients this returns lam^T dN/dphi in phibar
 * (nnod, ng), lam^T dN/dd in dnbar (nnod, ng, 6), lam^T dN/dk in *kbar and
 * lam^T dN/dp in sigbar (nnod, ng, 4 + ng), the dkdp layout of
 * adp_adjoint_sens.  Face arrays use the reference's nod%dn layout; an
 * interior face's coefficient is one variable, held in the slot of the
 * face's plus-side node (its minus face; a boundary face in its own slot):
 * lam is read there and dnbar written there, other slots are ignored on
 * input and 0 on output.  *resid receives max |N(phi, d, k) - d| at the
 * state.  The building block of adp_adjoint_sens; no counterpart in the
 * reference.  Any output may be NULL.  ng <= 4; not for FDM. */
adp_status adp_nodal_vjp(adp_handle* h, const double* lam, double* phibar, double* dnbar, double* kbar,
                         double* sigbar, double* resid);

/* -- output edits of control::forward (mod_control.f90:33-44) -------------- */

/* AsmPow (mod_io.f90:3267-3403): PowDis of the current flux, axially
 * averaged per node column (weights zdel), area-weighted per assembly of
 * xdiv(nx) x ydiv(ny) columns, normalised so that the assemblies with
 * power average 1.  fasm (nx, ny), i fastest; imax/jmax: the first maximum
 * (1-based).  The node power never leaves the device. */
adp_status adp_edit_asmpow(adp_handle* h, int nx, int ny, const int* xdiv, const int* ydiv, double* fasm, int* imax,
                           int* jmax);
/* AxiPow (mod_io.f90:3406-3498): PowDis summed over each axial region of
 * zdiv(nz) planes and divided by the region's volume, normalised so that
 * the regions with power average 1.  faxi (nz); kmax: the first maximum. */
adp_status adp_edit_axipow(adp_handle* h, int nz, const int* zdiv, double* faxi, int* kmax);
/* AsmFlux (mod_io.f90:3501-3644): per group, the flux axially averaged per
 * column (weights: node volumes) and area-weighted per assembly; when
 * norm > 0 scaled by norm / (sum of the positive assembly values) * norm
 * (control::forward passes 1.0).  fasm (nx, ny, ng); negative = 1 when an
 * assembly value is negative (the reference prints a warning). */
adp_status adp_edit_asmflux(adp_handle* h, int nx, int ny, const int* xdiv, const int* ydiv, double norm, double* fasm,
                            int* negative);

/* -- adjoint-weighted edits (mod_trans.f90:648-746) ----------------------- */

/* reactivity (mod_trans.f90:648-688) of the handle's current flux and
 * fission source: rho = (src - lea - rem) / fde with the weight af
 * (nnod, ng) (an adjoint flux: outer_ad's, or adp_adjoint_sens's psi), the
 * scattering-in and fission sources, the net leakage of Lxyz from df, dn
 * and the flux, and the removal sigrp (nnod, ng; NULL for the handle's
 * sigr).  For a converged static solution rho = 1 - 1/k for any af. */
adp_status adp_reactivity(adp_handle* h, const double* af, const double* sigrp, double* rho);
/* calc_beta (mod_trans.f90:692-746): core-averaged delayed neutron
 * fraction weighted by af (nnod, ng), from the delayed fractions
 * ibeta (nmat, nf) of the materials mat (nnod), 1 <= nf <= 8. */
adp_status adp_core_beta(adp_handle* h, const double* af, int nmat, int nf, const double* ibeta, const int* mat,
                         double* beta);

/* -- rod ejection transient (mod_trans.f90:17-640, mod_cmfd.f90:800-952) -- */

/* Delayed neutron data and time integration of the transient: nf (1..8)
 * precursor families' fractions and decay constants, ng group velocities,
 * theta of the theta method (%THET, 0.001..1), and whether the exponential
 * flux transformation is on (%EXTR). */
typedef struct adp_trans_opts {
  int nf;
  const double* beta;
  const double* lambda;
  const double* velo;
  double theta;
  int extr;
} adp_trans_opts;

typedef struct adp_trans_result {
  double rho;               /* adjoint-weighted reactivity (mod_trans.f90:648-688) */
  double rho_dollar;        /* rho / total beta                                */
  double relpow;            /* PowTot relative to the initial state            */
  double power;             /* PowTot                                          */
  int maxi;                 /* 1 when the step's outer_tr reached nout          */
  int outers;               /* outers of the step                               */
  double device_ms;
} adp_trans_result;

/* After the steady state of rod_eject (forward outer, k brought to one,
 * the adjoint af (nnod, ng) of outer_ad, the forward outer again): iPden,
 * PowTot and the reactivity of the initial state (rho in absolute units),
 * and the leakage the first step's source needs. */
adp_status adp_trans_init(adp_handle* h, const adp_trans_opts* opts, const double* af, adp_trans_result* r0);
/* One time step of trans_calc (mod_trans.f90:332-479) after the host has
 * moved the rods and uploaded the step's cross sections (adp_xs_updt or
 * adp_xs_updt_nodes): removal sigr + 1/(theta v dt) + omega/v, get_exsrc,
 * outer_tr (the FP64 kernel, or the mixed kernel on a mixed-precision
 * handle; nodal update in its transient form, FP64), uPden,
 * PowTot and the reactivity with the step's XS_updt removal.  omeg_mode 1:
 * omega = log(f0/ft)/dt (rod_eject applies it from the second step on when
 * %EXTR is given), 0: omega = 0.  Reaching nout only sets r->maxi. */
adp_status adp_trans_step(adp_handle* h, double dt, int omeg_mode, adp_trans_result* r);

/* -- batched solves ------------------------------------------------------ */

/* Many independent cores solved together; no counterpart in the reference,
 * whose process solves one core (control::forward, mod_control.f90:11-47).
 * A batch owns one handle per core (adp_batch_core gives it, for
 * adp_get_state and friends) and solves all cores in one persistent
 * cooperative launch captured in a CUDA graph: per core XS_updt, the
 * first-call start, outer iterations with nodal updates and PowDis, each
 * core on a team of thread blocks that synchronise only among themselves.
 * All cores share ng (1..4), kern and precision. */
typedef struct adp_batch adp_batch;

/* Launch shape and schedule: threads per block (256 or 512), the largest
 * team of blocks on one core, grain (for the first schedule, before any
 * solve is timed: cores are split into teams so that a team member's share
 * is about 1/grain of a block's average load; once cores are timed, each
 * takes the smallest team that meets the schedule's target end), blocks
 * per SM (2 with 256 threads selects the kernel built for two
 * resident blocks per SM, 128 registers a thread), and whether the solve is
 * replayed from a captured graph. */
typedef struct adp_batch_config {
  int threads;
  int max_team;
  double grain;
  int blocks_per_sm;
  int use_graph;
} adp_batch_config;

typedef struct adp_batch_result {
  int status;               /* adp_status of the core                          */
  int converged, outers, nodal_updates;
  double keff, ser, fer, ndmax;
  double device_ms;         /* device time of the core (global timer), from    */
                            /* the arrival of its team's last block           */
  int team;                 /* blocks that solved it                           */
} adp_batch_result;

adp_status adp_batch_create(int n, const adp_geom* geoms, const adp_opts* opts, adp_batch** out);
adp_status adp_batch_destroy(adp_batch* b);
size_t adp_batch_last_error(const adp_batch* b, char* buf, size_t len);
/* Node-wise cross sections of core i, as adp_xs_updt_nodes. */
adp_status adp_batch_set_xs(adp_batch* b, int i, int nmat, const double* sigtr, const double* siga, const double* nuf,
                            const double* sigf, const double* chi, const int* mat, const double* sigs,
                            const double* dc);
/* Sets the configuration and re-plans the schedule from the latest per-core
 * times (so a call with the unchanged configuration after a solve re-plans
 * with that solve's times); a change of use_graph alone keeps the schedule. */
adp_status adp_batch_set_config(adp_batch* b, const adp_batch_config* c);
adp_status adp_batch_get_config(const adp_batch* b, adp_batch_config* c);
/* Solve every core from a fresh start; res has n entries (may be NULL);
 * device_ms is the whole launch (CUDA events).  Returns the first failing
 * core's status, or ADP_OK. */
adp_status adp_batch_solve(adp_batch* b, adp_batch_result* res, double* device_ms);
/* Time the batch over the kernel shapes (threads, blocks per SM) = (256, 1),
 * (256, 2), (512, 1) x max_team {4, 8, 16, 32} and keep the fastest: one
 * solve to time the cores, then each candidate solved twice (the second
 * schedule planned with the times of the first), 25 solves of the whole
 * batch.  best_ms is the winner's second solve. */
adp_status adp_batch_autotune(adp_batch* b, adp_batch_config* best, double* best_ms);
/* The schedule a batch would run, computed on the host alone (no GPU, no
 * batch): n cores with weights rows[i] (box rows x groups, the weight
 * before any solve is timed) and, when t_ns is not NULL, each core's
 * measured time t_ns[i] on a team of t_team[i] blocks (the timed,
 * target-end plan, with the duration model t(s) = A (1/s + 0.03)), on
 * `blocks` blocks with c->max_team and c->grain.  Writes team[n], and for
 * each block b its tasks begin[b] .. begin[b+1]-1 (begin has blocks + 1
 * entries) as the core index task_core[k] and the block's rank in that
 * core's team task_rank[k] (cap entries available), and the predicted end
 * (makespan, may be NULL).  ADP_ERR_INPUT on bad arguments or too small a
 * cap (sum of the teams). */
adp_status adp_batch_plan_preview(int n, const double* rows, const double* t_ns, const int* t_team, int blocks,
                                  const adp_batch_config* c, int cap, int* team, int* begin, int* task_core,
                                  int* task_rank, double* makespan);
adp_status adp_batch_core(adp_batch* b, int i, adp_handle** h);
/* Per-outer trace of core i from the last adp_batch_solve (as the trace of
 * adp_report; any array may be NULL); returns the number of entries written
 * (at most cap), or -1 on bad arguments. */
int adp_batch_trace(adp_batch* b, int i, int cap, double* k, double* ser, double* fer, int* flags, double* ndmax);
/* Normalised node power of core i after adp_batch_solve (nnod entries). */
adp_status adp_batch_power(adp_batch* b, int i, double* p);

/* Device timers of the handle. */
adp_status adp_get_timers(const adp_handle* h, adp_timers* t);

/* Launch shape of the persistent CMFD kernel: blocks (0 = automatic: one
 * block per SM at most, the same rows for every thread) and threads per
 * block (0 = automatic: 512, or 256 when 512-thread blocks would leave more
 * than half of the SMs idle).  Results are reproducible for a fixed shape;
 * another shape sums the partial products in another grouping. */
adp_status adp_set_launch(adp_handle* h, int blocks, int threads);

#ifdef __cplusplus
}
#endif

#endif /* ADPRES_GB300_H */
