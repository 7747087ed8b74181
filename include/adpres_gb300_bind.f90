!
! adpres_gb300_bind.f90 -- Fortran 2003 ISO_C_BINDING interface to the C ABI
! declared in adpres_gb300.h, for a Fortran host (such as ADPRES) that
! replaces its own outer()/outer_ad() (mod_cmfd.f90:415, :602) and PowDis
! (:1290) with the GB300 solver.  Arrays are passed in the host's own
! column-major layouts (node index fastest), 1-based indices as in sdata.
!
! This module has not been compiled in the build environment, which has no
! Fortran compiler; it follows the C declarations one to one.
!
module adpres_gb300_bind
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: ADP_OK = 0
  integer(c_int), parameter :: ADP_FORWARD = 0, ADP_ADJOINT = 1, ADP_FROZEN_DN = 4
  integer(c_int), parameter :: ADP_KERN_FDM = 0, ADP_KERN_PNM = 1, ADP_KERN_SANM = 2
  integer(c_int), parameter :: ADP_FP64 = 0, ADP_MIXED = 1

  type, bind(C) :: adp_geom
    integer(c_int) :: nxx, nyy, nzz
    integer(c_int) :: nnod
    type(c_ptr)    :: ix, iy, iz          ! int[nnod]
    type(c_ptr)    :: xdel, ydel, zdel    ! double[nxx], [nyy], [nzz]
    integer(c_int) :: east, west, north, south, bottom, top
  end type

  type, bind(C) :: adp_opts
    integer(c_int) :: ng, nin, nout, nac, nupd
    real(c_double) :: serc, ferc
    integer(c_int) :: kern, precision
  end type

  type, bind(C) :: adp_report
    integer(c_int) :: outers, converged, nodal_updates
    real(c_double) :: keff, ser, fer, ndmax
    integer(c_int) :: im, jm, km
    integer(c_int) :: trace_cap
    type(c_ptr)    :: trace_k, trace_ser, trace_fer, trace_flags, trace_ndmax
    real(c_double) :: device_ms
  end type

  ! feedback tables (mod_xsec.f90:11-46, 230-303, 394-521); the pointers
  ! are c_loc of the reference's arrays (xsigtr(nmat,ng), ..., the change
  ! tables of each card, fbmap gathered per node)
  type, bind(C) :: adp_fb_tables
    integer(c_int) :: nmat
    type(c_ptr)    :: xsigtr, xsiga, xnuf, xsigf, xsigs, chi, mat, dc
    integer(c_int) :: nstate
    type(c_ptr)    :: kind, ref, dsig          ! int[nstate], double[nstate], c_ptr[5*nstate]
    integer(c_int) :: nbank
    type(c_ptr)    :: rsig, bank               ! c_ptr[5], int[nnod]
    real(c_double) :: coreh, pos0, ssize
  end type

  type, bind(C) :: adp_trans_opts
    integer(c_int) :: nf
    type(c_ptr)    :: beta, lambda, velo   ! double[nf], [nf], [ng]
    real(c_double) :: theta
    integer(c_int) :: extr
  end type

  type, bind(C) :: adp_trans_result
    real(c_double) :: rho, rho_dollar, relpow, power
    integer(c_int) :: maxi, outers
    real(c_double) :: device_ms
  end type

  interface
    integer(c_int) function adp_create(geom, opts, h) bind(C, name="adp_create")
      import :: adp_geom, adp_opts, c_int, c_ptr
      type(adp_geom), intent(in) :: geom
      type(adp_opts), intent(in) :: opts
      type(c_ptr), intent(out)   :: h
    end function

    integer(c_int) function adp_destroy(h) bind(C, name="adp_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_size_t) function adp_last_error(h, buf, len) bind(C, name="adp_last_error")
      import :: c_size_t, c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_size_t), value :: len
    end function

    integer(c_int) function adp_xs_updt(h, nmat, xsigtr, xsiga, xnuf, xsigf, chi, mat, xsigs, dc) &
        bind(C, name="adp_xs_updt")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nmat
      real(c_double), intent(in) :: xsigtr(*), xsiga(*), xnuf(*), xsigf(*), chi(*), xsigs(*), dc(*)
      integer(c_int), intent(in) :: mat(*)
    end function

    ! node tables sigtr/siga/nuf/sigf(nnod, ng), sigs(nnod, ng, ng): the
    ! host's XS_updt with its feedback updates (mod_xsec.f90:11-46) hands
    ! its results over here before each outer (th::cbsearch, mod_th.f90:752)
    integer(c_int) function adp_xs_updt_nodes(h, nmat, sigtr, siga, nuf, sigf, chi, mat, sigs, dc) &
        bind(C, name="adp_xs_updt_nodes")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nmat
      real(c_double), intent(in) :: sigtr(*), siga(*), nuf(*), sigf(*), chi(*), sigs(*), dc(*)
      integer(c_int), intent(in) :: mat(*)
    end function

    integer(c_int) function adp_fb_set(h, t) bind(C, name="adp_fb_set")
      import :: c_int, c_ptr, adp_fb_tables
      type(c_ptr), value :: h
      type(adp_fb_tables), intent(in) :: t
    end function

    integer(c_int) function adp_fb_updt(h, state, bpos) bind(C, name="adp_fb_updt")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: state(*), bpos(*)   ! bcon, ftem, mtem, cden as given; bank positions
    end function

    ! tip(b) is 0-based from the bottom (-1: no plane holds the tip)
    integer(c_int) function adp_fb_rod_tips(nzz, zdel, coreh, pos0, ssize, nbank, bpos, tip, vf) &
        bind(C, name="adp_fb_rod_tips")
      import :: c_int, c_double
      integer(c_int), value :: nzz, nbank
      real(c_double), intent(in) :: zdel(*), bpos(*)
      real(c_double), value :: coreh, pos0, ssize
      integer(c_int), intent(out) :: tip(*)
      real(c_double), intent(out) :: vf(*)
    end function

    integer(c_int) function adp_set_xs(h, nmat, D, sigr, nuf, sigf, chi, mat, sigs, dc) bind(C, name="adp_set_xs")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nmat
      real(c_double), intent(in) :: D(*), sigr(*), nuf(*), sigf(*), chi(*), sigs(*), dc(*)
      integer(c_int), intent(in) :: mat(*)
    end function

    integer(c_int) function adp_outer(h, mode, popt, rep) bind(C, name="adp_outer")
      import :: c_int, c_ptr, adp_report
      type(c_ptr), value :: h
      integer(c_int), value :: mode, popt
      type(adp_report), intent(inout) :: rep
    end function

    integer(c_int) function adp_get_state(h, f0, fs0, keff, dn) bind(C, name="adp_get_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: f0(*), fs0(*), keff, dn(*)
    end function

    integer(c_int) function adp_set_state(h, f0, fs0, keff, dn) bind(C, name="adp_set_state")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: f0(*), fs0(*), keff, dn(*)
    end function

    integer(c_int) function adp_reset(h) bind(C, name="adp_reset")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function adp_power(h, p) bind(C, name="adp_power")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: p(*)
    end function

    ! dkdp(nnod, ng, 4+ng) and psi(nnod, ng); pass c_null_ptr-free arrays
    integer(c_int) function adp_adjoint_sens(h, tol, dkdp, psi, rep) bind(C, name="adp_adjoint_sens")
      import :: c_int, c_ptr, c_double, adp_report
      type(c_ptr), value :: h
      real(c_double), value :: tol
      real(c_double), intent(out) :: dkdp(*), psi(*)
      type(adp_report), intent(inout) :: rep
    end function

    ! the same with nod%dn held at the forward solution
    integer(c_int) function adp_adjoint_sens_frozen(h, tol, dkdp, psi, rep) bind(C, name="adp_adjoint_sens_frozen")
      import :: c_int, c_ptr, c_double, adp_report
      type(c_ptr), value :: h
      real(c_double), value :: tol
      real(c_double), intent(out) :: dkdp(*), psi(*)
      type(adp_report), intent(inout) :: rep
    end function

    ! single stages: the CMFD matrix A7(nnod, ng, 7), one nodal update, S1..S3
    integer(c_int) function adp_get_matrix(h, A7) bind(C, name="adp_get_matrix")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: A7(*)
    end function
    integer(c_int) function adp_nodal_step(h, rep) bind(C, name="adp_nodal_step")
      import :: c_int, c_ptr, adp_report
      type(c_ptr), value :: h
      type(adp_report), intent(inout) :: rep
    end function
    integer(c_int) function adp_get_nodal_sources(h, S) bind(C, name="adp_get_nodal_sources")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: S(*)
    end function

    ! time limit of a grid-barrier wait in seconds (0: 2 s)
    integer(c_int) function adp_set_wait_limit(h, seconds) bind(C, name="adp_set_wait_limit")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), value :: seconds
    end function

    ! failure injection for tests: every barrier wait of the next outers runs out
    integer(c_int) function adp_test_missing_block(h, on) bind(C, name="adp_test_missing_block")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: on
    end function

    ! reverse-mode derivative of one nodal update at the current state
    integer(c_int) function adp_nodal_vjp(h, lam, phibar, dnbar, kbar, sigbar, resid) bind(C, name="adp_nodal_vjp")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: lam(*)
      real(c_double), intent(out) :: phibar(*), dnbar(*), sigbar(*)
      real(c_double), intent(out) :: kbar, resid
    end function

    ! output edits of control::forward (mod_io.f90:3267-3644)
    integer(c_int) function adp_edit_asmpow(h, nx, ny, xdiv, ydiv, fasm, imax, jmax) bind(C, name="adp_edit_asmpow")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nx, ny
      integer(c_int), intent(in) :: xdiv(*), ydiv(*)
      real(c_double), intent(out) :: fasm(*)
      integer(c_int), intent(out) :: imax, jmax
    end function

    integer(c_int) function adp_edit_axipow(h, nz, zdiv, faxi, kmax) bind(C, name="adp_edit_axipow")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nz
      integer(c_int), intent(in) :: zdiv(*)
      real(c_double), intent(out) :: faxi(*)
      integer(c_int), intent(out) :: kmax
    end function

    integer(c_int) function adp_edit_asmflux(h, nx, ny, xdiv, ydiv, norm, fasm, negative) &
        bind(C, name="adp_edit_asmflux")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nx, ny
      integer(c_int), intent(in) :: xdiv(*), ydiv(*)
      real(c_double), value :: norm
      real(c_double), intent(out) :: fasm(*)
      integer(c_int), intent(out) :: negative
    end function

    ! adjoint-weighted edits (mod_trans.f90:648-746); sigrp may be c_null_ptr
    integer(c_int) function adp_reactivity(h, af, sigrp, rho) bind(C, name="adp_reactivity")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: af(*)
      type(c_ptr), value :: sigrp
      real(c_double), intent(out) :: rho
    end function

    integer(c_int) function adp_core_beta(h, af, nmat, nf, ibeta, mat, beta) bind(C, name="adp_core_beta")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(in) :: af(*), ibeta(*)
      integer(c_int), value :: nmat, nf
      integer(c_int), intent(in) :: mat(*)
      real(c_double), intent(out) :: beta
    end function

    ! rod ejection transient (mod_trans.f90:17-640)
    integer(c_int) function adp_trans_init(h, opts, af, r0) bind(C, name="adp_trans_init")
      import :: c_int, c_ptr, c_double, adp_trans_opts, adp_trans_result
      type(c_ptr), value :: h
      type(adp_trans_opts), intent(in) :: opts
      real(c_double), intent(in) :: af(*)
      type(adp_trans_result), intent(out) :: r0
    end function

    integer(c_int) function adp_trans_step(h, dt, omeg_mode, r) bind(C, name="adp_trans_step")
      import :: c_int, c_ptr, c_double, adp_trans_result
      type(c_ptr), value :: h
      real(c_double), value :: dt
      integer(c_int), value :: omeg_mode
      type(adp_trans_result), intent(out) :: r
    end function
  end interface

end module adpres_gb300_bind
