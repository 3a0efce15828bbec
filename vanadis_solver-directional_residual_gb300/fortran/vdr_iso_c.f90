! vdr_iso_c.f90 -- ISO_C_BINDING interfaces of libvdr.so for the Vanadis
! Fortran driver.
!
! The reference driver (src_v2026_2_1/VANADIS.FOR:809-810) calls
!     CALL kernel_dbcg_simple(NON,FMV3,TNW2,TOL,IL_I,ITER,ERR,BB,
!    &                        ISS,DIAG,NAX,NAY,NAZ,bc_dirichlet)
! through an implicit interface; gfortran emits the symbol
! kernel_dbcg_simple_ with every argument by reference, which libvdr.so
! exports unchanged, so that call links as it is.  This module adds an
! explicit interface for it and for the handle API (include/vdr.h), which
! keeps mesh, fields and operator on the GPU across time steps.
!
! Arrays keep the driver's layouts: xx/yy/zz(N), iss(E,8) and kod(E,6)
! column-major with 1-based node ids, vel(E,3), lam/pdec/q(E),
! bc_dirichlet(N).  Handles are opaque type(c_ptr) values.
module vdr_iso_c
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: VDR_OK = 0, VDR_NOT_CONVERGED = 1, &
       VDR_BREAKDOWN = 2, VDR_CUDA_ERROR = 3, VDR_BAD_ARGUMENT = 4, &
       VDR_TIMEOUT = 5, VDR_IO_ERROR = 6
  integer(c_int), parameter :: VDR_DR_OT = 0, VDR_DR_GP = 1, VDR_DR_VF = 2
  integer(c_int), parameter :: VDR_SCATTER_AUTO = 0, VDR_SCATTER_ATOMIC = 1, &
       VDR_SCATTER_COLOR = 2, VDR_SCATTER_WARP = 3
  integer(c_int), parameter :: VDR_APPLY_AUTO = 0, VDR_APPLY_STORED = 1, &
       VDR_APPLY_MATRIX_FREE = 2
  integer(c_int), parameter :: VDR_SOLVER_BICGSTAB = 0, VDR_SOLVER_BICG = 1
  integer(c_int), parameter :: VDR_STORE_AUTO = 0, VDR_STORE_FP64 = 1, &
       VDR_STORE_DF = 2
  integer(c_int), parameter :: VDR_PRECISION_FP64 = 0, VDR_PRECISION_MIXED = 1
  integer(c_int), parameter :: VDR_BUILD_AUTO = 0, VDR_BUILD_RECOMPUTE = 1

  type, bind(c) :: vdr_options
     integer(c_int) :: dr_variant, scatter, apply_mode, solver
     integer(c_int) :: iters_per_graph, device, matrix_storage
     integer(c_int) :: precision
     integer(c_int) :: reserved(8)
  end type vdr_options

  interface
     subroutine kernel_dbcg_simple(n, b, x, tol, itmax, iter, err, bb, iss, &
          diag, nax, nay, naz, bc_dirichlet) bind(c, name="kernel_dbcg_simple_")
       import :: c_int, c_double
       integer(c_int), intent(in) :: n, itmax, nax, nay, naz
       real(c_double), intent(in) :: b(*), tol, bb(*), diag(*)
       real(c_double), intent(inout) :: x(*)
       integer(c_int), intent(out) :: iter
       real(c_double), intent(out) :: err
       integer(c_int), intent(in) :: iss(*), bc_dirichlet(*)
     end subroutine kernel_dbcg_simple

     integer(c_int) function vdr_default_options(opt) bind(c, name="vdr_default_options")
       import :: c_int, vdr_options
       type(vdr_options), intent(out) :: opt
     end function vdr_default_options

     integer(c_int) function vdr_create(h, nnode, nelem, xx, yy, zz, iss, kod, &
          opt) bind(c, name="vdr_create")
       import :: c_int, c_double, c_ptr, vdr_options
       type(c_ptr), intent(out) :: h
       integer(c_int), value :: nnode, nelem
       real(c_double), intent(in) :: xx(*), yy(*), zz(*)
       integer(c_int), intent(in) :: iss(*), kod(*)
       type(vdr_options), intent(in) :: opt
     end function vdr_create

     integer(c_int) function vdr_set_fields(h, vel, lam, pdec, q, robin_alpha) &
          bind(c, name="vdr_set_fields")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(in) :: vel(*), lam(*), pdec(*), q(*)
       real(c_double), value :: robin_alpha
     end function vdr_set_fields

     integer(c_int) function vdr_set_dirichlet(h, bc) bind(c, name="vdr_set_dirichlet")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), intent(in) :: bc(*)
     end function vdr_set_dirichlet

     integer(c_int) function vdr_set_operator(h, ah, am) bind(c, name="vdr_set_operator")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), value :: ah, am
     end function vdr_set_operator

     ! element geometry of the build: the mesh's geometric factors formed
     ! once (VDR_BUILD_AUTO) or the Jacobians at every build
     integer(c_int) function vdr_set_build_mode(h, mode) bind(c, name="vdr_set_build_mode")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: mode
     end function vdr_set_build_mode

     integer(c_int) function vdr_geometry_status(h, cached, bytes) &
          bind(c, name="vdr_geometry_status")
       import :: c_int, c_long_long, c_ptr
       type(c_ptr), value :: h
       integer(c_int), intent(out) :: cached
       integer(c_long_long), intent(out) :: bytes
     end function vdr_geometry_status

     integer(c_int) function vdr_apply(h, x, y, transpose) bind(c, name="vdr_apply")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(in) :: x(*)
       real(c_double), intent(out) :: y(*)
       integer(c_int), value :: transpose
     end function vdr_apply

     integer(c_int) function vdr_assemble_rhs(h, cf, rm, t_old, b) &
          bind(c, name="vdr_assemble_rhs")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), value :: cf, rm
       real(c_double), intent(in) :: t_old(*)
       real(c_double), intent(out) :: b(*)
     end function vdr_assemble_rhs

     integer(c_int) function vdr_get_diag(h, diag) bind(c, name="vdr_get_diag")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(out) :: diag(*)
     end function vdr_get_diag

     integer(c_int) function vdr_get_element_matrices(h, bb) &
          bind(c, name="vdr_get_element_matrices")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(out) :: bb(*)
     end function vdr_get_element_matrices

     integer(c_int) function vdr_solve(h, b, x, tol, itmax, iter, err) &
          bind(c, name="vdr_solve")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(in) :: b(*)
       real(c_double), intent(inout) :: x(*)
       real(c_double), value :: tol
       integer(c_int), value :: itmax
       integer(c_int), intent(out) :: iter
       real(c_double), intent(out) :: err
     end function vdr_solve

     integer(c_int) function vdr_mass(h, c, mass) bind(c, name="vdr_mass")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(in) :: c(*)
       real(c_double), intent(out) :: mass
     end function vdr_mass

     integer(c_int) function vdr_destroy(h) bind(c, name="vdr_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function vdr_destroy

     ! The step's T_sssss.TXT (scale 1d6 as the driver writes TNW2 * 1d6)
     ! and the X/Y/Z slice files; dir is a NUL-terminated path, e.g.
     ! 'output'//c_null_char.
     integer(c_int) function vdr_write_result_txt(dir, step, nnode, xx, yy, &
          zz, t, scale) bind(c, name="vdr_write_result_txt")
       import :: c_int, c_long, c_double, c_char
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: step
       integer(c_long), value :: nnode
       real(c_double), intent(in) :: xx(*), yy(*), zz(*), t(*)
       real(c_double), value :: scale
     end function vdr_write_result_txt

     integer(c_int) function vdr_write_slices_txt(dir, step, nax, nay, naz, &
          xx, yy, zz, t, scale) bind(c, name="vdr_write_slices_txt")
       import :: c_int, c_double, c_char
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: step, nax, nay, naz
       real(c_double), intent(in) :: xx(*), yy(*), zz(*), t(*)
       real(c_double), value :: scale
     end function vdr_write_slices_txt
  end interface
end module vdr_iso_c
