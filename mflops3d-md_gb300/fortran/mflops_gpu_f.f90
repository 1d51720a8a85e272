! mflops_gpu_f -- ISO_C_BINDING front end of libmflops_gb300 for Fortran callers.
!
! Mirrors the module procedures of the reference so that a caller can swap
!   use class_derivatives   -> use mflops_gpu_f
!   use class_solver_3d     -> use mflops_gpu_f
! keeping names, argument orders and meanings:
!   der_coeffs_init(grid,dc,n,solve,so)          class_derivatives.f90:111
!   der(dc,x,dx), dder, der_s, dder_s            class_derivatives.f90:186-260
!   dertype(dc)                                  class_derivatives.f90:96
!   solver_coeffs_init_3d(g1,g2,g3,sc,n1,n2,n3,bct,so)   class_solver_3d.f90:380
!   solve_3d(sc,rhs,sigma,solf,bcx,bcy,bcz,n1,n2,n3)     class_solver_3d.f90:83
! and adds array-level forms of the class_field pencil drivers
! (derx..dderz, class_field.f90:629-978) and of solver_3d (:1072), and the
! one-domain Navier-Stokes time step of navier3d.f90:48-261
! (navier_defaults, navier_initialization_gpu, navier_set_field,
! navier_get_field, navier_step, navier_destroy).
!
! Arrays are passed by address; host arrays are staged by the library and
! the call returns when the result is in host memory.  Errors stop the
! program with the library's message, as the reference stops on its own
! failures (e.g. complex eigenvalues, class_solver_3d.f90:537-540).
!
! This file is shipped as source; build it with any Fortran 2003 compiler and
! link against libmflops_gb300.so.
module mflops_gpu_f
  use iso_c_binding
  implicit none
  private

  integer, parameter :: rk = c_double

  type, public :: derivatives_coefficients
     type(c_ptr) :: h = c_null_ptr
     integer :: n = 0
  end type derivatives_coefficients

  type, public :: solver_coeffs_3d
     type(c_ptr) :: h = c_null_ptr
     integer :: n1 = 0, n2 = 0, n3 = 0
  end type solver_coeffs_3d

  integer(c_int), parameter, public :: MF_PREC_FP64 = 0, MF_PREC_SPLIT_BF16 = 1, MF_PREC_3XTF32 = 2

  ! mf_navier_params_t (field order and types as in the C header)
  type, bind(C), public :: navier_params
     real(c_double) :: ts, reynolds
     integer(c_int) :: nlt, pt, tou, top, so_solver, so_der, flow_rate, nmodes, precision, refine
     integer(c_int) :: les_type
     real(c_double) :: les_c
     integer(c_int) :: nsubite
     type(c_ptr) :: md_cache_dir
     integer(c_int) :: md_interface
  end type navier_params

  type, public :: navier3d_gpu
     type(c_ptr) :: h = c_null_ptr
     integer :: nx = 0, ny = 0, nz = 0
  end type navier3d_gpu

  public :: der_coeffs_init, der, dder, der_s, dder_s, dertype, der_destroy
  public :: derx, dery, derz, dderx, ddery, dderz
  public :: solver_coeffs_init_3d, solve_3d, solve_3d_mixed, solver_3d, solver_destroy
  public :: navier_defaults, navier_initialization_gpu, navier_set_field, navier_get_field
  public :: navier_step, navier_destroy
  public :: les_network_init, les_network_destroy, navier_set_les_network
  integer(c_int), parameter, public :: MF_LES_LEARNED = 4

  ! learned LES coefficient network (les_type 4): parameters and scaling
  ! come from training (mflops_gb300.learn) and are loaded here
  type, public :: les_network
     type(c_ptr) :: h = c_null_ptr
  end type les_network
  public :: mesh_grid_init
  integer(c_int), parameter, public :: MF_GRID_UNIFORM = 0, MF_GRID_ARCSIN = 1, MF_GRID_TANH = 2

  interface
     function c_last_error() bind(C, name="mf_last_error") result(p)
       import :: c_ptr
       type(c_ptr) :: p
     end function c_last_error

     function c_der_coeffs_init(grid, n, solver_type, so, dc) bind(C, name="mf_der_coeffs_init") result(rc)
       import :: c_double, c_int, c_ptr
       real(c_double), intent(in) :: grid(*)
       integer(c_int), value :: n, solver_type, so
       type(c_ptr), intent(out) :: dc
       integer(c_int) :: rc
     end function c_der_coeffs_init

     function c_der_destroy(dc) bind(C, name="mf_der_destroy") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: dc
       integer(c_int) :: rc
     end function c_der_destroy

     function c_der_apply(dc, axis, order, f, df, nx, ny, nz, stream) bind(C, name="mf_der_apply") result(rc)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dc
       integer(c_int), value :: axis, order, nx, ny, nz
       real(c_double), intent(in) :: f(*)
       real(c_double), intent(inout) :: df(*)
       type(c_ptr), value :: stream
       integer(c_int) :: rc
     end function c_der_apply

     function c_der_lines(dc, order, variant, x, dx, count, stream) bind(C, name="mf_der_lines") result(rc)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dc
       integer(c_int), value :: order, variant, count
       real(c_double), intent(in) :: x(*)
       real(c_double), intent(inout) :: dx(*)
       type(c_ptr), value :: stream
       integer(c_int) :: rc
     end function c_der_lines

     function c_dertype(dc, st) bind(C, name="mf_dertype") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: dc
       integer(c_int), intent(out) :: st
       integer(c_int) :: rc
     end function c_dertype

     function c_solver_init(g1, g2, g3, n1, n2, n3, bct, so, sc) &
          bind(C, name="mf_solver_coeffs_init_3d") result(rc)
       import :: c_double, c_int, c_ptr
       real(c_double), intent(in) :: g1(*), g2(*), g3(*)
       integer(c_int), value :: n1, n2, n3, so
       integer(c_int), intent(in) :: bct(6)
       type(c_ptr), intent(out) :: sc
       integer(c_int) :: rc
     end function c_solver_init

     function c_solver_destroy(sc) bind(C, name="mf_solver3d_destroy") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: sc
       integer(c_int) :: rc
     end function c_solver_destroy

     function c_solve_3d(sc, rhs, sigma, solf, bcx, bcy, bcz, n1, n2, n3, stream) &
          bind(C, name="mf_solve_3d") result(rc)
       import :: c_double, c_int, c_ptr
       type(c_ptr), value :: sc
       real(c_double), intent(in) :: rhs(*), bcx(*), bcy(*), bcz(*)
       real(c_double), value :: sigma
       real(c_double), intent(inout) :: solf(*)
       integer(c_int), value :: n1, n2, n3
       type(c_ptr), value :: stream
       integer(c_int) :: rc
     end function c_solve_3d

     function c_solve_3d_mixed(sc, rhs, sigma, solf, bcx, bcy, bcz, n1, n2, n3, prec, refine, stream) &
          bind(C, name="mf_solve_3d_mixed") result(rc)
       import :: c_double, c_int, c_ptr
       type(c_ptr), value :: sc
       real(c_double), intent(in) :: rhs(*), bcx(*), bcy(*), bcz(*)
       real(c_double), value :: sigma
       real(c_double), intent(inout) :: solf(*)
       integer(c_int), value :: n1, n2, n3, prec, refine
       type(c_ptr), value :: stream
       integer(c_int) :: rc
     end function c_solve_3d_mixed

     function c_solver_3d(sc, g, u, bcx, bcy, bcz, nx, ny, nz, sigma, prec, stream) &
          bind(C, name="mf_solver_3d") result(rc)
       import :: c_double, c_int, c_ptr
       type(c_ptr), value :: sc
       real(c_double), intent(in) :: g(*), bcx(*), bcy(*), bcz(*)
       real(c_double), intent(inout) :: u(*)
       integer(c_int), value :: nx, ny, nz, prec
       real(c_double), value :: sigma
       type(c_ptr), value :: stream
       integer(c_int) :: rc
     end function c_solver_3d

     function c_navier_defaults(p) bind(C, name="mf_navier_defaults") result(rc)
       import :: c_int, navier_params
       type(navier_params), intent(out) :: p
       integer(c_int) :: rc
     end function c_navier_defaults

     function c_navier_create(gx, nx, gy, ny, gz, nz, p, nav) bind(C, name="mf_navier_create") result(rc)
       import :: c_double, c_int, c_ptr, navier_params
       real(c_double), intent(in) :: gx(*), gy(*), gz(*)
       integer(c_int), value :: nx, ny, nz
       type(navier_params), intent(in) :: p
       type(c_ptr), intent(out) :: nav
       integer(c_int) :: rc
     end function c_navier_create

     function c_navier_destroy(nav) bind(C, name="mf_navier_destroy") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: nav
       integer(c_int) :: rc
     end function c_navier_destroy

     function c_navier_set_field(nav, var, level, f, stream) bind(C, name="mf_navier_set_field") result(rc)
       import :: c_double, c_int, c_ptr
       type(c_ptr), value :: nav, stream
       integer(c_int), value :: var, level
       real(c_double), intent(in) :: f(*)
       integer(c_int) :: rc
     end function c_navier_set_field

     function c_navier_get_field(nav, var, level, f, stream) bind(C, name="mf_navier_get_field") result(rc)
       import :: c_double, c_int, c_ptr
       type(c_ptr), value :: nav, stream
       integer(c_int), value :: var, level
       real(c_double), intent(out) :: f(*)
       integer(c_int) :: rc
     end function c_navier_get_field

     function c_navier_step(nav, diag, stream) bind(C, name="mf_navier_step") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: nav, diag, stream
       integer(c_int) :: rc
     end function c_navier_step

     function c_mlp_create(seed, mlp) bind(C, name="mf_mlp_create") result(rc)
       import :: c_int, c_long_long, c_ptr
       integer(c_long_long), value :: seed
       type(c_ptr), intent(out) :: mlp
       integer(c_int) :: rc
     end function c_mlp_create

     function c_mlp_destroy(mlp) bind(C, name="mf_mlp_destroy") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: mlp
       integer(c_int) :: rc
     end function c_mlp_destroy

     function c_mlp_set_params(mlp, params) bind(C, name="mf_mlp_set_params") result(rc)
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: mlp
       real(c_float), intent(in) :: params(*)
       integer(c_int) :: rc
     end function c_mlp_set_params

     function c_mlp_set_scaling(mlp, mean, istd, lo, hi, cscale, loss_scale) &
          bind(C, name="mf_mlp_set_scaling") result(rc)
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: mlp
       real(c_float), intent(in) :: mean(*), istd(*), lo(*), hi(*)
       real(c_float), value :: cscale, loss_scale
       integer(c_int) :: rc
     end function c_mlp_set_scaling

     function c_navier_set_les_network(nav, mlp) bind(C, name="mf_navier_set_les_network") result(rc)
       import :: c_int, c_ptr
       type(c_ptr), value :: nav, mlp
       integer(c_int) :: rc
     end function c_navier_set_les_network

     function c_mesh_grid_init(choice, n, dom_coord, ndomains, kind, param, grid1d, dgrid1d) &
          bind(C, name="mf_mesh_grid_init") result(rc)
       import :: c_char, c_int, c_double
       character(kind=c_char), value :: choice
       integer(c_int), value :: n, dom_coord, ndomains, kind
       real(c_double), value :: param
       real(c_double), intent(out) :: grid1d(*), dgrid1d(*)
       integer(c_int) :: rc
     end function c_mesh_grid_init
  end interface

contains

  subroutine check(rc, where)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    character(len=512) :: text
    integer :: i
    if (rc == 0) return
    call c_f_pointer(c_last_error(), msg, [512])
    text = ' '
    do i = 1, 512
       if (msg(i) == c_null_char) exit
       text(i:i) = msg(i)
    enddo
    print '(a,a,a)', where, ': ', trim(text)
    stop
  end subroutine check

  ! ------------------------------------------------- learned LES coefficient
  ! A network of the learned eddy-viscosity coefficient: params(4673) and the
  ! six-feature scaling as written by the training (mflops_gb300.learn).
  subroutine les_network_init(net, params, mean, istd, lo, hi, cscale)
    type(les_network), intent(out) :: net
    real(c_float), intent(in) :: params(4673), mean(6), istd(6), lo(6), hi(6)
    real(c_float), intent(in) :: cscale
    call check(c_mlp_create(0_c_long_long, net%h), 'les_network_init')
    call check(c_mlp_set_params(net%h, params), 'les_network_init')
    call check(c_mlp_set_scaling(net%h, mean, istd, lo, hi, cscale, 1.0_c_float), 'les_network_init')
  end subroutine les_network_init

  subroutine les_network_destroy(net)
    type(les_network), intent(inout) :: net
    if (c_associated(net%h)) call check(c_mlp_destroy(net%h), 'les_network_destroy')
    net%h = c_null_ptr
  end subroutine les_network_destroy

  ! les_type 4: the step's eddy viscosity from the network (Smagorinsky with
  ! les_c**2 outside its training range); net must outlive the steps.
  subroutine navier_set_les_network(nav, net)
    type(navier3d_gpu), intent(in) :: nav
    type(les_network), intent(in) :: net
    call check(c_navier_set_les_network(nav%h, net%h), 'navier_set_les_network')
  end subroutine navier_set_les_network

  ! ---------------------------------------------------------------- grids
  ! mesh_grid_init (class_mesh.f90:113-339) on plain arrays: grid1d(n) and
  ! dgrid1d(n) of direction choice ('x', 'y' or 'z') for subdomain dom_coord
  ! (0-based) of ndomains along it.  Default: the reference's arcsin grid
  ! (beta = 33.3); kind/param select MF_GRID_UNIFORM or MF_GRID_TANH.
  subroutine mesh_grid_init(grid1d, dgrid1d, choice, n, dom_coord, ndomains, kind, param)
    integer, intent(in) :: n
    real(rk), intent(out) :: grid1d(n), dgrid1d(n)
    character(len=1), intent(in) :: choice
    integer, intent(in), optional :: dom_coord, ndomains, kind
    real(rk), intent(in), optional :: param
    integer(c_int) :: c, nd, k
    real(c_double) :: p
    c = 0; nd = 1; k = MF_GRID_ARCSIN; p = 33.3_rk
    if (present(dom_coord)) c = int(dom_coord, c_int)
    if (present(ndomains)) nd = int(ndomains, c_int)
    if (present(kind)) k = int(kind, c_int)
    if (present(param)) p = param
    call check(c_mesh_grid_init(choice, int(n, c_int), c, nd, k, p, grid1d, dgrid1d), 'mesh_grid_init')
  end subroutine mesh_grid_init

  ! ---------------------------------------------------------------- derivatives
  subroutine der_coeffs_init(grid, dc, n, solve, so)
    type(derivatives_coefficients), intent(out) :: dc
    integer, intent(in) :: n, so
    real(rk), intent(in) :: grid(n)
    logical :: solve
    integer(c_int) :: st
    st = 0
    if (solve) st = 1
    call check(c_der_coeffs_init(grid, int(n, c_int), st, int(so, c_int), dc%h), 'der_coeffs_init')
    dc%n = n
  end subroutine der_coeffs_init

  subroutine der_destroy(dc)
    type(derivatives_coefficients), intent(inout) :: dc
    call check(c_der_destroy(dc%h), 'der_destroy')
    dc%h = c_null_ptr
  end subroutine der_destroy

  function dertype(dc)
    type(derivatives_coefficients), intent(in) :: dc
    logical :: dertype
    integer(c_int) :: st
    call check(c_dertype(dc%h, st), 'dertype')
    dertype = (st /= 0)
  end function dertype

  subroutine der(dc, x, dx)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: x(:)
    real(rk), intent(out) :: dx(:)
    call check(c_der_lines(dc%h, 1_c_int, 0_c_int, x, dx, 1_c_int, c_null_ptr), 'der')
  end subroutine der

  subroutine dder(dc, x, ddx)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: x(:)
    real(rk), intent(out) :: ddx(:)
    call check(c_der_lines(dc%h, 2_c_int, 0_c_int, x, ddx, 1_c_int, c_null_ptr), 'dder')
  end subroutine dder

  subroutine der_s(dc, x, dx)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: x(:)
    real(rk), intent(out) :: dx(:)
    call check(c_der_lines(dc%h, 1_c_int, 1_c_int, x, dx, 1_c_int, c_null_ptr), 'der_s')
  end subroutine der_s

  subroutine dder_s(dc, x, ddx)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: x(:)
    real(rk), intent(out) :: ddx(:)
    call check(c_der_lines(dc%h, 2_c_int, 1_c_int, x, ddx, 1_c_int, c_null_ptr), 'dder_s')
  end subroutine dder_s

  ! Array forms of the class_field pencil drivers: df = d^order f / dx_axis^order.
  subroutine apply(dc, axis, order, f, df, what)
    type(derivatives_coefficients), intent(in) :: dc
    integer, intent(in) :: axis, order
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    character(*), intent(in) :: what
    call check(c_der_apply(dc%h, int(axis, c_int), int(order, c_int), f, df, &
         int(size(f,1), c_int), int(size(f,2), c_int), int(size(f,3), c_int), c_null_ptr), what)
  end subroutine apply

  subroutine derx(dc, f, df)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    call apply(dc, 0, 1, f, df, 'derx')
  end subroutine derx

  subroutine dery(dc, f, df)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    call apply(dc, 1, 1, f, df, 'dery')
  end subroutine dery

  subroutine derz(dc, f, df)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    call apply(dc, 2, 1, f, df, 'derz')
  end subroutine derz

  subroutine dderx(dc, f, df)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    call apply(dc, 0, 2, f, df, 'dderx')
  end subroutine dderx

  subroutine ddery(dc, f, df)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    call apply(dc, 1, 2, f, df, 'ddery')
  end subroutine ddery

  subroutine dderz(dc, f, df)
    type(derivatives_coefficients), intent(in) :: dc
    real(rk), intent(in) :: f(:,:,:)
    real(rk), intent(out) :: df(:,:,:)
    call apply(dc, 2, 2, f, df, 'dderz')
  end subroutine dderz

  ! --------------------------------------------------------------------- solver
  subroutine solver_coeffs_init_3d(grid1, grid2, grid3, sc, n1, n2, n3, bct, so)
    type(solver_coeffs_3d), intent(out) :: sc
    integer, intent(in) :: n1, n2, n3, so
    real(rk), intent(in) :: grid1(n1), grid2(n2), grid3(n3)
    integer, intent(in) :: bct(6)
    integer(c_int) :: b(6)
    b = int(bct, c_int)
    call check(c_solver_init(grid1, grid2, grid3, int(n1, c_int), int(n2, c_int), int(n3, c_int), &
         b, int(so, c_int), sc%h), 'solver_coeffs_init_3d')
    sc%n1 = n1 - 2 ; sc%n2 = n2 - 2 ; sc%n3 = n3 - 2
  end subroutine solver_coeffs_init_3d

  subroutine solver_destroy(sc)
    type(solver_coeffs_3d), intent(inout) :: sc
    call check(c_solver_destroy(sc%h), 'solver_destroy')
    sc%h = c_null_ptr
  end subroutine solver_destroy

  subroutine solve_3d(sc, rhs, sigma, solf, bcx, bcy, bcz, n1, n2, n3)
    type(solver_coeffs_3d), intent(in) :: sc
    integer, intent(in) :: n1, n2, n3
    real(rk), intent(inout) :: rhs(n1,n2,n3)
    real(rk), intent(inout) :: solf(0:n1+1,0:n2+1,0:n3+1)
    real(rk), intent(in) :: bcx(n2,n3,2), bcy(n1,n3,2), bcz(n1,n2,2)
    real(rk), intent(in) :: sigma
    call check(c_solve_3d(sc%h, rhs, sigma, solf, bcx, bcy, bcz, int(n1, c_int), int(n2, c_int), &
         int(n3, c_int), c_null_ptr), 'solve_3d')
  end subroutine solve_3d

  subroutine solve_3d_mixed(sc, rhs, sigma, solf, bcx, bcy, bcz, n1, n2, n3, refine)
    type(solver_coeffs_3d), intent(in) :: sc
    integer, intent(in) :: n1, n2, n3, refine
    real(rk), intent(in) :: rhs(n1,n2,n3)
    real(rk), intent(inout) :: solf(0:n1+1,0:n2+1,0:n3+1)
    real(rk), intent(in) :: bcx(n2,n3,2), bcy(n1,n3,2), bcz(n1,n2,2)
    real(rk), intent(in) :: sigma
    call check(c_solve_3d_mixed(sc%h, rhs, sigma, solf, bcx, bcy, bcz, int(n1, c_int), int(n2, c_int), &
         int(n3, c_int), MF_PREC_SPLIT_BF16, int(refine, c_int), c_null_ptr), 'solve_3d_mixed')
  end subroutine solve_3d_mixed

  ! Array form of class_field::solver_3d(sc,g,u,bc,sigma): g, u are (nx,ny,nz).
  subroutine solver_3d(sc, g, u, bcx, bcy, bcz, sigma)
    type(solver_coeffs_3d), intent(in) :: sc
    real(rk), intent(in) :: g(:,:,:)
    real(rk), intent(inout) :: u(:,:,:)
    real(rk), intent(in) :: bcx(:,:,:), bcy(:,:,:), bcz(:,:,:)
    real(rk), intent(in) :: sigma
    call check(c_solver_3d(sc%h, g, u, bcx, bcy, bcz, int(size(u,1), c_int), int(size(u,2), c_int), &
         int(size(u,3), c_int), sigma, MF_PREC_FP64, c_null_ptr), 'solver_3d')
  end subroutine solver_3d

  ! ------------------------------------------------------- Navier-Stokes step
  ! The reference's defaults (command_line.f90:14-35) in p.
  subroutine navier_defaults(p)
    type(navier_params), intent(out) :: p
    call check(c_navier_defaults(p), 'navier_defaults')
  end subroutine navier_defaults

  ! navier_initialization for one domain (class_navier_3D.f90:2084-2345).
  subroutine navier_initialization_gpu(gx, gy, gz, nav, p)
    real(rk), intent(in) :: gx(:), gy(:), gz(:)
    type(navier3d_gpu), intent(out) :: nav
    type(navier_params), intent(in) :: p
    call check(c_navier_create(gx, int(size(gx), c_int), gy, int(size(gy), c_int), gz, int(size(gz), c_int), &
         p, nav%h), 'navier_initialization_gpu')
    nav%nx = size(gx)
    nav%ny = size(gy)
    nav%nz = size(gz)
  end subroutine navier_initialization_gpu

  ! var 0..4 = u, v, w, p, phi; level 0 = it(1) ... 3 = it(nt).
  subroutine navier_set_field(nav, var, level, f)
    type(navier3d_gpu), intent(in) :: nav
    integer, intent(in) :: var, level
    real(rk), intent(in) :: f(:,:,:)
    call check(c_navier_set_field(nav%h, int(var, c_int), int(level, c_int), f, c_null_ptr), 'navier_set_field')
  end subroutine navier_set_field

  subroutine navier_get_field(nav, var, level, f)
    type(navier3d_gpu), intent(in) :: nav
    integer, intent(in) :: var, level
    real(rk), intent(out) :: f(:,:,:)
    call check(c_navier_get_field(nav%h, int(var, c_int), int(level, c_int), f, c_null_ptr), 'navier_get_field')
  end subroutine navier_get_field

  ! One iteration of the time loop (navier3d.f90:48-261); diag receives the
  ! driver's printed numbers (div V, V and P errors, kinetic energy,
  ! stationarity).
  subroutine navier_step(nav, diag)
    type(navier3d_gpu), intent(in) :: nav
    real(rk), intent(out), target, optional :: diag(12)
    if (present(diag)) then
       call check(c_navier_step(nav%h, c_loc(diag), c_null_ptr), 'navier_step')
    else
       call check(c_navier_step(nav%h, c_null_ptr, c_null_ptr), 'navier_step')
    endif
  end subroutine navier_step

  subroutine navier_destroy(nav)
    type(navier3d_gpu), intent(inout) :: nav
    call check(c_navier_destroy(nav%h), 'navier_destroy')
    nav%h = c_null_ptr
  end subroutine navier_destroy

end module mflops_gpu_f
