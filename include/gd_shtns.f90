! gd_shtns.f90 -- module shtns on the GB300 library: a replacement for the
! reference's src/shtns.f90 with the same module name, the same public
! routines and module data, and the same argument meanings, so that
! dyn_run.f90-style callers (`use shtns`) link unchanged against it instead of
! SHTns/FFTW.  Build it after kinds.f90 and gd_api.f90 and link
! libgdcore.so.
!
!   shtns_init(nlon, nlat, ntrunc[, nthreads, polar_opt])   shtns.f90:90-156
!   shtns_destroy()                                         shtns.f90:158-169
!   grdtospec(datagrid, dataspec)                           shtns.f90:171-201
!   spectogrd(dataspec, datagrid)                           shtns.f90:203-231
!   getuv(vrtspec, divspec, ugrid, vgrid, rsphere)          shtns.f90:233-273
!   getvrtdivspec(ugrid, vgrid, vrtspec, divspec, rsphere)  shtns.f90:275-311
!   getgrad(dataspec, ugrid, vgrid, rsphere)                shtns.f90:313-352
!   module data: nlm, current_nlon, current_nlat, current_ntrunc, lats, lons,
!   gauwts, areawts, degree, order, lap, invlap             shtns.f90:58-60, 77-85
!
! Each routine is generic over the two kinds the reference builds with
! (r_kind = 4, the default, and 8; src/kinds.f90:100): single-precision
! arrays go to the library's gd_*_f entry points, which copy them as they are
! and convert on the device; the transforms themselves run in FP64 on the GPU,
! as SHTns computes in double whatever r_kind is.
!
! Differences from the reference, by design:
!  - nthreads and polar_opt are accepted and ignored: the transforms run on
!    the GPU, with exact Gauss quadrature and no polar threshold (the
!    reference's default polar_opt = 1e-10 perturbs SHTns at ~1e-10);
!  - the library's transforms take the sphere radius 6.3712e6 m (physcons
!    rerth); another rsphere is applied here by the scaling the reference's
!    prescale / postscale implies (u, v ~ rsphere; vrt, div, grad ~ 1/rsphere);
!  - one library context serves the module; calls from concurrent OpenMP
!    threads (dyn_run.f90:101) are serialised by a named critical section.
!    Callers that can should pass all levels at once to gd_spectogrd and
!    friends (module gd_api, nb = nlevs), which is the fast path;
!  - errors print the library's message and stop, as the reference does.
!
! Not compiled on the build machine or the GPU host: neither has a Fortran
! compiler.
module shtns
  use iso_c_binding
  use kinds, only: r_kind, r_double
  use gd_api
  implicit none
  private
  public :: shtns_init, grdtospec, spectogrd, getuv, getvrtdivspec, getgrad, shtns_destroy
  public :: gauwts, lats, lons, nlm, degree, order, lap, invlap, &
            current_nlon, current_nlat, current_ntrunc, areawts

  integer, save :: current_nlon = -1
  integer, save :: current_nlat = -1
  integer, save :: current_ntrunc = -1
  integer :: nlm
  real(r_kind), dimension(:), allocatable :: lap, invlap, gauwts
  real(r_kind), dimension(:,:), allocatable :: lats, lons, areawts
  integer, dimension(:), allocatable :: degree, order

  type(c_ptr), save :: ctx = c_null_ptr
  real(c_double), parameter :: rsphere_lib = 6.3712d6

  interface grdtospec
    module procedure grdtospec_r4, grdtospec_r8
  end interface
  interface spectogrd
    module procedure spectogrd_r4, spectogrd_r8
  end interface
  interface getuv
    module procedure getuv_r4, getuv_r8
  end interface
  interface getvrtdivspec
    module procedure getvrtdivspec_r4, getvrtdivspec_r8
  end interface
  interface getgrad
    module procedure getgrad_r4, getgrad_r8
  end interface

contains

  subroutine check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == GD_OK) return
    call c_f_pointer(gd_last_error(ctx), msg, [4096])
    n = 0
    do while (n < 4096)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    print *, 'shtns (GB300 library): ', what, ' failed, status ', rc, ': ', msg(1:n)
    stop
  end subroutine check

  subroutine shtns_init(nlon, nlat, ntrunc, nthreads, polar_opt)
    integer, intent(in) :: nlon, nlat, ntrunc
    integer, intent(in), optional :: nthreads
    real(r_double), intent(in), optional :: polar_opt
    type(gd_config) :: cfg
    real(c_double) :: ak(4), bk(4), pi
    real(c_double), allocatable :: lats1(:), gw(:), aw(:), lp(:), ilp(:)
    integer(c_int), allocatable :: deg(:), ord(:)
    integer :: i, j
    call shtns_destroy()
    ! a transform-only context: three sigma levels, no physics
    call check(gd_default_config(cfg), 'gd_default_config')
    cfg%ntrunc = ntrunc
    cfg%nlon = nlon
    cfg%nlat = nlat
    cfg%nlev = 3
    cfg%ntrac = 0
    cfg%precision = GD_PREC_FP64
    cfg%adiabatic = 1
    cfg%heldsuarez = 0
    ak = 0.0d0
    bk = [0.0d0, 1.0d0 / 3.0d0, 2.0d0 / 3.0d0, 1.0d0]
    call check(gd_init(cfg, ak, bk, ctx), 'gd_init')
    nlm = (ntrunc + 1) * (ntrunc + 2) / 2
    current_nlon = nlon
    current_nlat = nlat
    current_ntrunc = ntrunc
    allocate(lats1(nlat), gw(nlat), aw(nlat), lp(nlm), ilp(nlm), deg(nlm), ord(nlm))
    call check(gd_grid_info(ctx, lats1, gw, aw, deg, ord, lp, ilp), 'gd_grid_info')
    allocate(lats(nlon, nlat), lons(nlon, nlat), areawts(nlon, nlat), gauwts(nlat))
    allocate(degree(nlm), order(nlm), lap(nlm), invlap(nlm))
    pi = 4.0d0 * atan(1.0d0)
    do j = 1, nlat
      gauwts(j) = real(gw(j), r_kind)
      do i = 1, nlon
        lats(i, j) = real(lats1(j), r_kind)
        lons(i, j) = real(2.0d0 * pi * real(i - 1, c_double) / nlon, r_kind)
        areawts(i, j) = real(aw(j), r_kind)     ! gauwts / sum over the grid: sums to 1
      end do
    end do
    degree = deg
    order = ord
    lap = real(lp, r_kind)
    invlap = real(ilp, r_kind)
    deallocate(lats1, gw, aw, lp, ilp, deg, ord)
  end subroutine shtns_init

  subroutine shtns_destroy()
    integer(c_int) :: rc
    if (c_associated(ctx)) then
      rc = gd_finalize(ctx)
      ctx = c_null_ptr
    end if
    if (allocated(lats)) deallocate(lats)
    if (allocated(lons)) deallocate(lons)
    if (allocated(areawts)) deallocate(areawts)
    if (allocated(gauwts)) deallocate(gauwts)
    if (allocated(degree)) deallocate(degree)
    if (allocated(order)) deallocate(order)
    if (allocated(lap)) deallocate(lap)
    if (allocated(invlap)) deallocate(invlap)
  end subroutine shtns_destroy

  ! ---------------------------------------------------- single precision --
  subroutine grdtospec_r4(datagrid, dataspec)
    real(c_float), dimension(:,:), intent(in) :: datagrid
    complex(c_float_complex), dimension(:), intent(out) :: dataspec
    real(c_float) :: g(size(datagrid, 1), size(datagrid, 2))
    complex(c_float_complex) :: s(nlm)
    integer(c_int) :: rc
    g = datagrid
    !$omp critical (gd_shtns)
    rc = gd_grdtospec_f(ctx, 1_c_int, g, s)
    !$omp end critical (gd_shtns)
    call check(rc, 'grdtospec')
    dataspec = s
  end subroutine grdtospec_r4

  subroutine spectogrd_r4(dataspec, datagrid)
    complex(c_float_complex), dimension(:), intent(in) :: dataspec
    real(c_float), dimension(:,:), intent(out) :: datagrid
    real(c_float) :: g(size(datagrid, 1), size(datagrid, 2))
    complex(c_float_complex) :: s(nlm)
    integer(c_int) :: rc
    s = dataspec
    !$omp critical (gd_shtns)
    rc = gd_spectogrd_f(ctx, 1_c_int, s, g)
    !$omp end critical (gd_shtns)
    call check(rc, 'spectogrd')
    datagrid = g
  end subroutine spectogrd_r4

  subroutine getuv_r4(vrtspec, divspec, ugrid, vgrid, rsphere)
    complex(c_float_complex), dimension(:), intent(in) :: vrtspec, divspec
    real(c_float), dimension(:,:), intent(out) :: ugrid, vgrid
    real(c_float), intent(in) :: rsphere
    real(c_float) :: u(size(ugrid, 1), size(ugrid, 2)), v(size(vgrid, 1), size(vgrid, 2))
    complex(c_float_complex) :: a(nlm), b(nlm)
    integer(c_int) :: rc
    a = vrtspec
    b = divspec
    !$omp critical (gd_shtns)
    rc = gd_getuv_f(ctx, 1_c_int, a, b, u, v)
    !$omp end critical (gd_shtns)
    call check(rc, 'getuv')
    ugrid = u * real(rsphere / rsphere_lib, c_float)
    vgrid = v * real(rsphere / rsphere_lib, c_float)
  end subroutine getuv_r4

  subroutine getvrtdivspec_r4(ugrid, vgrid, vrtspec, divspec, rsphere)
    real(c_float), dimension(:,:), intent(in) :: ugrid, vgrid
    complex(c_float_complex), dimension(:), intent(out) :: vrtspec, divspec
    real(c_float), intent(in) :: rsphere
    real(c_float) :: u(size(ugrid, 1), size(ugrid, 2)), v(size(vgrid, 1), size(vgrid, 2))
    complex(c_float_complex) :: a(nlm), b(nlm)
    integer(c_int) :: rc
    u = ugrid
    v = vgrid
    !$omp critical (gd_shtns)
    rc = gd_getvrtdivspec_f(ctx, 1_c_int, u, v, a, b)
    !$omp end critical (gd_shtns)
    call check(rc, 'getvrtdivspec')
    vrtspec = a * real(rsphere_lib / rsphere, c_float)
    divspec = b * real(rsphere_lib / rsphere, c_float)
  end subroutine getvrtdivspec_r4

  subroutine getgrad_r4(dataspec, ugrid, vgrid, rsphere)
    complex(c_float_complex), dimension(:), intent(in) :: dataspec
    real(c_float), dimension(:,:), intent(out) :: ugrid, vgrid
    real(c_float), intent(in) :: rsphere
    real(c_float) :: gx(size(ugrid, 1), size(ugrid, 2)), gy(size(vgrid, 1), size(vgrid, 2))
    complex(c_float_complex) :: s(nlm)
    integer(c_int) :: rc
    s = dataspec
    !$omp critical (gd_shtns)
    rc = gd_getgrad_f(ctx, 1_c_int, s, gx, gy)
    !$omp end critical (gd_shtns)
    call check(rc, 'getgrad')
    ugrid = gx * real(rsphere_lib / rsphere, c_float)
    vgrid = gy * real(rsphere_lib / rsphere, c_float)
  end subroutine getgrad_r4

  ! ---------------------------------------------------- double precision --
  subroutine grdtospec_r8(datagrid, dataspec)
    real(c_double), dimension(:,:), intent(in) :: datagrid
    complex(c_double_complex), dimension(:), intent(out) :: dataspec
    real(c_double) :: g(size(datagrid, 1), size(datagrid, 2))
    complex(c_double_complex) :: s(nlm)
    integer(c_int) :: rc
    g = datagrid
    !$omp critical (gd_shtns)
    rc = gd_grdtospec(ctx, 1_c_int, g, s)
    !$omp end critical (gd_shtns)
    call check(rc, 'grdtospec')
    dataspec = s
  end subroutine grdtospec_r8

  subroutine spectogrd_r8(dataspec, datagrid)
    complex(c_double_complex), dimension(:), intent(in) :: dataspec
    real(c_double), dimension(:,:), intent(out) :: datagrid
    real(c_double) :: g(size(datagrid, 1), size(datagrid, 2))
    complex(c_double_complex) :: s(nlm)
    integer(c_int) :: rc
    s = dataspec
    !$omp critical (gd_shtns)
    rc = gd_spectogrd(ctx, 1_c_int, s, g)
    !$omp end critical (gd_shtns)
    call check(rc, 'spectogrd')
    datagrid = g
  end subroutine spectogrd_r8

  subroutine getuv_r8(vrtspec, divspec, ugrid, vgrid, rsphere)
    complex(c_double_complex), dimension(:), intent(in) :: vrtspec, divspec
    real(c_double), dimension(:,:), intent(out) :: ugrid, vgrid
    real(c_double), intent(in) :: rsphere
    real(c_double) :: u(size(ugrid, 1), size(ugrid, 2)), v(size(vgrid, 1), size(vgrid, 2))
    complex(c_double_complex) :: a(nlm), b(nlm)
    integer(c_int) :: rc
    a = vrtspec
    b = divspec
    !$omp critical (gd_shtns)
    rc = gd_getuv(ctx, 1_c_int, a, b, u, v)
    !$omp end critical (gd_shtns)
    call check(rc, 'getuv')
    ugrid = u * (rsphere / rsphere_lib)
    vgrid = v * (rsphere / rsphere_lib)
  end subroutine getuv_r8

  subroutine getvrtdivspec_r8(ugrid, vgrid, vrtspec, divspec, rsphere)
    real(c_double), dimension(:,:), intent(in) :: ugrid, vgrid
    complex(c_double_complex), dimension(:), intent(out) :: vrtspec, divspec
    real(c_double), intent(in) :: rsphere
    real(c_double) :: u(size(ugrid, 1), size(ugrid, 2)), v(size(vgrid, 1), size(vgrid, 2))
    complex(c_double_complex) :: a(nlm), b(nlm)
    integer(c_int) :: rc
    u = ugrid
    v = vgrid
    !$omp critical (gd_shtns)
    rc = gd_getvrtdivspec(ctx, 1_c_int, u, v, a, b)
    !$omp end critical (gd_shtns)
    call check(rc, 'getvrtdivspec')
    vrtspec = a * (rsphere_lib / rsphere)
    divspec = b * (rsphere_lib / rsphere)
  end subroutine getvrtdivspec_r8

  subroutine getgrad_r8(dataspec, ugrid, vgrid, rsphere)
    complex(c_double_complex), dimension(:), intent(in) :: dataspec
    real(c_double), dimension(:,:), intent(out) :: ugrid, vgrid
    real(c_double), intent(in) :: rsphere
    real(c_double) :: gx(size(ugrid, 1), size(ugrid, 2)), gy(size(vgrid, 1), size(vgrid, 2))
    complex(c_double_complex) :: s(nlm)
    integer(c_int) :: rc
    s = dataspec
    !$omp critical (gd_shtns)
    rc = gd_getgrad(ctx, 1_c_int, s, gx, gy)
    !$omp end critical (gd_shtns)
    call check(rc, 'getgrad')
    ugrid = gx * (rsphere_lib / rsphere)
    vgrid = gy * (rsphere_lib / rsphere)
  end subroutine getgrad_r8

end module shtns
