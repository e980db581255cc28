! gd_api.f90 -- ISO_C_BINDING interface module of include/gd_api.h for a
! Fortran host (the reference's src/*.f90).  One interface per entry point,
! same names and argument order as the C declarations; every function
! returns the C status (GD_OK = 0 or a negative GD_ERR_*).
!
! Conventions of the binding:
!  - the context, pattern and network handles are type(c_ptr) values;
!  - host arrays are assumed-size dummies in the C layout: spectral
!    complex(c_double_complex) (nlm, nb) -- the reference's
!    complex(r_kind) dataspec(ndimspec, nlevs) with r_kind = 8 -- or
!    complex(c_float_complex) for the *_f entry points (r_kind = 4,
!    src/kinds.f90:100); grids real(c_double) / real(c_float) (nlon, nlat, nb);
!  - device pointers (gd_diag_static, gd_mlp_*) and CUDA streams are passed
!    as type(c_ptr), value;
!  - returned C strings (gd_last_error and friends) are type(c_ptr): convert
!    with c_f_pointer to a character(kind=c_char) array up to the NUL;
!  - path arguments are NUL-terminated: trim(path)//c_null_char.
!
! Not compiled on the build machine or the GPU host: neither has a Fortran
! compiler.  The C side of every interface is exercised through ctypes by
! the test suite.
module gd_api
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: GD_OK = 0, GD_ERR_ARG = -1, GD_ERR_CUDA = -2, GD_ERR_STATE = -3, &
                               GD_ERR_NOMEM = -4, GD_ERR_UNSUPPORTED = -5, GD_ERR_NUMERIC = -6, &
                               GD_ERR_IO = -7
  integer(c_int), parameter :: GD_PREC_FP64 = 0, GD_PREC_FP32 = 1, GD_PREC_TF32X3 = 2, &
                               GD_PREC_BF16X3 = 3, GD_PREC_F64_TF32X3 = 4, GD_PREC_F64_EDDY = 5
  integer(c_int), parameter :: GD_DIAG_STATIC_MAX_NLAT = 4096
  integer, parameter :: GD_SIG_MAXLEVS = 256, GD_SIG_MAXTRAC = 100

  ! gd_config: the namelist values of src/params.f90 the step needs
  type, bind(c) :: gd_config
    integer(c_int)  :: ntrunc, nlon, nlat, nlev, ntrac
    real(c_double)  :: dt
    integer(c_int)  :: precision, explicit_, adiabatic, heldsuarez, massfix, dry, ndiss
    real(c_double)  :: efold, hdif_fac, hdif_fac2, fshk, taustratdamp, pdryini
    integer(c_int)  :: device
    integer(c_int)  :: dcmip
  end type

  ! gd_sighead: the fields of sigio_head (src/sigio_module.f90); vcoord(k,j)
  ! and cfvars(:,i) index as there
  type, bind(c) :: gd_sighead
    character(kind=c_char) :: clabsig(32)
    real(c_float)   :: fhour
    integer(c_int)  :: idate(4)
    real(c_float)   :: si(101), sl(100), ak(101), bk(101)
    integer(c_int)  :: jcap, levs, itrun, iorder, irealf, igen, latf, lonf, latb, lonb, latr, lonr
    integer(c_int)  :: ntrac, icen2, iens(2), idpp, idsl, idvc, idvm, idvt, idrun, idusr
    real(c_float)   :: pdryini
    integer(c_int)  :: ncldt, ixgr, ivs, nvcoord
    real(c_float)   :: vcoord(GD_SIG_MAXLEVS + 1, 3)
    character(kind=c_char) :: cfvars(8, 5 + GD_SIG_MAXTRAC)
    integer(c_int)  :: nxgr, nxss, nhead, ndata
    real(c_float)   :: cpi(GD_SIG_MAXTRAC + 1), ri(GD_SIG_MAXTRAC + 1)
  end type

  interface
    ! ---------------------------------------------- lifecycle and state --
    integer(c_int) function gd_default_config(cfg) bind(c, name='gd_default_config')
      import :: c_int, gd_config
      type(gd_config), intent(out) :: cfg
    end function
    integer(c_int) function gd_init(cfg, ak, bk, ctx) bind(c, name='gd_init')
      import :: c_int, c_double, c_ptr, gd_config
      type(gd_config), intent(in) :: cfg
      real(c_double), intent(in) :: ak(*), bk(*)
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function gd_finalize(ctx) bind(c, name='gd_finalize')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function gd_set_state(ctx, vrt, div, tv, trc, lnps, topo) bind(c, name='gd_set_state')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(in) :: vrt(*), div(*), tv(*), trc(*), lnps(*), topo(*)
    end function
    integer(c_int) function gd_get_state(ctx, vrt, div, tv, trc, lnps) bind(c, name='gd_get_state')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: vrt(*), div(*), tv(*), trc(*), lnps(*)
    end function
    integer(c_int) function gd_set_state_f(ctx, vrt, div, tv, trc, lnps, topo) bind(c, name='gd_set_state_f')
      import :: c_int, c_ptr, c_float_complex
      type(c_ptr), value :: ctx
      complex(c_float_complex), intent(in) :: vrt(*), div(*), tv(*), trc(*), lnps(*), topo(*)
    end function
    integer(c_int) function gd_get_state_f(ctx, vrt, div, tv, trc, lnps) bind(c, name='gd_get_state_f')
      import :: c_int, c_ptr, c_float_complex
      type(c_ptr), value :: ctx
      complex(c_float_complex), intent(out) :: vrt(*), div(*), tv(*), trc(*), lnps(*)
    end function
    integer(c_int) function gd_get_topo(ctx, topo) bind(c, name='gd_get_topo')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: topo(*)
    end function
    ! --------------------------------------------------- step and physics --
    integer(c_int) function gd_getdyntend(ctx, rkstage, inverse_only, dvrt, ddiv, dtv, dtrc, dlnps) &
        bind(c, name='gd_getdyntend')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: rkstage, inverse_only
      complex(c_double_complex), intent(out) :: dvrt(*), ddiv(*), dtv(*), dtrc(*), dlnps(*)
    end function
    integer(c_int) function gd_getphytend(ctx, dvrt, ddiv, dtv, dtrc, dlnps) bind(c, name='gd_getphytend')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: dvrt(*), ddiv(*), dtv(*), dtrc(*), dlnps(*)
    end function
    integer(c_int) function gd_advance(ctx, t, nsteps) bind(c, name='gd_advance')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: t
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function gd_set_iau(ctx, nfiles, fhrs, delthrs, vrt, div, tv, trc, lnps) &
        bind(c, name='gd_set_iau')
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nfiles
      real(c_double), intent(in) :: fhrs(*)
      real(c_double), value :: delthrs
      complex(c_double_complex), intent(in) :: vrt(*), div(*), tv(*), trc(*), lnps(*)
    end function
    integer(c_int) function gd_set_iau_files(ctx, nfiles, fhrs, delthrs, fg, anl) &
        bind(c, name='gd_set_iau_files')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nfiles
      real(c_double), intent(in) :: fhrs(*)
      real(c_double), value :: delthrs
      type(c_ptr), intent(in) :: fg(*), anl(*)   ! c_loc of NUL-terminated paths
    end function
    integer(c_int) function gd_dfi(ctx, t, ntdfi) bind(c, name='gd_dfi')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: t
      integer(c_int), value :: ntdfi
    end function
    integer(c_int) function gd_dfi_weights(ntdfi, w) bind(c, name='gd_dfi_weights')
      import :: c_int, c_double
      integer(c_int), value :: ntdfi
      real(c_double), intent(out) :: w(*)
    end function
    ! --------------------------------------------------------- transforms --
    integer(c_int) function gd_spectogrd(ctx, nb, spec, grid) bind(c, name='gd_spectogrd')
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      complex(c_double_complex), intent(in) :: spec(*)
      real(c_double), intent(out) :: grid(*)
    end function
    integer(c_int) function gd_grdtospec(ctx, nb, grid, spec) bind(c, name='gd_grdtospec')
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      real(c_double), intent(in) :: grid(*)
      complex(c_double_complex), intent(out) :: spec(*)
    end function
    integer(c_int) function gd_getuv(ctx, nb, vrt, div, u, v) bind(c, name='gd_getuv')
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      complex(c_double_complex), intent(in) :: vrt(*), div(*)
      real(c_double), intent(out) :: u(*), v(*)
    end function
    integer(c_int) function gd_getvrtdivspec(ctx, nb, u, v, vrt, div) bind(c, name='gd_getvrtdivspec')
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      real(c_double), intent(in) :: u(*), v(*)
      complex(c_double_complex), intent(out) :: vrt(*), div(*)
    end function
    integer(c_int) function gd_getgrad(ctx, nb, spec, gx, gy) bind(c, name='gd_getgrad')
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      complex(c_double_complex), intent(in) :: spec(*)
      real(c_double), intent(out) :: gx(*), gy(*)
    end function
    integer(c_int) function gd_spectogrd_f(ctx, nb, spec, grid) bind(c, name='gd_spectogrd_f')
      import :: c_int, c_ptr, c_float, c_float_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      complex(c_float_complex), intent(in) :: spec(*)
      real(c_float), intent(out) :: grid(*)
    end function
    integer(c_int) function gd_grdtospec_f(ctx, nb, grid, spec) bind(c, name='gd_grdtospec_f')
      import :: c_int, c_ptr, c_float, c_float_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      real(c_float), intent(in) :: grid(*)
      complex(c_float_complex), intent(out) :: spec(*)
    end function
    integer(c_int) function gd_getuv_f(ctx, nb, vrt, div, u, v) bind(c, name='gd_getuv_f')
      import :: c_int, c_ptr, c_float, c_float_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      complex(c_float_complex), intent(in) :: vrt(*), div(*)
      real(c_float), intent(out) :: u(*), v(*)
    end function
    integer(c_int) function gd_getvrtdivspec_f(ctx, nb, u, v, vrt, div) bind(c, name='gd_getvrtdivspec_f')
      import :: c_int, c_ptr, c_float, c_float_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      real(c_float), intent(in) :: u(*), v(*)
      complex(c_float_complex), intent(out) :: vrt(*), div(*)
    end function
    integer(c_int) function gd_getgrad_f(ctx, nb, spec, gx, gy) bind(c, name='gd_getgrad_f')
      import :: c_int, c_ptr, c_float, c_float_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: nb
      complex(c_float_complex), intent(in) :: spec(*)
      real(c_float), intent(out) :: gx(*), gy(*)
    end function
    integer(c_int) function gd_grid_info(ctx, lats, gauwts, areawts, degree, order, lap, invlap) &
        bind(c, name='gd_grid_info')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: lats(*), gauwts(*), areawts(*), lap(*), invlap(*)
      integer(c_int), intent(out) :: degree(*), order(*)
    end function
    ! -------------------------------------------------------- diagnostics --
    integer(c_int) function gd_get_grid(ctx, name, out) bind(c, name='gd_get_grid')
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: name(*)
      real(c_double), intent(out) :: out(*)
    end function
    integer(c_int) function gd_diag(ctx, out5) bind(c, name='gd_diag')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out5(5)
    end function
    integer(c_int) function gd_profile_step(ctx, ms, nphase) bind(c, name='gd_profile_step')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: ms(*)
      integer(c_int), value :: nphase
    end function
    integer(c_int) function gd_diag_static(ug, vg, nlev, psg, dlnpsdt, gauwts, nlat, nlon, out4, stream) &
        bind(c, name='gd_diag_static')
      import :: c_int, c_ptr
      type(c_ptr), value :: ug, vg, psg, dlnpsdt, gauwts, out4, stream   ! device pointers, cudaStream_t
      integer(c_int), value :: nlev, nlat, nlon
    end function
    integer(c_int) function gd_set_stream(ctx, stream) bind(c, name='gd_set_stream')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, stream
    end function
    integer(c_int) function gd_sync(ctx) bind(c, name='gd_sync')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_long_long) function gd_launch_count(ctx) bind(c, name='gd_launch_count')
      import :: c_long_long, c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function gd_last_error(ctx) bind(c, name='gd_last_error')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    ! ------------------------------------------ stochastic patterns, SPPT --
    integer(c_int) function gd_pattern_init(lscale, delt, tscale, stdev, iseed, nlon, nlat, jcap, &
        normalization, nfields, device, p) bind(c, name='gd_pattern_init')
      import :: c_int, c_double, c_ptr
      real(c_double), value :: lscale, delt, tscale, stdev
      integer(c_int), value :: iseed, nlon, nlat, jcap
      real(c_double), value :: normalization
      integer(c_int), value :: nfields, device
      type(c_ptr), intent(out) :: p
    end function
    integer(c_int) function gd_pattern_start(p) bind(c, name='gd_pattern_start')
      import :: c_int, c_ptr
      type(c_ptr), value :: p
    end function
    integer(c_int) function gd_pattern_advance(p, nsteps) bind(c, name='gd_pattern_advance')
      import :: c_int, c_ptr
      type(c_ptr), value :: p
      integer(c_int), value :: nsteps
    end function
    integer(c_int) function gd_pattern_getnoise(p, noise) bind(c, name='gd_pattern_getnoise')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: p
      complex(c_double_complex), intent(out) :: noise(*)
    end function
    integer(c_int) function gd_pattern_get(p, spec) bind(c, name='gd_pattern_get')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: p
      complex(c_double_complex), intent(out) :: spec(*)
    end function
    integer(c_int) function gd_pattern_set(p, spec) bind(c, name='gd_pattern_set')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: p
      complex(c_double_complex), intent(in) :: spec(*)
    end function
    integer(c_int) function gd_pattern_spectra(p, varspectrum, varspectrum1d, phi) bind(c, name='gd_pattern_spectra')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: p
      real(c_double), intent(out) :: varspectrum(*), varspectrum1d(*), phi(*)
    end function
    integer(c_int) function gd_pattern_destroy(p) bind(c, name='gd_pattern_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: p
    end function
    integer(c_int) function gd_pattern_set_stream(p, stream) bind(c, name='gd_pattern_set_stream')
      import :: c_int, c_ptr
      type(c_ptr), value :: p, stream
    end function
    integer(c_int) function gd_pattern_sync(p) bind(c, name='gd_pattern_sync')
      import :: c_int, c_ptr
      type(c_ptr), value :: p
    end function
    integer(c_long_long) function gd_pattern_launch_count(p) bind(c, name='gd_pattern_launch_count')
      import :: c_long_long, c_ptr
      type(c_ptr), value :: p
    end function
    type(c_ptr) function gd_pattern_last_error(p) bind(c, name='gd_pattern_last_error')
      import :: c_ptr
      type(c_ptr), value :: p
    end function
    integer(c_int) function gd_set_sppt(ctx, pattern, sigtop, sigbot) bind(c, name='gd_set_sppt')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx, pattern
      real(c_double), value :: sigtop, sigbot
    end function
    integer(c_int) function gd_ensemble_advance(ctxs, n, t, nsteps) bind(c, name='gd_ensemble_advance')
      import :: c_int, c_ptr, c_double
      type(c_ptr), intent(in) :: ctxs(*)
      integer(c_int), value :: n
      real(c_double), value :: t
      integer(c_int), value :: nsteps
    end function
    ! ------------------------------------------------ DCMIP initial states --
    integer(c_int) function gd_dcmip_ics(ctx, testcase) bind(c, name='gd_dcmip_ics')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: testcase
    end function
    integer(c_int) function gd_dcmip_point(testcase, moist, lon, lat, p, out) bind(c, name='gd_dcmip_point')
      import :: c_int, c_double
      integer(c_int), value :: testcase, moist
      real(c_double), value :: lon, lat, p
      real(c_double), intent(out) :: out(*)
    end function
    ! -------------------------------------------------------- sigma files --
    integer(c_int) function gd_sigio_head_init(head) bind(c, name='gd_sigio_head_init')
      import :: c_int, gd_sighead
      type(gd_sighead), intent(out) :: head
    end function
    integer(c_int) function gd_sigio_read_head(path, head) bind(c, name='gd_sigio_read_head')
      import :: c_int, c_char, gd_sighead
      character(kind=c_char), intent(in) :: path(*)
      type(gd_sighead), intent(out) :: head
    end function
    integer(c_int) function gd_sigio_read(path, jcap, levs, ntrac, head, vrt, div, tv, trc, lnps, topo) &
        bind(c, name='gd_sigio_read')
      import :: c_int, c_char, c_double_complex, gd_sighead
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), value :: jcap, levs, ntrac
      type(gd_sighead), intent(out) :: head
      complex(c_double_complex), intent(out) :: vrt(*), div(*), tv(*), trc(*), lnps(*), topo(*)
    end function
    integer(c_int) function gd_sigio_write(path, head, ntrac, vrt, div, tv, trc, lnps, topo) &
        bind(c, name='gd_sigio_write')
      import :: c_int, c_char, c_double_complex, gd_sighead
      character(kind=c_char), intent(in) :: path(*)
      type(gd_sighead), intent(inout) :: head
      integer(c_int), value :: ntrac
      complex(c_double_complex), intent(in) :: vrt(*), div(*), tv(*), trc(*), lnps(*), topo(*)
    end function
    integer(c_int) function gd_sigio_config(head, cfg, ak, bk) bind(c, name='gd_sigio_config')
      import :: c_int, c_double, gd_sighead, gd_config
      type(gd_sighead), intent(in) :: head
      type(gd_config), intent(inout) :: cfg
      real(c_double), intent(out) :: ak(*), bk(*)
    end function
    integer(c_int) function gd_read_sig(ctx, path, head) bind(c, name='gd_read_sig')
      import :: c_int, c_ptr, c_char, gd_sighead
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
      type(gd_sighead), intent(out) :: head
    end function
    integer(c_int) function gd_write_sig(ctx, path, fhour, head) bind(c, name='gd_write_sig')
      import :: c_int, c_ptr, c_char, c_double, gd_sighead
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
      real(c_double), value :: fhour
      type(gd_sighead), intent(inout) :: head
    end function
    type(c_ptr) function gd_sigio_last_error() bind(c, name='gd_sigio_last_error')
      import :: c_ptr
    end function
    ! ------------------------------------------------------------ tuning --
    integer(c_int) function gd_autotune(ctx, choices) bind(c, name='gd_autotune')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: choices(3)
    end function
    ! ------------------------------------------- learned per-column closure --
    integer(c_int) function gd_mlp_init(nin, nhidden, nlayers, nout, seed, device, net) bind(c, name='gd_mlp_init')
      import :: c_int, c_long_long, c_ptr
      integer(c_int), value :: nin, nhidden, nlayers, nout
      integer(c_long_long), value :: seed   ! unsigned long long in C
      integer(c_int), value :: device
      type(c_ptr), intent(out) :: net
    end function
    integer(c_int) function gd_mlp_destroy(net) bind(c, name='gd_mlp_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: net
    end function
    integer(c_int) function gd_mlp_nparams(net, n) bind(c, name='gd_mlp_nparams')
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: net
      integer(c_long_long), intent(out) :: n
    end function
    integer(c_int) function gd_mlp_get_params(net, params) bind(c, name='gd_mlp_get_params')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: net
      real(c_float), intent(out) :: params(*)
    end function
    integer(c_int) function gd_mlp_set_params(net, params) bind(c, name='gd_mlp_set_params')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: net
      real(c_float), intent(in) :: params(*)
    end function
    integer(c_int) function gd_mlp_set_norm(net, in_mu, in_sd, out_mu, out_sd) bind(c, name='gd_mlp_set_norm')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: net
      real(c_float), intent(in) :: in_mu(*), in_sd(*), out_mu(*), out_sd(*)
    end function
    ! forward, loss_grad and train_step take the batch as device arrays; the
    ! loss and gradient outputs are host arrays that may be NULL (c_null_ptr)
    integer(c_int) function gd_mlp_forward(net, x, ncols, y) bind(c, name='gd_mlp_forward')
      import :: c_int, c_ptr
      type(c_ptr), value :: net, x, y
      integer(c_int), value :: ncols
    end function
    integer(c_int) function gd_mlp_loss_grad(net, x, t, ncols, loss, grad) bind(c, name='gd_mlp_loss_grad')
      import :: c_int, c_ptr
      type(c_ptr), value :: net, x, t, loss, grad
      integer(c_int), value :: ncols
    end function
    integer(c_int) function gd_mlp_train_step(net, x, t, ncols, lr, loss) bind(c, name='gd_mlp_train_step')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: net, x, t, loss
      integer(c_int), value :: ncols
      real(c_float), value :: lr
    end function
    integer(c_int) function gd_mlp_set_stream(net, stream) bind(c, name='gd_mlp_set_stream')
      import :: c_int, c_ptr
      type(c_ptr), value :: net, stream
    end function
    integer(c_int) function gd_mlp_sync(net) bind(c, name='gd_mlp_sync')
      import :: c_int, c_ptr
      type(c_ptr), value :: net
    end function
    type(c_ptr) function gd_mlp_last_error(net) bind(c, name='gd_mlp_last_error')
      import :: c_ptr
      type(c_ptr), value :: net
    end function
    integer(c_int) function gd_set_closure(ctx, net) bind(c, name='gd_set_closure')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, net
    end function
    integer(c_int) function gd_closure_features(ctx, x) bind(c, name='gd_closure_features')
      import :: c_int, c_ptr, c_float
      type(c_ptr), value :: ctx
      real(c_float), intent(out) :: x(*)   ! host (3 nlev + 1, nlon nlat)
    end function
  end interface
end module gd_api
