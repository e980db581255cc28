/*
 * gd_api.h -- C ABI of the GB300 (sm_103a) GFS spectral dycore step.
 *
 * Drop-in boundary for the time-step path of jswhit/gfs-dycore: the Fortran
 * host keeps init_dyn / getdyntend / advance / finalize_dyn and the shtns
 * transform facade, and binds these entry points through ISO_C_BINDING.
 *
 * Conventions
 *  - Every function returns an int status: GD_OK (0) or a negative GD_ERR_*.
 *    Nothing aborts; gd_last_error() describes the last failure.
 *  - Host arrays are caller-owned, read or written only during the call,
 *    in the reference layouts:
 *      spectral  double _Complex [nlev][nlm]  == Fortran complex(ndimspec,nlevs)
 *                (interleaved re,im doubles; m-major triangular order,
 *                 src/shtns.f90:149-150)
 *      grid      double [nlev][nlat][nlon]     == Fortran real(nlons,nlats,nlevs)
 *                (latitudes north to south, 3-D fields bottom to top,
 *                 src/grid_data.f90:14)
 *      tracers   double _Complex [ntrac][nlev][nlm]
 *  - Spectral harmonics are orthonormal without Condon-Shortley phase
 *    (src/shtns.f90:110); m > 0 coefficients stand for the (+m,-m) pair of a
 *    real field.
 *  - One context = one device state and one CUDA stream.  Calls on one
 *    context must be serialised by the caller (src/dyn_run.f90 calls the
 *    transforms from OpenMP threads; such callers use one context per
 *    thread or a lock).
 */
#ifndef GD_API_H
#define GD_API_H

#ifdef __cplusplus
extern "C" {
#endif

#define GD_OK 0
#define GD_ERR_ARG (-1)         /* bad argument, shape or null pointer      */
#define GD_ERR_CUDA (-2)        /* CUDA runtime error (message has detail)  */
#define GD_ERR_STATE (-3)       /* call out of order (e.g. no state set)    */
#define GD_ERR_NOMEM (-4)       /* device allocation failed                 */
#define GD_ERR_UNSUPPORTED (-5) /* configuration not supported              */
#define GD_ERR_NUMERIC (-6)     /* non-finite value detected in the state   */

/* Arithmetic of the transforms and the state. */
#define GD_PREC_FP64 0        /* everything FP64 (reference with default_real=2) */
#define GD_PREC_FP32 1        /* FP32 state and SIMT FP32 Legendre GEMMs          */
#define GD_PREC_TF32X3 2      /* FP32 state, Legendre as TF32x3 tcgen05 products  */
#define GD_PREC_BF16X3 3      /* FP32 state, Legendre as BF16x3 tcgen05 products  */
#define GD_PREC_F64_TF32X3 4  /* FP64 state, FFTs, column kernels and stage; the
                                 Legendre orders m >= 1 as TF32x3 tcgen05
                                 products of FP32-rounded operands, order 0
                                 on the FP64 SIMT path                           */
#define GD_PREC_F64_EDDY 5    /* FP64 state, column kernels and stage; every zonal
                                 mean (order 0) transformed in FP64; the eddy
                                 orders m >= 1 in FP32: longitude FFTs in FP32
                                 (the FP64 row mean taken out before rounding)
                                 and Legendre as TF32x3 tcgen05 products.  On
                                 grids whose nlon/2 has no four-step FFT kernel
                                 (64, 96, 192, 384, 576) the FFTs stay FP64, as
                                 in GD_PREC_F64_TF32X3                           */

typedef struct gd_config {
  int ntrunc;          /* triangular truncation T (params.f90 ntrunc)       */
  int nlon, nlat;      /* Gaussian grid; nlon = 2^a 3^b, nlat even          */
  int nlev;            /* levels (>= 3)                                     */
  int ntrac;           /* tracers; tracer 1 is humidity in the energy term  */
  double dt;           /* time step in seconds (params.f90 dt)              */
  int precision;       /* GD_PREC_*                                         */
  int explicit_;       /* params.f90 explicit (0 = semi-implicit IMEX RK3)  */
  int adiabatic;       /* params.f90 adiabatic (1 = no physics)             */
  int heldsuarez;      /* Held-Suarez physics plugin (phy_run_hs.f90)       */
  int massfix;         /* params.f90 massfix (dry-mass fixer)               */
  int dry;             /* params.f90 dry                                    */
  int ndiss;           /* params.f90 ndiss (0 -> 8)                         */
  double efold;        /* params.f90 efold (<= 0 -> GFS default)            */
  double hdif_fac, hdif_fac2, fshk, taustratdamp; /* params.f90:76-86      */
  double pdryini;      /* 0 -> set on the first stage-1 call               */
  int device;          /* CUDA device ordinal                               */
  int dcmip;           /* params.f90:62 dcmip: -1 none; 4x or 5x selects the
                          DCMIP simple physics plugin (phy_run_simple.f90;
                          moist unless dry, turbulent fluxes for 43 and 5x,
                          latitude-dependent SST for 4x) -- not together
                          with heldsuarez                                 */
} gd_config;

typedef struct gd_ctx gd_ctx;

/* Fills the reference's namelist defaults (src/params.f90:39-86) for a
   T42 128x64 L20 Held-Suarez run. */
int gd_default_config(gd_config* cfg);

/* Replaces init_dyn (src/dyn_init.f90:37-91) and shtns_init
   (src/shtns.f90:90-156): Gaussian grid, Legendre tables, damping
   (setdampspec, dyn_init.f90:450-494) and semi-implicit inverses
   (init_semimpdata, semimp_data.f90:127-256), all computed on the GPU in
   FP64.  ak, bk: nlev+1 interface coefficients, top to bottom
   (dyn_init.f90:52-56). */
int gd_init(const gd_config* cfg, const double* ak, const double* bk, gd_ctx** ctx);

/* Replaces finalize_dyn (src/dyn_finalize.f90:19-28). */
int gd_finalize(gd_ctx* ctx);

/* Sets / reads the prognostic spectral state (spectral_data.f90:11-21).
   trc may be NULL when ntrac = 0; topo may be NULL (flat orography).
   gd_set_state also derives phis and its gradient (dyn_init.f90:76-84). */
int gd_set_state(gd_ctx* ctx, const double* vrt, const double* div, const double* tv,
                 const double* trc, const double* lnps, const double* topo);
int gd_get_state(gd_ctx* ctx, double* vrt, double* div, double* tv, double* trc,
                 double* lnps);

/* gd_set_state / gd_get_state with single-precision host arrays (float
   _Complex, interleaved re, im floats, same layouts): the spectral state of
   the reference's default build (complex(r_kind), r_kind = 4,
   src/kinds.f90:100; spectral_data.f90:11-21), bound without a host-side
   widening copy.  Conversion to and from the context's state precision
   runs on the device; topo (may be NULL) is complex(r_kind) too. */
int gd_set_state_f(gd_ctx* ctx, const float* vrt, const float* div, const float* tv, const float* trc,
                   const float* lnps, const float* topo);
int gd_get_state_f(gd_ctx* ctx, float* vrt, float* div, float* tv, float* trc, float* lnps);

/* Reads the orography of the last gd_set_state (complex [nlm], metres; zero
   when it was given as NULL), the reference's topodataspec
   (spectral_data.f90, set at dyn_init.f90:76), so a caller can set a
   modified state again over the same surface. */
int gd_get_topo(gd_ctx* ctx, double* topo);

/* Replaces getdyntend (src/dyn_run.f90:33-305) on the current state.
   inverse_only != 0 is the just_do_inverse_transform form (grid fields,
   pressure data and getomega only; no tendencies are written). */
int gd_getdyntend(gd_ctx* ctx, int rkstage, int inverse_only, double* dvrt, double* ddiv,
                  double* dtv, double* dtrc, double* dlnps);

/* Replaces the physics plugin contract getphytend(dvrtspecdt, ddivspecdt,
   dvirtempspecdt, dtracerspecdt, dlnpsspecdt, t, dt) for the Held-Suarez
   forcing (src/phy_run_hs.f90:22-84), evaluated on the grid fields of the
   last gd_getdyntend call.  dtrc (may be NULL) is set to 0. */
int gd_getphytend(gd_ctx* ctx, double* dvrt, double* ddiv, double* dtv, double* dtrc,
                  double* dlnps);

/* Replaces nsteps calls of advance(t) (src/run.f90:194-565): IMEX RK3 with
   the semi-implicit solve, implicit hyperdiffusion, time-split Held-Suarez
   physics and the dry-mass fixer.  t (s) is the model time of the first
   step, t + k dt of the next ones; it matters only for the IAU forcing.
   Runs asynchronously on the context stream; the state stays on the
   device. */
int gd_advance(gd_ctx* ctx, double t, int nsteps);

/* Incremental analysis update (src/iau_module.f90, run.f90:250-258,
   301-308): increments (analysis - first guess) at nfiles >= 2 equally
   spaced forecast hours fhrs, in the state layouts with a leading nfiles
   axis: vrt, div, tv [nfiles][nlev][nlm], trc [nfiles][ntrac][nlev][nlm],
   lnps [nfiles][nlm].  Each step of gd_advance at time t adds the forcing
   of getiauforcing (iau_module.f90:88-135) -- the increments interpolated
   linearly in time between the bracketing files, divided by delthrs hours,
   zero outside [fhrs[0], fhrs[nfiles-1]] -- to the explicit tendencies of
   all three RK stages.  nfiles = 0 detaches. */
int gd_set_iau(gd_ctx* ctx, int nfiles, const double* fhrs, double delthrs, const double* vrt, const double* div,
               const double* tv, const double* trc, const double* lnps);
/* init_iau (iau_module.f90:19-79): the increments from pairs of sigma files
   (first guess fg[n], analysis anl[n], read as readin_sig reads them). */
int gd_set_iau_files(gd_ctx* ctx, int nfiles, const double* fhrs, double delthrs, const char* const* fg,
                     const char* const* anl);

/* Digital filter initialisation (run.f90:58-145): advances 2 ntdfi steps
   from time t, accumulating the Lanczos-weighted state (set_dfi_wts,
   run.f90:567-588; FP64 accumulator), then replaces the state by that
   average, valid at t + ntdfi dt; the accumulated precipitation restarts
   at 0 (init_phydata).  Synchronous. */
int gd_dfi(gd_ctx* ctx, double t, int ntdfi);
/* The 2 ntdfi + 1 filter weights of gd_dfi (host only). */
int gd_dfi_weights(int ntdfi, double* w);

/* Transform facade of src/shtns.f90, batched over nb 2-D fields
   (spectral [nb][nlm], grid [nb][nlat][nlon]); rsphere = 6.3712e6 m.
   gd_spectogrd    <- spectogrd     (shtns.f90:203-231)
   gd_grdtospec    <- grdtospec     (shtns.f90:171-201)
   gd_getuv        <- getuv         (shtns.f90:233-273)
   gd_getvrtdivspec<- getvrtdivspec (shtns.f90:275-311)
   gd_getgrad      <- getgrad       (shtns.f90:313-352) */
int gd_spectogrd(gd_ctx* ctx, int nb, const double* spec, double* grid);
int gd_grdtospec(gd_ctx* ctx, int nb, const double* grid, double* spec);
int gd_getuv(gd_ctx* ctx, int nb, const double* vrt, const double* div, double* u, double* v);
int gd_getvrtdivspec(gd_ctx* ctx, int nb, const double* u, const double* v, double* vrt,
                     double* div);
int gd_getgrad(gd_ctx* ctx, int nb, const double* spec, double* gx, double* gy);

/* The same five transforms with single-precision host arrays: the
   reference's default build passes complex(r_kind) / real(r_kind) with
   r_kind = 4 (src/kinds.f90:100) to the shtns.f90 wrappers, which widen
   them to double on the host before SHTns (shtns.f90:192-197, 222-229).
   Here the float arrays are copied as they are and converted on the device
   (half the bytes over the host link); the arithmetic is the context's
   precision mode.  Spectral arrays are float _Complex (interleaved re, im
   floats) [nb][nlm], grids float [nb][nlat][nlon]. */
int gd_spectogrd_f(gd_ctx* ctx, int nb, const float* spec, float* grid);
int gd_grdtospec_f(gd_ctx* ctx, int nb, const float* grid, float* spec);
int gd_getuv_f(gd_ctx* ctx, int nb, const float* vrt, const float* div, float* u, float* v);
int gd_getvrtdivspec_f(gd_ctx* ctx, int nb, const float* u, const float* v, float* vrt, float* div);
int gd_getgrad_f(gd_ctx* ctx, int nb, const float* spec, float* gx, float* gy);

/* Module data of src/shtns.f90:58-60: lats (radians, nlat), gauwts (nlat),
   areawts per latitude (nlat; sum over the grid is 1), degree, order (nlm),
   lap, invlap (nlm).  Any pointer may be NULL. */
int gd_grid_info(gd_ctx* ctx, double* lats, double* gauwts, double* areawts, int* degree,
                 int* order, double* lap, double* invlap);

/* Grid fields of the last getdyntend: "ug" "vg" "vrtg" "divg" "tvg" "trcg"
   "dlnpdtg" "etadot" "lnpsg" "psg" "dlnpsdt" "prs" "dphisdx" "dphisdy", "sppt"
   (the logit-transformed stochastic-physics pattern of the last step, while
   one is attached), and the physics fields of phy_data.f90 "precip" (mm/s),
   "apcp" (mm, accumulated), "pwat" (kg/m^2) -- zero but for the moist
   DCMIP physics. */
int gd_get_grid(gd_ctx* ctx, const char* name, double* out);

/* Step diagnostics of src/run.f90:159-161 after the last step:
   out[0] spdmax (m/s), out[1] min ps (hPa), out[2] max ps (hPa),
   out[3] ps tendency RMS (hPa/hr), out[4] pdryini (Pa). */
int gd_diag(gd_ctx* ctx, double* out5);

/* Runs one time step eagerly with CUDA events between its phases (the
   reference prints per-stage system_clock times, src/run.f90:311,361,427,
   :506,:525).  ms[0..7] receive milliseconds spent in: 0 Legendre
   synthesis, 1 longitude FFT synthesis, 2 grid-space column kernels,
   3 longitude FFT analysis, 4 Legendre analysis, 5 semi-implicit / RK
   stage updates, 6 physics grid work and update, 7 other, and with
   nphase >= 9: 8 the DCMIP column-physics kernel alone (else counted in
   6).  The state advances by one step.  nphase must be >= 8. */
int gd_profile_step(gd_ctx* ctx, double* ms, int nphase);

/* Allocation-free step diagnostics.  This entry point has no counterpart in
   the reference; it exists for callers that cannot call cudaMalloc (a host
   model whose device memory belongs to another runtime's pool allocator,
   or a process whose device-memory budget is fully committed).  It computes
   what gd_diag reports (out4[0] spdmax, [1] min ps hPa, [2] max ps hPa,
   [3] ps tendency RMS hPa/hr; src/run.f90:159-161) from caller-provided,
   device-accessible arrays: ug, vg [nlev][nlat][nlon], psg and dlnpsdt
   [nlat][nlon], gauwts [nlat] (Gauss weights, sum 2), out4 [4] doubles.
   No context is needed and nothing is allocated: the per-latitude scratch
   is a fixed device array of GD_DIAG_STATIC_MAX_NLAT rows that every GPU
   loading the library holds until exit; nlat above that limit is rejected
   with GD_ERR_ARG.  The first call on a device looks up that array's
   address with the device current; make that first call before any stream
   capture.  The address is kept with the id of the CUDA context it belongs
   to: after a cudaDeviceReset the next call (under the new context) looks
   it up again, and that call too should come before any stream capture.
   All calls share the array, so calls that overlap on the GPU race.  Work is enqueued on stream (cudaStream_t as void*, NULL = legacy
   default stream) and is complete when the stream is. */
#define GD_DIAG_STATIC_MAX_NLAT 4096
int gd_diag_static(const double* ug, const double* vg, int nlev, const double* psg,
                   const double* dlnpsdt, const double* gauwts, int nlat, int nlon, double* out4,
                   void* stream);

/* ---- stochastic pattern generator (src/patterngenerator.f90) -------------
   AR(1) random patterns in spherical-harmonic space with a Gaussian spatial
   covariance of length scale lscale (m) and e-folding time tscale (s), drawn
   from the w3lib Mersenne twister (src/w3lib/mersenne_twister.f) as the
   reference does; single-precision arithmetic as in the reference's default
   build.  One generator owns one random stream and nfields patterns that
   draw from it in turn (stoch_data.f90:120-142 uses one stream for all
   levels).  Spectral arrays are double _Complex[nfields][nlm], m-major
   triangular (the reference's complex(ndimspec, nfields)). */
typedef struct gd_pattern gd_pattern;
/* patterngenerator_init (patterngenerator.f90:33-65) + gaussian_spect
   (:145-177).  normalization is the reference's normfact (2*pi in every
   call of stoch_data.f90); iseed 0 takes a seed from the clock, as the
   reference does. */
int gd_pattern_init(double lscale, double delt, double tscale, double stdev, int iseed, int nlon, int nlat,
                    int jcap, double normalization, int nfields, int device, gd_pattern** out);
/* The start of a pattern (stoch_data.f90:58, 81, 104, 124-127):
   spec = stdev * getnoise * varspectrum, field after field. */
int gd_pattern_start(gd_pattern* p);
/* patterngenerator_advance (patterngenerator.f90:134-143) nsteps times,
   advancing every field in turn at each step. */
int gd_pattern_advance(gd_pattern* p, int nsteps);
/* getnoise (patterngenerator.f90:115-132): one draw of unit-variance white
   noise, noise = double _Complex[nlm]. */
int gd_pattern_getnoise(gd_pattern* p, double* noise);
/* The patterns (the reference's spec_sppt & co.), read and written. */
int gd_pattern_get(gd_pattern* p, double* spec);
int gd_pattern_set(gd_pattern* p, const double* spec);
/* rpattern%varspectrum [nlm], %varspectrum1d [jcap+1] and %phi; any output
   may be NULL. */
int gd_pattern_spectra(gd_pattern* p, double* varspectrum, double* varspectrum1d, double* phi);
/* patterngenerator_destroy (patterngenerator.f90:67-71). */
int gd_pattern_destroy(gd_pattern* p);
/* Runs the generator on an external CUDA stream (cudaStream_t as void*). */
int gd_pattern_set_stream(gd_pattern* p, void* stream);
/* Waits for the generator's work. */
int gd_pattern_sync(gd_pattern* p);
/* Number of GPU kernel launches issued by the generator so far. */
long long gd_pattern_launch_count(gd_pattern* p);
/* Text of the last error on p (or of the last failed gd_pattern_init if NULL). */
const char* gd_pattern_last_error(gd_pattern* p);

/* Stochastically perturbed physics (SPPT).  Attaches pattern (NULL
   detaches) to ctx: at the start of every gd_advance step the pattern is
   advanced one AR(1) step and put on the grid with the logit transform
   2/(1+exp(g))-1 (src/run.f90:277-281), and the physics tendencies are scaled
   by 1 + vfact(k) * pattern (src/phy_run_gfs.f90:617-620), vfact 1 below
   sigma sigbot, 0 above sigtop, linear between (src/stoch_data.f90:86-94,
   sigbot 0.10, sigtop 0.05 there).  Here the physics is the Held-Suarez
   forcing, whose Tv, vorticity and divergence tendencies are scaled on the
   grid.  The pattern must live on ctx's device with a truncation at most
   ctx's; it is advanced on ctx's stream. */
int gd_set_sppt(gd_ctx* ctx, gd_pattern* pattern, double sigtop, double sigbot);
/* Advances n independent contexts (ensemble members, any mix of
   truncations, one device) by nsteps steps each.  Once every member has a
   captured step graph (after its first two steps, taken member by member on
   the members' streams), each ensemble step is one launch of a graph holding
   every member's step as an independent child, so the members' steps
   overlap on the GPU.  Members with per-step host work (the IAU forcing)
   step member by member.  Returns when all are done.  Members must not share
   a closure net (their steps run at once).  No counterpart in the reference,
   which runs one member per process. */
int gd_ensemble_advance(gd_ctx** ctxs, int n, double t, int nsteps);

/* DCMIP-2012 initial state (dcmip_ics, src/dyn_init.f90:330-416) on ctx's grid:
   testcase 4x the baroclinic wave (src/dcmip_initial_conditions_test_4_v3.f90;
   ps = 1e5 Pa; tracers 2 and 3 potential temperature and |Ertel PV|;
   humidity in tracer 1 unless dry), 5x the tropical cyclone
   (src/dcmip_initial_conditions_test_5_v1.f90; moist only).  The point
   values are evaluated on the host at the model's layer pressures (its ak,
   bk and the case's ps), Tv = T (1 + fvirt q), and transformed with ctx's
   own transforms (winds through gd_getvrtdivspec, orography phis/g) into
   the state, as gd_set_state.  Needs ntrac >= 3 for 4x, >= 1 for 5x. */
int gd_dcmip_ics(gd_ctx* ctx, int testcase);
/* The analytic state of gd_dcmip_ics at one point, host only (no context):
   out[8] = u, v, T, phis, ps, q, q1, q2 (q1, q2 zero for 5x) at longitude,
   latitude (radians) and pressure p (Pa); moist as for test 4. */
int gd_dcmip_point(int testcase, int moist, double lon, double lat, double p, double* out);

/* ---- sigma files (src/sigio_module.f90) ----------------------------------
   The GFS spectral "sigma" file: big-endian Fortran unformatted sequential
   records (4-byte length markers before and after each record), in either
   header version the reference reads: ivs 200509 ('GFS SIG ' label, header
   records of 32, 4*(nhead+ndata), 200, 4*(levs+1)*nvcoord, 8*(5+ntrac)
   bytes, then cpi and ri when mod(idvm/10,10) == 3) or 198410 (a 32-byte
   ON85 label and one 250-word record).  The data records follow: orography,
   ln(ps in cb), levs temperature records, levs (divergence, vorticity)
   pairs, ntrac*levs tracer records, nxgr grid records of lonb*latb words,
   and nxss scalars; nc = (jcap+1)(jcap+2) words each, 4-byte floats unless
   irealf == 2 (8-byte).  Records are read and written whole; a record of
   2^31 bytes or more (gfortran subrecords) is not supported.
   All file calls are host-only (no GPU) and thread-safe on distinct files;
   gd_sigio_last_error() reports the calling thread's last failure. */
#define GD_ERR_IO (-7)             /* file cannot be opened, read or written, or
                                      is not a sigma file of a known version   */
#define GD_SIG_MAXLEVS 256         /* levels a header can describe            */
#define GD_SIG_MAXTRAC 100         /* tracers a header can describe           */
#define GD_SIG_FILL (-9999.0f)     /* sigio_realfill / sigio_intfill          */

/* type sigio_head (sigio_module.f90:337-379), fixed-size.  vcoord(k,j) of
   the Fortran header is vcoord[j-1][k-1] (k = 1..levs+1 bottom to top,
   j = 1..nvcoord <= 3); cfvars holds 5+ntrac blank-padded 8-character
   names; cpi and ri hold ntrac+1 values when mod(idvm/10,10) == 3.  nxgr,
   nxss, nhead, ndata are derived from the other fields (sigio_adhead,
   sigio_module.f90:1323-1382) on every read and write. */
typedef struct gd_sighead {
  char clabsig[32];
  float fhour;
  int idate[4];                        /* hour, month, day, year          */
  float si[101], sl[100], ak[101], bk[101];
  int jcap, levs, itrun, iorder, irealf, igen, latf, lonf, latb, lonb, latr, lonr;
  int ntrac, icen2, iens[2], idpp, idsl, idvc, idvm, idvt, idrun, idusr;
  float pdryini;                       /* cb                               */
  int ncldt, ixgr, ivs, nvcoord;
  float vcoord[3][GD_SIG_MAXLEVS + 1];
  char cfvars[5 + GD_SIG_MAXTRAC][8];
  int nxgr, nxss, nhead, ndata;
  float cpi[GD_SIG_MAXTRAC + 1], ri[GD_SIG_MAXTRAC + 1];
} gd_sighead;

/* The default-initialised sigio_head: every number the fill value, every
   label blank (sigio_module.f90:338-379). */
int gd_sigio_head_init(gd_sighead* head);
/* sigio_sropen + sigio_srhead (sigio_module.f90:430-442, 470-576).  As in
   the reference, a 200509 header comes back with si, sl, ak, bk and pdryini
   set to the fill value (the file's pdryini word is not kept), and a 198410
   header with jcap..ixgr truncated from its real-valued ext words, ntrac at
   least 1, and vcoord taken from its sigma/hybrid words by idvc. */
int gd_sigio_read_head(const char* path, gd_sighead* head);
/* readin_sig (src/dyn_init.f90:120-149) = sigio_srohdc + copyspecin: reads
   header and data and renormalises every spectral field from the NCEP
   normalisation to the model's orthonormal one, c = sqrt(2 pi) *
   (re, im) per coefficient (dyn_init.f90:93-104, pi the reference's
   single-rounded con_pi), sequentially with no reordering.  Values pass
   through single precision as in the reference (irealf 2 data are rounded
   to float by sigio_srdata).  The file must have truncation jcap, levs
   levels and at least ntrac tracers (the first ntrac are read); outputs
   are double _Complex: vrt, div, tv [levs][nlm], trc [ntrac][levs][nlm],
   lnps (ln of ps in cb, as stored) and topo (orography, m) [nlm],
   nlm = (jcap+1)(jcap+2)/2; any output may be NULL. */
int gd_sigio_read(const char* path, int jcap, int levs, int ntrac, gd_sighead* head, double* vrt,
                  double* div, double* tv, double* trc, double* lnps, double* topo);
/* copyspecout + sigio_swohdc (dyn_init.f90:106-118, sigio_module.f90:942-962,
   578-676, 836-915): writes head (its version chooses the header layout;
   nxgr/nxss/nhead/ndata are recomputed into it) and the spectral fields
   divided by sqrt(2 pi) and rounded to float (then widened when irealf ==
   2).  trc holds ntrac <= head->ntrac tracers; the remaining tracer
   records, and any extra grid/scalar records the header declares, are
   written as zeros (the reference writes its unset buffers there).  A 198410
   header with a sigma coordinate whose vcoord(1,1) is 1 gets its layer
   values from sigio_modpr (sigio_module.f90:1207-1321) at ps = 1. */
int gd_sigio_write(const char* path, gd_sighead* head, int ntrac, const double* vrt, const double* div,
                   const double* tv, const double* trc, const double* lnps, const double* topo);
/* The model configuration a header implies (src/params.f90:250-264 and
   src/dyn_init.f90:52-66): cfg->ntrunc = jcap, nlon = lonb, nlat = latb,
   nlev = levs, pdryini = 1000 * head pdryini (Pa), 0 when above 1e5 Pa; ak, bk
   [levs+1] top to bottom from the hybrid vcoord, reversed.  A header whose
   pdryini is the fill value (every 200509 header as read) gives 0, i.e. the
   first step's dry mass; the reference would take -9.999e6 Pa there.  Other
   cfg fields are left as they are; idvc other than 2 returns
   GD_ERR_UNSUPPORTED as the reference stops there. */
int gd_sigio_config(const gd_sighead* head, gd_config* cfg, double* ak, double* bk);
/* readin_sig and the start of init_dyn on a context (dyn_init.f90:44-48):
   reads path (jcap, levs must be ctx's, at least ctx's ntrac tracers),
   converts ln(ps in cb) to ln(ps in Pa) -- the reference's spectogrd,
   1000*exp, log, grdtospec round trip, which for the band-limited field is
   the constant ln(1000) added to the (0,0) coefficient, done here that way
   -- and sets the state and orography as gd_set_state does. */
int gd_read_sig(gd_ctx* ctx, const char* path, gd_sighead* head);
/* wrtout_sig (dyn_init.f90:151-191): head->fhour = fhour, head->pdryini =
   the context's pdryini / 1000 (cb); writes the context's state with ln(ps)
   back in cb (the constant ln(1000) taken off the (0,0) coefficient) and
   the orography of the last gd_set_state / gd_read_sig.  head's jcap and
   levs must be ctx's and head->ntrac at least ctx's ntrac. */
int gd_write_sig(gd_ctx* ctx, const char* path, double fhour, gd_sighead* head);
/* Text of the calling thread's last sigma-file failure. */
const char* gd_sigio_last_error(void);

/* Autotuner: times the candidate tile shapes of this context's kernels on
   its own buffers (a state must be set) and keeps the fastest for the later
   steps.  choices must hold 3 ints: choices[0] = the synthesis Legendre
   GEMM's latitude tile (split precision modes; 0 otherwise), choices[1] =
   the column kernel's levels per warp, choices[2] = the A-operand slots in
   tensor memory requested for both Legendre GEMMs (split modes; 0
   otherwise).  Results do not depend on the tile or the slots; the levels
   per warp change the order of the column sums (last-bit differences). */
int gd_autotune(gd_ctx* ctx, int* choices);

/* ---- Learned per-column closure -----------------------------------------
   A fully connected network nin -> nhidden (GELU) x nlayers -> nout with
   BF16 weights and FP32 accumulation, trained on the GPU by the library's
   own forward and backward kernels (mean-squared error, Adam).  The closure
   configuration is a coarse run (T62L64) whose tendencies the network
   corrects from each grid column's u, v, Tv (levels bottom to top) and ps:
   nin = 3 nlev + 1, nout = 3 nlev (du/dt, dv/dt, dTv/dt).  It has no
   counterpart in the reference; the plain step stays the fallback and the
   measure of its error.  x, t and y below are device pointers of float
   [ncols][nin] / [ncols][nout]; parameters are host float arrays in the
   packed layout (per layer W [fout][fin] row-major, then b [fout]). */
typedef struct gd_mlp gd_mlp;
/* A net with He-normal hidden weights from seed (output layer x 0.1). */
int gd_mlp_init(int nin, int nhidden, int nlayers, int nout, unsigned long long seed, int device, gd_mlp** out);
int gd_mlp_destroy(gd_mlp* net);
int gd_mlp_nparams(gd_mlp* net, long long* n);
int gd_mlp_get_params(gd_mlp* net, float* params);
int gd_mlp_set_params(gd_mlp* net, const float* params);
/* Normalisation of a closure's raw inputs ((x - in_mu) / in_sd) and outputs
   (y out_sd + out_mu), host arrays of nin and nout. */
int gd_mlp_set_norm(gd_mlp* net, const float* in_mu, const float* in_sd, const float* out_mu, const float* out_sd);
/* y = net(x) on the net's stream (asynchronous). */
int gd_mlp_forward(gd_mlp* net, const float* x, int ncols, float* y);
/* Mean-squared error of net(x) against t and its gradient with respect to
   the parameters (host float[nparams], may be NULL); synchronous. */
int gd_mlp_loss_grad(gd_mlp* net, const float* x, const float* t, int ncols, float* loss, float* grad);
/* One Adam step (beta 0.9, 0.999, eps 1e-8) on the batch (x, t); the loss
   before the step to *loss when not NULL (then synchronous). */
int gd_mlp_train_step(gd_mlp* net, const float* x, const float* t, int ncols, float lr, float* loss);
/* Runs the net's own calls on an external CUDA stream (NULL: its own). */
int gd_mlp_set_stream(gd_mlp* net, void* stream);
int gd_mlp_sync(gd_mlp* net);
/* Text of the last error on net (or of the last failed gd_mlp_init if NULL). */
const char* gd_mlp_last_error(gd_mlp* net);
/* Attaches a trained net (with its normalisation) to ctx: every step, after
   the forcing, the net's tendencies times dt are added to Tv and, through
   the vector analysis, to vorticity and divergence.  NULL detaches.  The net
   must live on ctx's device with nin = 3 nlev + 1 and nout = 3 nlev; it
   runs on ctx's stream while attached and must outlive the attachment
   (detach before gd_mlp_destroy). */
int gd_set_closure(gd_ctx* ctx, gd_mlp* net);
/* The raw closure inputs of ctx's current state, host float[nlat nlon][3
   nlev + 1]: u, v, Tv at the levels bottom to top and ps (Pa) per column. */
int gd_closure_features(gd_ctx* ctx, float* x);

/* Runs the context on an external CUDA stream (cudaStream_t as void*). */
int gd_set_stream(gd_ctx* ctx, void* stream);
/* Waits for all work of the context. */
int gd_sync(gd_ctx* ctx);
/* Number of GPU kernel launches issued by the context so far. */
long long gd_launch_count(gd_ctx* ctx);
/* Text of the last error on ctx (or of the last failed gd_init if NULL). */
const char* gd_last_error(gd_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* GD_API_H */
