/*
 * gd_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * C interface of the FP64 CPU oracle: a restatement of the GFS spectral
 * dycore time step of jswhit/gfs-dycore (src/shtns.f90, src/dyn_run.f90,
 * src/pressure_data.f90, src/semimp_data.f90, src/run.f90::advance,
 * src/phy_run_hs.f90, src/dyn_init.f90::setdampspec) in plain C++ with
 * OpenMP over levels.  It is the parity oracle for the CUDA library and
 * the timed CPU baseline; nothing in the product links or calls it.
 *
 * Parity status: the reference cannot be built here (no Fortran compiler,
 * no SHTns, no FFTW) and ships no golden vectors, so the transforms are
 * pinned by analytic known-answer tests (scipy Gauss-Legendre nodes and
 * associated Legendre values, orthonormality, band-limited round trips,
 * solid-body rotation winds) and the semi-implicit inverses by scipy's
 * LAPACK dgetrf/dgetri -- the routines src/semimp_data.f90:248-249 calls.
 *
 * Layouts follow the reference: spectral arrays are Fortran
 * complex(ndimspec,nlevs) == C [nlev][nlm] interleaved (re,im) doubles,
 * m-major triangular order (src/shtns.f90:149-150); grid arrays are
 * Fortran (nlons,nlats,nlevs) == C [nlev][nlat][nlon], latitudes north to
 * south, 3-D grid fields bottom to top (src/grid_data.f90:14).
 */
#ifndef GD_ORACLE_H
#define GD_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_config {
  int ntrunc, nlon, nlat, nlev, ntrac;
  double dt;
  int explicit_;   /* params.f90:67 explicit */
  int adiabatic;   /* params.f90:54 */
  int heldsuarez;  /* params.f90:60 (HS forcing as physics plugin) */
  int massfix;     /* params.f90:42 */
  int dry;         /* params.f90:53 */
  int ndiss;       /* params.f90:72 (0 -> 8) */
  double efold;    /* params.f90:75 (<=0 -> GFS default) */
  double hdif_fac, hdif_fac2, fshk, taustratdamp;
  double pdryini;  /* 0 -> set on first stage-1 call (dyn_run.f90:147) */
  int nthreads;    /* OpenMP threads, 0 -> default */
  int dcmip;       /* params.f90:62 (-1 none; 4x, 5x: DCMIP simple physics) */
} ora_config;

void ora_default_config(ora_config* c);
void* ora_create(const ora_config* c, const double* ak, const double* bk);
void ora_destroy(void* h);
int ora_nlm(void* h);

/* state I/O; spectral arrays interleaved complex, reference layout */
void ora_set_state(void* h, const double* vrt, const double* div, const double* tv,
                   const double* trc, const double* lnps, const double* topo);
void ora_get_state(void* h, double* vrt, double* div, double* tv, double* trc,
                   double* lnps);

/* transforms batched over nb 2-D fields (shtns.f90 semantics) */
void ora_spectogrd(void* h, int nb, const double* spec, double* grid);
void ora_grdtospec(void* h, int nb, const double* grid, double* spec);
void ora_getuv(void* h, int nb, const double* vrt, const double* div, double* u, double* v);
void ora_getvrtdivspec(void* h, int nb, const double* u, const double* v, double* vrt, double* div);
void ora_getgrad(void* h, int nb, const double* spec, double* gx, double* gy);

/* dynamics tendencies on the current state (dyn_run.f90:33) */
void ora_getdyntend(void* h, int rkstage, int inverse_only, double* dvrt, double* ddiv,
                    double* dtv, double* dtrc, double* dlnps);
/* nsteps calls of advance (run.f90:194) */
void ora_advance(void* h, double t, int nsteps);

/* grid field readback after the last getdyntend: name in
   ug vg vrtg divg tvg trcg dlnpdtg etadot lnpsg psg dlnpsdt prs, and the
   physics fields precip apcp pwat (phy_data.f90) */
int ora_get_grid(void* h, const char* name, double* out);
void ora_grid_info(void* h, double* lats, double* gauwts, double* areawts, int* degree,
                   int* order, double* lap, double* invlap);
/* legendre tables for order m: P,H [nlat/2][ntrunc-m+1] */
void ora_legendre(void* h, int m, double* P, double* H);
/* semi-implicit matrices: amhyb,bmhyb [nlev][nlev] row-major (row k, col j),
   svhyb, tor_hyb [nlev], d_hyb_m [3][ntrunc+1][nlev][nlev], ym [nlev][nlev] */
void ora_semimp(void* h, double* amhyb, double* bmhyb, double* svhyb, double* tor,
                double* dhyb, double* ym);
void ora_damp(void* h, double* disspec, double* diff_prof, double* dmp_prof);
/* spdmax, psmin(hPa), psmax(hPa), pstendmean, pdryini */
void ora_diag(void* h, double* out5);
/* HS forcing tendencies from current grid state (phy_run_hs.f90:22) */
void ora_getphytend(void* h, double* dvrt, double* ddiv, double* dtv, double* dtrc, double* dlnps);
/* IAU increments [nf][...] (iau_module.f90), nf = 0 detaches; the forcing of time t;
   digital filter over 2 ntdfi steps (run.f90:58-145) and its weights */
void ora_set_iau(void* h, int nf, const double* fhrs, double delthrs, const double* vrt, const double* div,
                 const double* tv, const double* trc, const double* lnps);
void ora_getiauforcing(void* h, double t, double* dvrt, double* ddiv, double* dtv, double* dtrc, double* dlnps);
void ora_dfi(void* h, double t, int ntdfi);
void ora_dfi_weights(int ntdfi, double* w);
/* simple_physics_v5_1.f90 on ncol independent columns [ncol][n] top to
   bottom (pint [ncol][n+1]); t, q, u, v updated in place, precl out (m/s) */
void ora_simple_columns(int ncol, int n, double dtime, const double* lat, double* t, double* q, double* u, double* v,
                        const double* pmid, const double* pint, const double* ps, double* precl, int test,
                        int turbflux);

#ifdef __cplusplus
}
#endif
#endif
