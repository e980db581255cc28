// gd_oracle.cpp -- TEST INFRASTRUCTURE ONLY (parity oracle + timed CPU
// baseline).  FP64 CPU restatement of the GFS spectral dycore time step of
// jswhit/gfs-dycore.  Each routine cites the reference file:line it follows.
//
// Parity status: pinned by analytic known-answer tests and scipy LAPACK
// (see gd_oracle.h); the reference's own Fortran build is not runnable here.
//
// Precision: the reference compiled with default_real=2 (src/kinds.f90:100).
// Fortran literals without a kind suffix are default REAL (single), so
// constants such as 287.05 or 1./3. carry their float-rounded values into
// the double-precision build; FLIT() reproduces that.
#include "gd_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cplx;
static inline double FLIT(float x) { return (double)x; }

// src/physcons.f90:17-56 (single-precision literals)
const double PI_D = 3.14159265358979323846;
const double RERTH = FLIT(6.3712e+6f);
const double GRAV = FLIT(9.80665e+0f);
const double OMEGA = FLIT(7.2921e-5f);
const double RD = FLIT(2.8705e+2f);
const double RV = FLIT(4.6150e+2f);
const double CP = FLIT(1.0046e+3f);
const double CVAP = FLIT(1.8460e+3f);
const double KAPPA = RD / CP;  // con_rocp, evaluated in r_kind
const double FVIRT = RV / RD - 1.;  // con_fvirt

// src/semimp_data.f90:74-88 (Lorenz 3-cycle + trapezoidal IMEX tableau)
const double A21 = FLIT(1.f / 3.f), A31 = FLIT(1.f / 6.f), A32 = FLIT(1.f / 2.f);
const double AA21 = FLIT(1.f / 6.f), AA22 = FLIT(1.f / 6.f), AA31 = FLIT(1.f / 3.f);
const double AA32 = 0.0, AA33 = FLIT(1.f / 3.f);
const double B1 = FLIT(1.f / 2.f), B2 = FLIT(-1.f / 2.f), B3 = 1.0;
const double BB1 = FLIT(3.f / 8.f), BB2 = 0.0, BB3 = FLIT(3.f / 8.f), BB4 = FLIT(1.f / 4.f);
const double REF_TEMP = 300.0, REF_PRESS = 800.e2;  // semimp_data.f90:122-123
const double LOG2_SP = FLIT(logf(2.f));             // log(2.) in single precision

// ---------------------------------------------------------------------------
// Complex Stockham FFT (radices 4, 2, 3) of length M, used through the
// half-length trick for the real transforms of length nlon = 2M.  Role of
// FFTW inside SHTns (not vendored).
struct Fft {
  int n = 0;  // real length nlon
  int M = 0;  // complex length nlon/2
  std::vector<int> rad;
  std::vector<cplx> twM;  // exp(-2 pi i k / M)
  std::vector<cplx> twN;  // exp(-2 pi i k / nlon), k <= M
  void init(int n_) {
    n = n_;
    M = n / 2;
    int r = M;
    rad.clear();
    while (r % 4 == 0) rad.push_back(4), r /= 4;
    while (r % 2 == 0) rad.push_back(2), r /= 2;
    while (r % 3 == 0) rad.push_back(3), r /= 3;
    if (r != 1 || n % 2) fprintf(stderr, "oracle fft: nlon must be 2^a 3^b\n");
    twM.resize(M);
    for (int k = 0; k < M; ++k) twM[k] = cplx(cos(2 * PI_D * k / M), -sin(2 * PI_D * k / M));
    twN.resize(M + 1);
    for (int k = 0; k <= M; ++k) twN[k] = cplx(cos(2 * PI_D * k / n), -sin(2 * PI_D * k / n));
  }
  // in-place length-M transform, sign -1 forward, +1 inverse (unnormalised);
  // b is scratch of length M
  void cfft(cplx* a, cplx* b, int sign) const {
    int Ns = 1;
    cplx* x = a;
    cplx* y = b;
    for (int p : rad) {
      const int nb = M / p, tstep = M / (Ns * p);
      const cplx w3 = cplx(-0.5, sign * 0.86602540378443864676);
      for (int jj = 0; jj < nb; ++jj) {
        const int k = jj % Ns;
        cplx v[4];
        for (int q = 0; q < p; ++q) {
          cplx t = x[jj + q * nb];
          if (q > 0 && k > 0) {
            cplx w = twM[k * q * tstep];
            if (sign > 0) w = std::conj(w);
            t *= w;
          }
          v[q] = t;
        }
        if (p == 2) {
          cplx t = v[0];
          v[0] = t + v[1];
          v[1] = t - v[1];
        } else if (p == 4) {
          cplx s02 = v[0] + v[2], d02 = v[0] - v[2], s13 = v[1] + v[3], d13 = v[1] - v[3];
          cplx id13 = cplx(-sign * d13.imag(), sign * d13.real());
          v[0] = s02 + s13;
          v[2] = s02 - s13;
          v[1] = d02 + id13;
          v[3] = d02 - id13;
        } else {
          cplx y0 = v[0] + v[1] + v[2];
          cplx y1 = v[0] + w3 * v[1] + w3 * w3 * v[2];
          cplx y2 = v[0] + w3 * w3 * v[1] + w3 * v[2];
          v[0] = y0;
          v[1] = y1;
          v[2] = y2;
        }
        const int od = (jj / Ns) * Ns * p + k;
        for (int q = 0; q < p; ++q) y[od + q * Ns] = v[q];
      }
      std::swap(x, y);
      Ns *= p;
    }
    if (x != a) std::copy(x, x + M, a);
  }
  // out[i] = Re X0 + 2 Re sum_{k=1..T} X[k] exp(+2 pi i k i / n)
  void c2r(const cplx* X, int T, double* out, cplx* z, cplx* tmp) const {
    for (int k = 0; k < M; ++k) {
      cplx xk = (k <= T) ? X[k] : cplx(0, 0);
      if (k == 0) xk = cplx(xk.real(), 0.0);
      cplx xm = (k == 0 || M - k > T) ? cplx(0, 0) : std::conj(X[M - k]);
      cplx A = xk + xm, B = xk - xm;
      z[k] = A + cplx(0, 1) * B * std::conj(twN[k]);
    }
    cfft(z, tmp, +1);
    for (int k = 0; k < M; ++k) {
      out[2 * k] = z[k].real();
      out[2 * k + 1] = z[k].imag();
    }
  }
  // X[k] = sum_i g[i] exp(-2 pi i k i / n), k = 0..T
  void r2c(const double* g, int T, cplx* X, cplx* z, cplx* tmp) const {
    for (int k = 0; k < M; ++k) z[k] = cplx(g[2 * k], g[2 * k + 1]);
    cfft(z, tmp, -1);
    for (int k = 0; k <= T; ++k) {
      cplx zk = z[k], zm = std::conj(z[(M - k) % M]);
      cplx E = zk + zm, O = zk - zm;
      cplx Oi = cplx(O.imag(), -O.real());
      X[k] = 0.5 * (E + twN[k] * Oi);
    }
  }
};

// ---------------------------------------------------------------------------
// Gaussian-grid spherical harmonic transforms with the shtns.f90 contract:
// orthonormal harmonics without Condon-Shortley phase (shtns.f90:110),
// triangular truncation, m-major coefficient order (shtns.f90:149-150),
// real fields (m>0 coefficients stand for the +m/-m pair), latitudes north
// to south (shtns.f90:125-130), exact Gauss-Legendre quadrature (no polar
// truncation: polar_opt = 0).
struct Sht {
  int T = 0, nlon = 0, nlat = 0, nh = 0, nlm = 0;
  std::vector<double> mu, w, W, lat, coslat;
  std::vector<long> moff, toff;
  std::vector<double> P, H;  // [m block][j < nh][n-m]
  Fft fft;

  long idx(int n, int m) const { return moff[m] + (n - m); }

  void init(int T_, int nlon_, int nlat_) {
    T = T_;
    nlon = nlon_;
    nlat = nlat_;
    nh = nlat / 2;
    nlm = (T + 1) * (T + 2) / 2;  // shtns.f90:116
    moff.resize(T + 2);
    toff.resize(T + 2);
    moff[0] = 0;
    toff[0] = 0;
    for (int m = 0; m <= T; ++m) {
      moff[m + 1] = moff[m] + (T - m + 1);
      toff[m + 1] = toff[m] + (long)(T - m + 1) * nh;
    }
    gauss();
    tables();
    fft.init(nlon);
  }

  // Gauss-Legendre nodes by Newton iteration on P_nlat (role of
  // shtns_cos_array / shtns_gauss_wts, shtns.f90:125-126).
  void gauss() {
    mu.assign(nlat, 0);
    w.assign(nlat, 0);
    W.assign(nlat, 0);
    lat.assign(nlat, 0);
    coslat.assign(nlat, 0);
    const int N = nlat;
    for (int j = 0; j < nh; ++j) {
      double x = cos(PI_D * (j + 0.75) / (N + 0.5));
      double dp = 0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = x;
        for (int k = 1; k < N; ++k) {
          double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
          p0 = p1;
          p1 = p2;
        }
        dp = N * (x * p1 - p0) / (x * x - 1.0);
        double dx = p1 / dp;
        x -= dx;
        if (fabs(dx) <= 1e-16) break;
      }
      {
        double p0 = 1.0, p1 = x;
        for (int k = 1; k < N; ++k) {
          double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
          p0 = p1;
          p1 = p2;
        }
        dp = N * (x * p1 - p0) / (x * x - 1.0);
      }
      double wj = 2.0 / ((1.0 - x) * (1.0 + x) * dp * dp);
      mu[j] = x;
      mu[N - 1 - j] = -x;
      w[j] = w[N - 1 - j] = wj;
    }
    for (int j = 0; j < N; ++j) {
      W[j] = 2 * PI_D * w[j];
      lat[j] = asin(mu[j]);
      coslat[j] = sqrt((1.0 - mu[j]) * (1.0 + mu[j]));
    }
  }

  // Normalised associated Legendre functions and their latitude derivative
  // by the standard three-term recurrence in n (role of SHT_GAUSS_FLY
  // recurrences), with binary exponent rescaling so high orders near the
  // poles neither underflow nor lose the recurrence.
  void tables() {
    P.assign(toff[T + 1], 0);
    H.assign(toff[T + 1], 0);
    const double inv_s2pi = 1.0 / sqrt(2 * PI_D);
    const int SC = 600;
    for (int m = 0; m <= T; ++m) {
      const int K = T - m + 1;
      for (int j = 0; j < nh; ++j) {
        const double x = mu[j], s = coslat[j];
        double v = 1.0 / sqrt(2.0);
        int c = 0;
        for (int k = 1; k <= m; ++k) {
          v *= sqrt((2.0 * k + 1.0) / (2.0 * k)) * s;
          if (fabs(v) < ldexp(1.0, -SC)) {
            v = ldexp(v, SC);
            ++c;
          }
        }
        double pm1 = 0.0, p = v;  // scaled p_{n-1}, p_n
        double* Pr = &P[toff[m] + (long)j * K];
        double* Hr = &H[toff[m] + (long)j * K];
        for (int n = m; n <= T; ++n) {
          if (n == m + 1) {
            double pn = sqrt(2.0 * m + 3.0) * x * p;
            pm1 = p;
            p = pn;
          } else if (n > m + 1) {
            double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
            double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
            double pn = a * (x * p - b * pm1);
            pm1 = p;
            p = pn;
          }
          if (c > 0 && fabs(p) > ldexp(1.0, 300)) {
            p = ldexp(p, -SC);
            pm1 = ldexp(pm1, -SC);
            --c;
          }
          double cnm = (n > m) ? sqrt(((double)n * n - (double)m * m) * (2.0 * n + 1.0) / (2.0 * n - 1.0)) : 0.0;
          double h = (-n * x * p + cnm * pm1) / s;
          double pv = (c == 0) ? p : ldexp(p, -SC * c);
          double hv = (c == 0) ? h : ldexp(h, -SC * c);
          Pr[n - m] = pv * inv_s2pi;
          Hr[n - m] = hv * inv_s2pi;
        }
      }
    }
  }

  // ----- Legendre stage -----
  // F[m*nlat + j] = sum_n T_nm(mu_j) a_nm, T = P (useH=false) or dP/dphi.
  void synth(const cplx* a, cplx* F, bool useH) const {
    for (int m = 0; m <= T; ++m) {
      const int K = T - m + 1;
      const double* tab = useH ? &H[toff[m]] : &P[toff[m]];
      const cplx* am = a + moff[m];
      for (int j = 0; j < nh; ++j) {
        const double* r = tab + (long)j * K;
        cplx e = 0, o = 0;
        for (int q = 0; q < K; q += 2) e += r[q] * am[q];
        for (int q = 1; q < K; q += 2) o += r[q] * am[q];
        // parity about the equator: P(-mu) = (-1)^(n-m) P(mu); dP/dphi has
        // the opposite parity.
        if (!useH) {
          F[(long)m * nlat + j] = e + o;
          F[(long)m * nlat + nlat - 1 - j] = e - o;
        } else {
          F[(long)m * nlat + j] = e + o;
          F[(long)m * nlat + nlat - 1 - j] = -e + o;
        }
      }
    }
  }
  // a_nm = sum_j W_j T_nm(mu_j) G[m*nlat + j]
  void anal(const cplx* G, cplx* a, bool useH) const {
    for (int m = 0; m <= T; ++m) {
      const int K = T - m + 1;
      const double* tab = useH ? &H[toff[m]] : &P[toff[m]];
      cplx* am = a + moff[m];
      for (int q = 0; q < K; ++q) am[q] = 0;
      for (int j = 0; j < nh; ++j) {
        const double* r = tab + (long)j * K;
        cplx gn = W[j] * G[(long)m * nlat + j], gs = W[nlat - 1 - j] * G[(long)m * nlat + nlat - 1 - j];
        cplx ge = useH ? gn - gs : gn + gs;  // n-m even
        cplx go = useH ? gn + gs : gn - gs;  // n-m odd
        for (int q = 0; q < K; q += 2) am[q] += r[q] * ge;
        for (int q = 1; q < K; q += 2) am[q] += r[q] * go;
      }
    }
  }
  // multiply Fourier coefficient rows by i m / cos(lat)
  void imcos(cplx* F, double scale) const {
    for (int m = 0; m <= T; ++m)
      for (int j = 0; j < nlat; ++j) F[(long)m * nlat + j] *= cplx(0.0, m * scale / coslat[j]);
  }

  // ----- longitude stage -----
  // grid[j][i] = Re F_0 + 2 Re sum_{m=1..T} F_m exp(i m lambda_i)
  void f2g(const cplx* F, double* g) const {
    std::vector<cplx> X(T + 1), z(fft.M), tmp(fft.M);
    for (int j = 0; j < nlat; ++j) {
      for (int m = 0; m <= T; ++m) X[m] = F[(long)m * nlat + j];
      fft.c2r(X.data(), T, g + (long)j * nlon, z.data(), tmp.data());
    }
  }
  // F_m(j) = (1/nlon) sum_i g[j][i] exp(-i m lambda_i)
  void g2f(const double* g, cplx* F) const {
    std::vector<cplx> X(T + 1), z(fft.M), tmp(fft.M);
    for (int j = 0; j < nlat; ++j) {
      fft.r2c(g + (long)j * nlon, T, X.data(), z.data(), tmp.data());
      for (int m = 0; m <= T; ++m) F[(long)m * nlat + j] = X[m] / (double)nlon;
    }
  }

  // ----- shtns.f90 API (one 2-D field) -----
  long nf() const { return (long)(T + 1) * nlat; }
  void spectogrd(const cplx* a, double* g) const {  // shtns.f90:203-231
    std::vector<cplx> F(nf());
    synth(a, F.data(), false);
    f2g(F.data(), g);
  }
  void grdtospec(const double* g, cplx* a) const {  // shtns.f90:171-201
    std::vector<cplx> F(nf());
    g2f(g, F.data());
    anal(F.data(), a, false);
  }
  // u = (1/a)(-dPsi/dphi + 1/cos dChi/dlambda), v = (1/a)(1/cos dPsi/dlambda + dChi/dphi)
  // with Psi = a^2 invlap vrt, Chi = a^2 invlap div (shtns.f90:233-273).
  void getuv(const cplx* vrt, const cplx* div, double* u, double* v, double rs) const {
    std::vector<cplx> s(nlm), c(nlm), F1(nf()), F2(nf()), U(nf()), V(nf());
    for (int m = 0; m <= T; ++m)
      for (int n = m; n <= T; ++n) {
        long k = idx(n, m);
        double il = (n == 0) ? 0.0 : 1.0 / (-(double)n * (n + 1.0));
        s[k] = il * rs * vrt[k];
        c[k] = il * rs * div[k];
      }
    synth(s.data(), F1.data(), true);  // H s
    synth(c.data(), F2.data(), false);  // P c
    imcos(F2.data(), 1.0);
    for (long q = 0; q < nf(); ++q) U[q] = -F1[q] + F2[q];
    synth(s.data(), F1.data(), false);  // P s
    imcos(F1.data(), 1.0);
    synth(c.data(), F2.data(), true);  // H c
    for (long q = 0; q < nf(); ++q) V[q] = F1[q] + F2[q];
    f2g(U.data(), u);
    f2g(V.data(), v);
  }
  // (vrt,div) of (u,v) (shtns.f90:275-311)
  void getvrtdivspec(const double* u, const double* v, cplx* vrt, cplx* div, double rs) const {
    std::vector<cplx> U(nf()), V(nf()), t(nf()), a1(nlm), a2(nlm);
    g2f(u, U.data());
    g2f(v, V.data());
    // vrt = (1/a)[ P^T (i m/cos V) + H^T U ]
    t = V;
    imcos(t.data(), 1.0);
    anal(t.data(), a1.data(), false);
    anal(U.data(), a2.data(), true);
    for (int k = 0; k < nlm; ++k) vrt[k] = (a1[k] + a2[k]) / rs;
    // div = (1/a)[ P^T (i m/cos U) - H^T V ]
    t = U;
    imcos(t.data(), 1.0);
    anal(t.data(), a1.data(), false);
    anal(V.data(), a2.data(), true);
    for (int k = 0; k < nlm; ++k) div[k] = (a1[k] - a2[k]) / rs;
  }
  // gradient (1/(a cos) df/dlambda, (1/a) df/dphi) (shtns.f90:313-352)
  void getgrad(const cplx* f, double* gx, double* gy, double rs) const {
    std::vector<cplx> F(nf());
    synth(f, F.data(), false);
    imcos(F.data(), 1.0);
    for (auto& z : F) z /= rs;
    f2g(F.data(), gx);
    synth(f, F.data(), true);
    for (auto& z : F) z /= rs;
    f2g(F.data(), gy);
  }
};

// LU with partial pivoting + inverse (role of LAPACK dgetrf/dgetri,
// semimp_data.f90:248-249).  a is row-major n x n, replaced by inv(a).
void invert(std::vector<double>& a, int n) {
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(a[(long)i * n + k]) > fabs(a[(long)p * n + k])) p = i;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[(long)k * n + j], a[(long)p * n + j]);
    double d = a[(long)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double l = a[(long)i * n + k] / d;
      a[(long)i * n + k] = l;
      for (int j = k + 1; j < n; ++j) a[(long)i * n + j] -= l * a[(long)k * n + j];
    }
  }
  // inv(A) = inv(U) inv(L) P
  std::vector<double> inv((long)n * n, 0.0), col(n);
  for (int c = 0; c < n; ++c) {
    // solve A x = e_c via P, L, U
    for (int i = 0; i < n; ++i) col[i] = (i == c) ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k) std::swap(col[k], col[piv[k]]);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) col[i] -= a[(long)i * n + k] * col[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) col[i] -= a[(long)i * n + k] * col[k];
      col[i] /= a[(long)i * n + i];
    }
    for (int i = 0; i < n; ++i) inv[(long)i * n + c] = col[i];
  }
  a.swap(inv);
}

extern "C" {
void ora_pattern_advance(void* h, int nsteps);
void ora_pattern_get(void* h, double* out);
int ora_pattern_jcap(void* h);
}

// x**n for an integer n, as Fortran evaluates an integer power
double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// DCMIP simple physics for one column (src/simple_physics_v5_1.f90:1-462,
// Reed and Jablonowski 2012): large-scale condensation, then with turbflux
// the implicit surface fluxes of momentum, heat and moisture at the lowest
// level and the implicit boundary-layer diffusion (a tridiagonal solve per
// variable, eliminated bottom up and substituted top down).  Arrays are top
// (0) to bottom (n-1); pint has n+1 interfaces.  All arithmetic in double,
// the constants are the routine's own.  w holds 12 (n+1) scratch values.
void simple_column(int n, double dtime, double lat, double* t, double* q, double* u, double* v, const double* pmid,
                   const double* pint, const double* pdel, const double* rpdel, double ps, double* precl, int test,
                   bool turbflux, double* w) {
  const double gravit = 9.80616, rair = 287.0, cpair = 1.0045e3, latvap = 2.5e6, rh2o = 461.5;
  const double epsilo = rair / rh2o, zvir = (rh2o / rair) - 1.0, a = 6371220.0, omega = 7.29212e-5;
  const double pi = 4.0 * atan(1.0);
  const double C = 0.0011, SST_tc = 302.15, T0 = 273.16, e0 = 610.78, rhow = 1000.0;
  const double Cd0 = 0.0007, Cd1 = 0.000065, Cm = 0.002, v20 = 20.0, p0 = 100000.0;
  const double pbltop = 85000., pblconst = 10000., T00 = 288.0, u0 = 35.0, latw = 2.0 * pi / 9.0;
  const double eta0 = 0.252, etav = (1. - eta0) * 0.5 * pi;
  const double q0 = (double)0.021f;  // a literal without a kind suffix
  const double rk = rair / cpair;
  const int nb = n - 1;  // the lowest level
  // height of the lowest level (from the state before any update)
  const double dlnpint = log(ps) - log(pint[nb]);
  const double za = rair / gravit * t[nb] * (1. + zvir * q[nb]) * 0.5 * dlnpint;
  double Tsurf;
  if (test == 1) {
    const double sl = sin(lat), cl = cos(lat);
    Tsurf = (T00 + pi * u0 / rair * 1.5 * sin(etav) * pow(cos(etav), 0.5) *
                       ((-2. * ipow(sl, 6) * (cl * cl + 1. / 3.) + 10. / 63.) * u0 * pow(cos(etav), 1.5) +
                        (8. / 5. * ipow(cl, 3) * (sl * sl + 2. / 3.) - pi / 4.) * a * omega * 0.5)) /
            (1. + zvir * q0 * exp(-ipow(lat / latw, 4)));
  } else {
    Tsurf = SST_tc;
  }
  // large-scale condensation
  *precl = 0.0;
  for (int k = 0; k < n; ++k) {
    const double qsat = epsilo * e0 / pmid[k] * exp(-latvap / rh2o * ((1. / t[k]) - 1. / T0));
    if (q[k] > qsat) {
      const double tmp =
          1. / dtime * (q[k] - qsat) / (1. + (latvap / cpair) * (epsilo * latvap * qsat / (rair * (t[k] * t[k]))));
      t[k] = t[k] + (latvap / cpair * tmp) * dtime;
      q[k] = q[k] + (-tmp) * dtime;
      *precl = *precl + tmp * pdel[k] / (gravit * rhow);
    }
  }
  if (!turbflux) return;
  double* Km = w;
  double* Ke = w + (n + 1);
  double* CA = w + 2 * (n + 1);
  double* CC = w + 3 * (n + 1);
  double* CAm = w + 4 * (n + 1);
  double* CCm = w + 5 * (n + 1);
  double* CE = w + 6 * (n + 1);
  double* CEm = w + 7 * (n + 1);
  double* CF = w + 8 * (n + 1);  // CFu, CFv, CFt, CFq interleaved by 4 (n+1 rows)
  const double wind = sqrt(u[nb] * u[nb] + v[nb] * v[nb]);
  double Cd;
  Ke[n] = C * wind * za;
  if (wind < v20) {
    Cd = Cd0 + Cd1 * wind;
    Km[n] = Cd * wind * za;
  } else {
    Cd = Cm;
    Km[n] = Cm * wind * za;
  }
  for (int k = 0; k < n; ++k) {
    if (pint[k] >= pbltop) {
      Km[k] = Km[n];
      Ke[k] = Ke[n];
    } else {
      const double x = pbltop - pint[k];
      Km[k] = Km[n] * exp(-(x * x) / (pblconst * pblconst));
      Ke[k] = Ke[n] * exp(-(x * x) / (pblconst * pblconst));
    }
  }
  // surface fluxes, implicit in the lowest level
  const double qsats = epsilo * e0 / ps * exp(-latvap / rh2o * ((1. / Tsurf) - 1. / T0));
  u[nb] = u[nb] / (1. + Cd * wind * dtime / za);
  v[nb] = v[nb] / (1. + Cd * wind * dtime / za);
  t[nb] = (t[nb] + C * wind * Tsurf * dtime / za) / (1. + C * wind * dtime / za);
  q[nb] = (q[nb] + C * wind * qsats * dtime / za) / (1. + C * wind * dtime / za);
  // boundary-layer diffusion
  for (int k = 0; k < n - 1; ++k) {
    const double rho = (pint[k + 1] / (rair * (t[k + 1] + t[k]) / 2.0));
    const double dpm = pmid[k + 1] - pmid[k];
    CAm[k] = rpdel[k] * dtime * gravit * gravit * Km[k + 1] * rho * rho / dpm;
    CCm[k + 1] = rpdel[k + 1] * dtime * gravit * gravit * Km[k + 1] * rho * rho / dpm;
    CA[k] = rpdel[k] * dtime * gravit * gravit * Ke[k + 1] * rho * rho / dpm;
    CC[k + 1] = rpdel[k + 1] * dtime * gravit * gravit * Ke[k + 1] * rho * rho / dpm;
  }
  CAm[n - 1] = 0.;
  CCm[0] = 0.;
  CEm[n] = 0.;
  CA[n - 1] = 0.;
  CC[0] = 0.;
  CE[n] = 0.;
  for (int i = 0; i < 4; ++i) CF[4 * n + i] = 0.;
  for (int k = n - 1; k >= 0; --k) {
    const double de = 1. + CA[k] + CC[k] - CA[k] * CE[k + 1];
    const double dm = 1. + CAm[k] + CCm[k] - CAm[k] * CEm[k + 1];
    CE[k] = CC[k] / de;
    CEm[k] = CCm[k] / dm;
    CF[4 * k + 0] = (u[k] + CAm[k] * CF[4 * (k + 1) + 0]) / dm;
    CF[4 * k + 1] = (v[k] + CAm[k] * CF[4 * (k + 1) + 1]) / dm;
    CF[4 * k + 2] = (pow(p0 / pmid[k], rk) * t[k] + CA[k] * CF[4 * (k + 1) + 2]) / de;
    CF[4 * k + 3] = (q[k] + CA[k] * CF[4 * (k + 1) + 3]) / de;
  }
  u[0] = CF[0];
  v[0] = CF[1];
  t[0] = CF[2] * pow(pmid[0] / p0, rk);
  q[0] = CF[3];
  for (int k = 1; k < n; ++k) {
    u[k] = CEm[k] * u[k - 1] + CF[4 * k + 0];
    v[k] = CEm[k] * v[k - 1] + CF[4 * k + 1];
    t[k] = (CE[k] * t[k - 1] * pow(p0 / pmid[k - 1], rk) + CF[4 * k + 2]) * pow(pmid[k] / p0, rk);
    q[k] = CE[k] * q[k - 1] + CF[4 * k + 3];
  }
}

struct Dycore {
  ora_config c;
  Sht sh;
  int L = 0, nt = 0, nlm = 0, nlon = 0, nlat = 0;
  long ng = 0;
  double pdryini = 0;
  // spectral state [lev][nlm] (spectral_data.f90:11-21)
  std::vector<cplx> vrt, div, tv, trc, lnps, topo;
  // grid state (grid_data.f90:11-29), [lev][nlat][nlon] bottom to top
  std::vector<double> ug, vg, vrtg, divg, tvg, trcg, dlnpdtg, etadot;
  std::vector<double> lnpsg, psg, dlnpsdt, phis, dphisdx, dphisdy, dlnpsdx, dlnpsdy;
  std::vector<double> dtvdx, dtvdy;
  // pressure_data.f90:276-296 (1-D top to bottom, prs bottom to top)
  std::vector<double> ak, bk, dbk, bkl, ck, si, sl;
  std::vector<double> pk, dpk, alfa, rlnp, prs;
  // semimp_data.f90:14-17
  std::vector<double> amhyb, bmhyb, svhyb, tor, dhyb, ym;
  // spectral_data.f90:18 damping
  std::vector<double> disspec, diff_prof, dmp_prof;
  std::vector<double> lapv, invlapv;
  std::vector<int> degree, order;
  // phy_data.f90: instantaneous precipitation (mm/s), accumulated (mm),
  // precipitable water (kg/m^2)
  std::vector<double> precip, apcp, pwat;

  long G(int k) const { return (long)k * ng; }

  void init(const ora_config& cfg, const double* ak_, const double* bk_) {
    c = cfg;
#ifdef _OPENMP
    if (c.nthreads > 0) omp_set_num_threads(c.nthreads);
#endif
    L = c.nlev;
    nt = c.ntrac;
    nlon = c.nlon;
    nlat = c.nlat;
    ng = (long)nlon * nlat;
    sh.init(c.ntrunc, nlon, nlat);
    nlm = sh.nlm;
    pdryini = c.pdryini;
    vrt.assign((long)L * nlm, 0);
    div = tv = vrt;
    trc.assign((long)nt * L * nlm, 0);
    lnps.assign(nlm, 0);
    topo.assign(nlm, 0);
    ug.assign((long)L * ng, 0);
    vg = vrtg = divg = tvg = dlnpdtg = dtvdx = dtvdy = ug;
    trcg.assign((long)nt * L * ng, 0);
    etadot.assign((long)(L + 1) * ng, 0);
    lnpsg.assign(ng, 0);
    psg = dlnpsdt = phis = dphisdx = dphisdy = dlnpsdx = dlnpsdy = lnpsg;
    precip = apcp = pwat = lnpsg;
    ak.assign(ak_, ak_ + L + 1);
    bk.assign(bk_, bk_ + L + 1);
    dbk.resize(L);
    bkl.resize(L);
    ck.resize(L);
    for (int k = 0; k < L; ++k) {  // dyn_init.f90:57-61
      dbk[k] = bk[k + 1] - bk[k];
      bkl[k] = 0.5 * (bk[k + 1] + bk[k]);
      ck[k] = ak[k + 1] * bk[k] - ak[k] * bk[k + 1];
    }
    si.resize(L + 1);
    sl.resize(L);
    pk.assign((long)(L + 1) * ng, 0);
    dpk.assign((long)L * ng, 0);
    alfa = rlnp = prs = dpk;
    degree.resize(nlm);
    order.resize(nlm);
    lapv.resize(nlm);
    invlapv.resize(nlm);
    for (int m = 0, k = 0; m <= c.ntrunc; ++m)  // shtns.f90:149-155
      for (int n = m; n <= c.ntrunc; ++n, ++k) {
        degree[k] = n;
        order[k] = m;
        lapv[k] = -(double)n * (n + 1.0);
        invlapv[k] = (k == 0) ? 0.0 : 1.0 / lapv[k];
      }
    sigma_levels();
    setdampspec();
    if (!c.explicit_) init_semimp();
  }

  // sigma levels as in calc_pressdata (pressure_data.f90:58-65)
  void sigma_levels() {
    for (int k = 0; k <= L; ++k) si[L - k] = ak[k] / 101300.0 + bk[k];
    for (int k = 0; k < L; ++k) sl[k] = 0.5 * (si[k] + si[k + 1]);
  }

  // dyn_init.f90:450-494
  void setdampspec() {
    int ndiss = c.ndiss == 0 ? 8 : c.ndiss;
    double efold = c.efold, fshk = c.fshk;
    const int T = c.ntrunc;
    if (efold <= 0) {
      if (T > 170) {
        float x = (float)T / 170.f;
        float x4 = (x * x) * (x * x);
        efold = 3600. / (c.hdif_fac2 * (double)x4 * FLIT(1.1f));
      } else if (T == 126 || T == 170) {
        efold = 1. / (c.hdif_fac2 * FLIT(12.E15f) / pow(RERTH, 4) * 41990400.0);
      } else {
        efold = 1. / (c.hdif_fac2 * FLIT(3.E15f) / pow(RERTH, 4) * 41990400.0);
      }
      efold = 2. * efold;
    }
    if (fshk <= 0) {
      fshk = 1.0 * c.hdif_fac;
      if (T > 170) fshk = FLIT(2.2f) * c.hdif_fac;
      if (T == 126) fshk = FLIT(1.5f) * c.hdif_fac;
    }
    double slrd0 = FLIT(0.002f);
    double dmp_prof1 = 1. / c.taustratdamp;
    diff_prof.resize(L);
    dmp_prof.assign(L, 0.0);
    for (int k = 0; k < L; ++k) {
      diff_prof[k] = pow(sl[k], log(1. / fshk));
      if (sl[k] < slrd0) dmp_prof[k] = dmp_prof1 * log(slrd0 / sl[k]);
    }
    double minlap = *std::min_element(lapv.begin(), lapv.end());
    disspec.resize(nlm);
    for (int k = 0; k < nlm; ++k) {
      double r = lapv[k] / minlap, rp = 1.0;
      for (int q = 0; q < ndiss / 2; ++q) rp *= r;
      disspec[k] = -(1. / efold) * rp;
    }
  }

  // semimp_data.f90:127-256
  void init_semimp() {
    std::vector<double> pkref(L + 1), dpkref(L), alfaref(L), yecm((long)L * L, 0), tecm((long)L * L, 0), vecm(L);
    for (int k = 0; k <= L; ++k) pkref[k] = ak[k] + bk[k] * REF_PRESS;
    for (int k = 0; k < L; ++k) dpkref[k] = pkref[k + 1] - pkref[k];
    alfaref[0] = LOG2_SP;
    for (int k = 1; k < L; ++k) alfaref[k] = 1. - (pkref[k] / dpkref[k]) * log(pkref[k + 1] / pkref[k]);
    for (int i = 0; i < L; ++i) {
      yecm[(long)i * L + i] = alfaref[i] * RD;
      for (int j = i + 1; j < L; ++j) yecm[(long)i * L + j] = RD * log(pkref[j + 1] / pkref[j]);
    }
    for (int i = 0; i < L; ++i) {
      tecm[(long)i * L + i] = KAPPA * REF_TEMP * alfaref[i];
      for (int j = 0; j < i; ++j)
        tecm[(long)i * L + j] = (KAPPA * REF_TEMP * dpkref[j] / dpkref[i]) * log(pkref[i + 1] / pkref[i]);
    }
    for (int k = 0; k < L; ++k) vecm[k] = dpkref[k] / REF_PRESS;
    amhyb.assign((long)L * L, 0);
    bmhyb.assign((long)L * L, 0);
    svhyb.resize(L);
    tor.resize(L);
    for (int j = 0; j < L; ++j) {
      svhyb[j] = vecm[L - 1 - j];
      for (int k = 0; k < L; ++k) {
        amhyb[(long)k * L + j] = yecm[(long)(L - 1 - k) * L + (L - 1 - j)];
        bmhyb[(long)k * L + j] = tecm[(long)(L - 1 - k) * L + (L - 1 - j)];
      }
    }
    const double a2 = RERTH * RERTH;
    for (auto& x : amhyb) x /= a2;
    for (int k = 0; k < L; ++k) tor[k] = RD * REF_TEMP / a2;
    ym.assign((long)L * L, 0);
    for (int i = 0; i < L; ++i) {
      for (int j = 0; j < L; ++j) ym[(long)i * L + j] = tor[i] * svhyb[j];
      for (int k = 0; k < L; ++k)
        for (int j = 0; j < L; ++j) ym[(long)i * L + j] += amhyb[(long)i * L + k] * bmhyb[(long)k * L + j];
    }
    const int T = c.ntrunc;
    dhyb.assign((long)3 * (T + 1) * L * L, 0);
    const double consts[3] = {AA22, AA33, BB4};
    for (int s = 0; s < 3; ++s) {
      for (int n = 0; n <= T; ++n) {
        double rnn1 = (double)n * (n + 1);
        std::vector<double> y((long)L * L);
        double f = (consts[s] * c.dt) * (consts[s] * c.dt) * rnn1;
        for (int i = 0; i < L; ++i)
          for (int j = 0; j < L; ++j) y[(long)i * L + j] = (i == j ? 1.0 : 0.0) + f * ym[(long)i * L + j];
        invert(y, L);
        std::copy(y.begin(), y.end(), dhyb.begin() + ((long)s * (T + 1) + n) * L * L);
      }
    }
  }

  // pressure_data.f90:58-100
  void calc_pressdata() {
    const double rk = KAPPA;
#pragma omp parallel for
    for (long p = 0; p < ng; ++p) {
      psg[p] = exp(lnpsg[p]);
      for (int k = 0; k <= L; ++k) pk[G(k) + p] = ak[k] + bk[k] * psg[p];
      for (int k = 0; k < L; ++k) {
        double a = pk[G(k + 1) + p], b = pk[G(k) + p];
        dpk[G(k) + p] = a - b;
        prs[G(L - 1 - k) + p] = pow((pow(a, rk) * a - pow(b, rk) * b) / ((rk + 1.) * dpk[G(k) + p]), 1. / rk);
      }
      alfa[p] = LOG2_SP;
      rlnp[p] = FLIT(99999.99f);
      for (int k = 1; k < L; ++k) {
        rlnp[G(k) + p] = log(pk[G(k + 1) + p] / pk[G(k) + p]);
        alfa[G(k) + p] = 1. - (pk[G(k) + p] / dpk[G(k) + p]) * rlnp[G(k) + p];
      }
    }
  }

  // dyn_run.f90:307-373 (one column p); arrays indexed as in the reference
  void getomega_col(long p, std::vector<double>& cg, std::vector<double>& cb, std::vector<double>& db,
                    std::vector<double>& wb, std::vector<double>& wc) {
    const double ps = psg[p];
    for (int k = 0; k < L; ++k)
      cg[k] = ug[G(L - 1 - k) + p] * dlnpsdx[p] + vg[G(L - 1 - k) + p] * dlnpsdy[p];
    db[0] = divg[G(L - 1) + p] * dpk[G(0) + p];
    cb[0] = cg[0] * dbk[0];
    for (int k = 0; k < L - 1; ++k) {
      db[k + 1] = db[k] + divg[G(L - 2 - k) + p] * dpk[G(k + 1) + p];
      cb[k + 1] = cb[k] + cg[k + 1] * dbk[k + 1];
    }
    dlnpsdt[p] = -db[L - 1] / ps - cb[L - 1];
    etadot[G(0) + p] = 0.;
    etadot[G(L) + p] = 0.;
    for (int k = 0; k < L - 1; ++k) etadot[G(k + 1) + p] = -ps * (bk[k + 1] * dlnpsdt[p] + cb[k]) - db[k];
    wb[0] = alfa[G(0) + p] * (divg[G(L - 1) + p] * dpk[G(0) + p] + ps * cb[0] * dbk[0]);
    for (int k = 1; k < L; ++k)
      wb[k] = rlnp[G(k) + p] * (db[k - 1] + ps * cb[k - 1]) +
              alfa[G(k) + p] * (divg[G(L - 1 - k) + p] * dpk[G(k) + p] + ps * cg[k] * dbk[k]);
    wc[0] = ps * cg[0] * dbk[0];
    for (int k = 1; k < L; ++k) wc[k] = ps * cg[k] * (dbk[k] + ck[k] * rlnp[G(k) + p] / dpk[G(k) + p]);
    for (int k = 0; k < L; ++k) dlnpdtg[G(L - 1 - k) + p] = (wc[k] - wb[k]) / dpk[G(k) + p];
  }

  // dyn_run.f90:375-451 (one column)
  void getpresgrad_col(long p, double* prsgx, double* prsgy, std::vector<double>& cofa,
                       std::vector<double>& cofb, std::vector<double>& px3u, std::vector<double>& px3v) {
    const double ps = psg[p];
    cofb[0] = -(1. / dpk[G(0) + p]) * (alfa[G(0) + p] * dbk[0]);
    for (int k = 1; k < L; ++k)
      cofb[k] = -(1. / dpk[G(k) + p]) * (bk[k] * rlnp[G(k) + p] + alfa[G(k) + p] * dbk[k]);
    for (int k = 0; k < L; ++k) {
      prsgx[G(L - 1 - k) + p] = cofb[k] * RD * tvg[G(L - 1 - k) + p] * ps * dlnpsdx[p];
      prsgy[G(L - 1 - k) + p] = cofb[k] * RD * tvg[G(L - 1 - k) + p] * ps * dlnpsdy[p];
    }
    for (int k = 0; k < L; ++k) {
      double pkk = pk[G(k) + p], pk1 = pk[G(k + 1) + p], dp = dpk[G(k) + p];
      cofa[k] = -(1. / dp) * (bk[k + 1] * pkk / pk1 - bk[k] + rlnp[G(k) + p] * (bk[k] - pkk * dbk[k] / dp));
    }
    cofb[L - 1] = 0.;
    cofb[L - 2] = -RD * (bk[L] / pk[G(L) + p] - bk[L - 1] / pk[G(L - 1) + p]) * tvg[G(0) + p];
    for (int k = 2; k <= L - 1; ++k)
      cofb[L - k - 1] = cofb[L - k] - RD * (bk[L + 1 - k] / pk[G(L + 1 - k) + p] - bk[L - k] / pk[G(L - k) + p]) *
                                          tvg[G(k - 1) + p];
    px3u[L - 1] = 0.;
    px3v[L - 1] = 0.;
    px3u[L - 2] = -RD * rlnp[G(L - 1) + p] * dtvdx[G(0) + p];
    px3v[L - 2] = -RD * rlnp[G(L - 1) + p] * dtvdy[G(0) + p];
    for (int k = 2; k <= L - 1; ++k) {
      px3u[L - k - 1] = px3u[L - k] - RD * rlnp[G(L - k) + p] * dtvdx[G(k - 1) + p];
      px3v[L - k - 1] = px3v[L - k] - RD * rlnp[G(L - k) + p] * dtvdy[G(k - 1) + p];
    }
    for (int k = 0; k < L; ++k) {
      long o = G(L - 1 - k) + p;
      prsgx[o] = prsgx[o] - dphisdx[p] + cofb[k] * ps * dlnpsdx[p] + px3u[k] - RD * alfa[G(k) + p] * dtvdx[o] -
                 cofa[k] * RD * tvg[o] * ps * dlnpsdx[p];
      prsgy[o] = prsgy[o] - dphisdy[p] + cofb[k] * ps * dlnpsdy[p] + px3v[k] - RD * alfa[G(k) + p] * dtvdy[o] -
                 cofa[k] * RD * tvg[o] * ps * dlnpsdy[p];
    }
  }

  // dyn_run.f90:453-476 (one column); d and out bottom to top
  void getvadv_col(long p, const double* d, double* out) {
    auto D = [&](int k) { return d[G(k) + p]; };
    out[G(L - 1) + p] = (0.5 / dpk[G(0) + p]) * etadot[G(1) + p] * (D(L - 2) - D(L - 1));
    out[G(0) + p] = (0.5 / dpk[G(L - 1) + p]) * etadot[G(L - 1) + p] * (D(0) - D(1));
    for (int k = 2; k <= L - 1; ++k)
      out[G(L - k) + p] = (0.5 / dpk[G(k - 1) + p]) * (etadot[G(k) + p] * (D(L - k - 1) - D(L - k)) +
                                                      etadot[G(k - 1) + p] * (D(L - k) - D(L - k + 1)));
  }

  // dyn_run.f90:478-603 (one column), Thuburn flux-limited scheme
  void getvadv_tracers_col(long p, const double* d, double* out, std::vector<double>& half, std::vector<double>& dd) {
    auto D = [&](int k) { return d[G(k) + p]; };
    for (int k = 1; k <= L - 1; ++k) {
      half[k] = 0.5 * (D(L - k - 1) + D(L - k));
      dd[k] = D(L - k - 1) - D(L - k);
    }
    half[0] = D(L - 1);
    half[L] = D(0);
    if (D(L - 1) >= 0)
      dd[0] = D(L - 1) - std::max(0., 2. * D(L - 1) - D(L - 2));
    else
      dd[0] = D(L - 1) - std::min(0., 2. * D(L - 1) - D(L - 2));
    if (D(0) >= 0)
      dd[L] = std::max(0., 2. * D(0) - D(1)) - D(0);
    else
      dd[L] = std::min(0., 2. * D(0) - D(1)) - D(0);
    const double epstiny = 2.2250738585072014e-308;  // tiny(1.d0)
    for (int k = 1; k <= L - 1; ++k)
      if (fabs(dd[k]) < epstiny) dd[k] = copysign(epstiny, dd[k]);
    for (int k = 1; k <= L - 1; ++k) {
      if (etadot[G(k) + p] > 0.) {
        double phi = dd[k - 1] / dd[k];
        half[k] = D(L - k) + (phi + fabs(phi)) / (1. + fabs(phi)) * (half[k] - D(L - k));
      } else {
        double phi = dd[k + 1] / dd[k];
        half[k] = D(L - k - 1) + (phi + fabs(phi)) / (1. + fabs(phi)) * (half[k] - D(L - k - 1));
      }
    }
    for (int k = 1; k <= L; ++k)
      out[G(L - k) + p] = (1. / dpk[G(k - 1) + p]) *
                          ((half[k] * etadot[G(k) + p] - half[k - 1] * etadot[G(k - 1) + p]) +
                           (D(L - k) * (etadot[G(k - 1) + p] - etadot[G(k) + p])));
  }

  // dyn_run.f90:33-305
  void getdyntend(cplx* dvrt, cplx* ddiv, cplx* dtv, cplx* dtrc, cplx* dlnps, int rkstage, bool inverse_only) {
    const long NL = nlm;
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < L; ++k) {
      sh.getuv(&vrt[k * NL], &div[k * NL], &ug[G(k)], &vg[G(k)], RERTH);
      sh.spectogrd(&vrt[k * NL], &vrtg[G(k)]);
      sh.spectogrd(&div[k * NL], &divg[G(k)]);
      sh.spectogrd(&tv[k * NL], &tvg[G(k)]);
      if (!inverse_only) sh.getgrad(&tv[k * NL], &dtvdx[G(k)], &dtvdy[G(k)], RERTH);
      for (int q = 0; q < nt; ++q) sh.spectogrd(&trc[((long)q * L + k) * NL], &trcg[((long)q * L + k) * ng]);
    }
    sh.spectogrd(lnps.data(), lnpsg.data());
    calc_pressdata();
    if (rkstage == 1) {  // dyn_run.f90:135-153
      double pmoist = 0;
      if (!c.dry) {
        const int ntuse = c.dcmip > 0 ? 1 : nt;
        for (int k = 0; k < L; ++k)
          for (int q = 0; q < ntuse; ++q)
            for (long p = 0; p < ng; ++p)
              pmoist += areawt(p) * dpk[G(L - 1 - k) + p] * trcg[((long)q * L + k) * ng + p];
      }
      double s = 0;
      for (long p = 0; p < ng; ++p) s += areawt(p) * psg[p];
      double pdry = s - pmoist;
      if (pdryini == 0) pdryini = pdry;
    }
    sh.getgrad(lnps.data(), dlnpsdx.data(), dlnpsdy.data(), RERTH);
#pragma omp parallel
    {
      std::vector<double> a(L + 1), b(L + 1), cc(L + 1), d(L + 1), e(L + 1);
#pragma omp for
      for (long p = 0; p < ng; ++p) getomega_col(p, a, b, cc, d, e);
    }
    if (inverse_only) return;
    sh.grdtospec(dlnpsdt.data(), dlnps);
    std::vector<double> prsgx((long)L * ng), prsgy((long)L * ng), vadvu((long)L * ng), vadvv((long)L * ng),
        vadvt((long)L * ng), vadvq((long)L * ng);
#pragma omp parallel
    {
      std::vector<double> a(L + 1), b(L + 1), cc(L + 1), d(L + 1);
#pragma omp for
      for (long p = 0; p < ng; ++p) {
        getpresgrad_col(p, prsgx.data(), prsgy.data(), a, b, cc, d);
        getvadv_col(p, ug.data(), vadvu.data());
        getvadv_col(p, vg.data(), vadvv.data());
        getvadv_col(p, tvg.data(), vadvt.data());
        for (int k = 0; k < L; ++k) {  // energy conversion, dyn_run.f90:194-214
          if (nt > 0)
            vadvq[G(k) + p] = KAPPA * dlnpdtg[G(k) + p] * tvg[G(k) + p] / (1. + (CVAP / CP - 1.) * trcg[G(k) + p]);
          else
            vadvq[G(k) + p] = KAPPA * dlnpdtg[G(k) + p] * tvg[G(k) + p];
        }
      }
    }
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < L; ++k) {  // dyn_run.f90:220-272
      std::vector<double> fx(ng), fy(ng);
      std::vector<cplx> ws(NL);
      for (long p = 0; p < ng; ++p) {
        long o = G(k) + p;
        double fcor = 2. * OMEGA * sin(sh.lat[p / nlon]);
        vadvv[o] = vadvv[o] - prsgy[o];
        vadvu[o] = vadvu[o] - prsgx[o];
        fx[p] = -ug[o] * dtvdx[o] - vg[o] * dtvdy[o] - vadvt[o] + vadvq[o];
      }
      sh.grdtospec(fx.data(), &dtv[k * NL]);
      for (long p = 0; p < ng; ++p) {
        long o = G(k) + p;
        double fcor = 2. * OMEGA * sin(sh.lat[p / nlon]);
        fx[p] = ug[o] * (vrtg[o] + fcor) + vadvv[o];
        fy[p] = vg[o] * (vrtg[o] + fcor) - vadvu[o];
      }
      sh.getvrtdivspec(fx.data(), fy.data(), &ddiv[k * NL], &dvrt[k * NL], RERTH);
      for (long q = 0; q < NL; ++q) dvrt[k * NL + q] = -dvrt[k * NL + q];
      for (long p = 0; p < ng; ++p) {
        long o = G(k) + p;
        fx[p] = 0.5 * (ug[o] * ug[o] + vg[o] * vg[o]);
      }
      sh.grdtospec(fx.data(), ws.data());
      for (long q = 0; q < NL; ++q) ddiv[k * NL + q] -= (lapv[q] / (RERTH * RERTH)) * ws[q];
    }
    for (int q = 0; q < nt; ++q) {  // dyn_run.f90:279-292
      const double* qg = &trcg[(long)q * L * ng];
#pragma omp parallel
      {
        std::vector<double> h(L + 1), dd(L + 1);
#pragma omp for
        for (long p = 0; p < ng; ++p) getvadv_tracers_col(p, qg, vadvq.data(), h, dd);
      }
#pragma omp parallel for schedule(dynamic)
      for (int k = 0; k < L; ++k) {
        std::vector<double> gx(ng), gy(ng), fx(ng);
        sh.getgrad(&trc[((long)q * L + k) * NL], gx.data(), gy.data(), RERTH);
        for (long p = 0; p < ng; ++p) {
          long o = G(k) + p;
          fx[p] = -ug[o] * gx[p] - vg[o] * gy[p] - vadvq[o];
        }
        sh.grdtospec(fx.data(), &dtrc[((long)q * L + k) * NL]);
      }
    }
  }

  double areawt(long p) const {  // shtns.f90:135-139 (normalised to sum 1)
    return sh.w[p / nlon] / (2.0 * nlon);
  }

  // Stochastically perturbed physics: a pattern of the single-precision
  // generator (gd_pattern_oracle.cpp) advanced at the start of each step and
  // put on the grid with the logit transform (run.f90:277-281); the HS
  // tendencies are scaled by 1 + vfact(k) pattern (phy_run_gfs.f90:617-620)
  // with vfact from stoch_data.f90:86-94.
  void* sppt = nullptr;
  std::vector<double> spptg, vfactv;
  void set_sppt(void* pat, double sigtop, double sigbot) {
    sppt = pat;
    vfactv.assign(L, 1.0);
    for (int k = 0; k < L; ++k) {
      if (sl[k] < sigbot && sl[k] > sigtop)
        vfactv[k] = (sl[k] - sigtop) / (sigbot - sigtop);
      else if (sl[k] <= sigtop)
        vfactv[k] = 0.0;
    }
  }
  void sppt_step() {
    ora_pattern_advance(sppt, 1);
    const int pj = ora_pattern_jcap(sppt), T = c.ntrunc;
    std::vector<double> pc((size_t)(pj + 1) * (pj + 2));  // complex pairs
    ora_pattern_get(sppt, pc.data());
    std::vector<cplx> full(nlm, cplx(0, 0));
    long pi = 0, fi = 0;
    for (int m = 0; m <= T; ++m)
      for (int n = m; n <= T; ++n, ++fi)
        if (m <= pj && n <= pj) {
          full[fi] = cplx(pc[2 * pi], pc[2 * pi + 1]);
          ++pi;
        }
    spptg.assign(ng, 0.0);
    sh.spectogrd(full.data(), spptg.data());
    for (long p = 0; p < ng; ++p) spptg[p] = 2.0 / (1.0 + exp(spptg[p])) - 1.0;
  }

  // The physics plugin of the build: Held-Suarez (phy_run_hs.f90) or DCMIP
  // simple physics (phy_run_simple.f90); none gives zero tendencies.
  void getphytend(cplx* dvrt, cplx* ddiv, cplx* dtv, cplx* dtrc, cplx* dlnps) {
    if (c.heldsuarez) {
      getphytend_hs(dvrt, ddiv, dtv, dtrc, dlnps);
    } else if (c.dcmip >= 0 && !c.dry) {
      getphytend_simple(dvrt, ddiv, dtv, dtrc, dlnps, c.dt);
    } else {  // phy_run_simple.f90:178-191 (dry), or no physics
      const long NS = (long)L * nlm;
      std::fill(dvrt, dvrt + NS, cplx(0));
      std::fill(ddiv, ddiv + NS, cplx(0));
      std::fill(dtv, dtv + NS, cplx(0));
      std::fill(dtrc, dtrc + (long)nt * NS, cplx(0));
      std::fill(dlnps, dlnps + nlm, cplx(0));
      std::fill(precip.begin(), precip.end(), 0.0);
      std::fill(apcp.begin(), apcp.end(), 0.0);
      std::fill(pwat.begin(), pwat.end(), 0.0);
    }
  }

  // phy_run_simple.f90:26-176: per column, the state (Tv to T with humidity
  // clipped at qmin, levels flipped to top-down) through simple_column,
  // back to Tv; grid increments to spectral tendencies (/dtx); precip, pwat,
  // apcp.  dcmip 4x uses the latitude-dependent SST (test 1), 5x the
  // constant one; turbulent fluxes for 43 and 5x.
  void getphytend_simple(cplx* dvrt, cplx* ddiv, cplx* dtv, cplx* dtrc, cplx* dlnps, double dtx) {
    const int test = (c.dcmip / 10 == 4) ? 1 : 0;
    const bool turbflux = (c.dcmip == 43 || c.dcmip / 10 == 5);
    const double qmin = FLIT(1.e-10f);
    std::vector<double> dtdt((long)L * ng), dudt((long)L * ng), dvdt((long)L * ng), dqdt((long)L * ng);
#pragma omp parallel
    {
      std::vector<double> gt(L), gq(L), gu(L), gv(L), prsl(L), prsi(L + 1), delp(L), rdelp(L), w(12 * (L + 1));
#pragma omp for schedule(dynamic, 64)
      for (long p = 0; p < ng; ++p) {
        for (int k = 0; k < L; ++k) {  // bottom-up k, top-down L-1-k
          const long o = G(k) + p;
          const double qq = trcg[o];
          gq[L - 1 - k] = qq;
          gu[L - 1 - k] = ug[o];
          gv[L - 1 - k] = vg[o];
          gt[L - 1 - k] = tvg[o] / (1. + FVIRT * std::max(qmin, qq));
          prsl[L - 1 - k] = prs[o];
        }
        for (int t = 0; t <= L; ++t) prsi[t] = pk[(long)t * ng + p];
        for (int t = 0; t < L; ++t) {
          delp[t] = prsi[t + 1] - prsi[t];
          rdelp[t] = 1. / delp[t];
        }
        double precl = 0;
        simple_column(L, dtx, sh.lat[p / nlon], gt.data(), gq.data(), gu.data(), gv.data(), prsl.data(), prsi.data(),
                      delp.data(), rdelp.data(), psg[p], &precl, test, turbflux, w.data());
        precip[p] = precl * 1000.;
        for (int t = 0; t < L; ++t) gt[t] = gt[t] * (1. + FVIRT * std::max(qmin, gq[t]));
        double pw = 0;
        for (int k = 0; k < L; ++k) {
          const long o = G(k) + p;
          dtdt[o] = gt[L - 1 - k] - tvg[o];
          dqdt[o] = gq[L - 1 - k] - trcg[o];
          dudt[o] = gu[L - 1 - k] - ug[o];
          dvdt[o] = gv[L - 1 - k] - vg[o];
          pw += dpk[G(L - 1 - k) + p] * (dqdt[o] + trcg[o]);
        }
        pwat[p] = pw;
      }
    }
    for (long p = 0; p < ng; ++p) pwat[p] = pwat[p] / GRAV;
    const long NL = nlm, NS = (long)L * nlm;
    std::fill(dtrc, dtrc + (long)nt * NS, cplx(0));
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < L; ++k) {
      sh.grdtospec(&dtdt[G(k)], &dtv[k * NL]);
      sh.getvrtdivspec(&dudt[G(k)], &dvdt[G(k)], &dvrt[k * NL], &ddiv[k * NL], RERTH);
      sh.grdtospec(&dqdt[G(k)], &dtrc[k * NL]);
    }
    for (long q = 0; q < NL; ++q) dlnps[q] = 0;
    for (long q = 0; q < NS; ++q) {
      dtv[q] = dtv[q] / dtx;
      dvrt[q] = dvrt[q] / dtx;
      ddiv[q] = ddiv[q] / dtx;
      dtrc[q] = dtrc[q] / dtx;
    }
    for (long p = 0; p < ng; ++p) apcp[p] = apcp[p] + precip[p] * dtx;
  }

  // phy_run_hs.f90:22-84
  void getphytend_hs(cplx* dvrt, cplx* ddiv, cplx* dtv, cplx* dtrc, cplx* dlnps) {
    const double sigbot = FLIT(0.7f), delthz = 10., tempstrat = 200.;
    const double kdrag = FLIT(1.f / (1.f * 86400.f)), krada = FLIT(1.f / (40.f * 86400.f)),
                 kradb = FLIT(1.f / (4.f * 86400.f));
    const double p0 = 1.e5, deltmp = 60., expo = FLIT(2.f / 7.f);
    const long NL = nlm;
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < L; ++k) {
      std::vector<double> f1(ng), f2(ng), f3(ng);
      for (long p = 0; p < ng; ++p) {
        long o = G(k) + p;
        double la = sh.lat[p / nlon];
        double bl = prs[o] / psg[p];
        double teq = pow(prs[o] / p0, expo) *
                     (315. - deltmp * sin(la) * sin(la) - delthz * log(prs[o] / p0) * cos(la) * cos(la));
        bl = (bl - sigbot) / (1. - sigbot);
        if (bl < 0) bl = 0;
        if (teq < tempstrat) teq = tempstrat;
        double cl = cos(la);
        const double f = sppt ? 1.0 + vfactv[k] * spptg[p] : 1.0;
        f1[p] = f * ((krada + (kradb - krada) * bl * cl * cl * cl * cl) * (teq - tvg[o]));
        f2[p] = f * (-(bl * kdrag) * vrtg[o]);
        f3[p] = f * (-(bl * kdrag) * divg[o]);
      }
      sh.grdtospec(f1.data(), &dtv[k * NL]);
      sh.grdtospec(f2.data(), &dvrt[k * NL]);
      sh.grdtospec(f3.data(), &ddiv[k * NL]);
    }
    for (long q = 0; q < NL; ++q) dlnps[q] = 0;
    // dtracerspecdt is never assigned by the reference; defined here as 0.
    for (long q = 0; q < (long)nt * L * NL; ++q) dtrc[q] = 0;
  }

  // IAU (iau_module.f90): increments analysis - first guess at iau_nf times
  int iau_nf = 0;
  std::vector<double> iau_fh;
  double iau_delthrs = 6.0;
  std::vector<cplx> ivrt, idiv, itv, itrc, ilnps;  // [nf][...]
  std::vector<cplx> fvrt, fdiv, ftv, ftrc, flnps;  // the forcing of the current step
  // getiauforcing (iau_module.f90:88-135)
  void getiauforcing(double t) {
    const long NS = (long)L * nlm, NT = (long)nt * NS;
    fvrt.assign(NS, 0);
    fdiv.assign(NS, 0);
    ftv.assign(NS, 0);
    ftrc.assign(NT, 0);
    flnps.assign(nlm, 0);
    const int nf = iau_nf;
    const double dt = iau_delthrs * 3600.;
    if (t < iau_fh[0] * 3600. || t > iau_fh[nf - 1] * 3600.) return;
    auto one = [&](int n) {
      for (long q = 0; q < NS; ++q) {
        fvrt[q] = ivrt[n * NS + q] / dt;
        fdiv[q] = idiv[n * NS + q] / dt;
        ftv[q] = itv[n * NS + q] / dt;
      }
      for (long q = 0; q < NT; ++q) ftrc[q] = itrc[n * NT + q] / dt;
      for (long q = 0; q < nlm; ++q) flnps[q] = ilnps[n * nlm + q] / dt;
    };
    if (t == 3600. * iau_fh[nf - 1]) return one(nf - 1);
    if (t == 3600. * iau_fh[0]) return one(0);
    int n = 0;
    while (n < nf && !(iau_fh[n] * 3600. > t)) ++n;
    const double delt = (iau_fh[n] - (t / 3600.)) / (iau_fh[n] - iau_fh[n - 1]);
    auto mix = [&](const std::vector<cplx>& v, long sz, long q) {
      return ((1. - delt) * v[n * sz + q] + delt * v[(n - 1) * sz + q]) / dt;
    };
    for (long q = 0; q < NS; ++q) {
      fvrt[q] = mix(ivrt, NS, q);
      fdiv[q] = mix(idiv, NS, q);
      ftv[q] = mix(itv, NS, q);
    }
    for (long q = 0; q < NT; ++q) ftrc[q] = mix(itrc, NT, q);
    for (long q = 0; q < nlm; ++q) flnps[q] = mix(ilnps, nlm, q);
  }
  void add_iau(cplx* dvrt, cplx* ddiv, cplx* dtv, cplx* dtrc, cplx* dlnps) {
    if (!iau_nf) return;
    const long NS = (long)L * nlm, NT = (long)nt * NS;
    for (long q = 0; q < NS; ++q) {
      dvrt[q] += fvrt[q];
      ddiv[q] += fdiv[q];
      dtv[q] += ftv[q];
    }
    for (long q = 0; q < NT; ++q) dtrc[q] += ftrc[q];
    for (long q = 0; q < nlm; ++q) dlnps[q] += flnps[q];
  }

  // set_dfi_wts (run.f90:567-588); the angles in single precision
  static void dfi_wts(int n, double* w) {
    const float pif = acosf(-1.0f);
    double tot = 0;
    for (int k = 0; k <= 2 * n; ++k) {
      w[k] = 1.;
      const double sx = pif * (float)(k - n) / (float)n;
      const double wx = pif * (float)(k - n) / (float)(n + 1);
      if (k != n) w[k] = sin(wx) / wx * sin(sx) / sx;
      tot += w[k];
    }
    for (int k = 0; k <= 2 * n; ++k) w[k] = w[k] / tot;
  }
  // run.f90:58-145 without the file output: the state becomes the
  // Lanczos-weighted average over 2 ntdfi steps; apcp restarts (init_phydata)
  void dfi(double t, int ntdfi) {
    std::vector<double> w(2 * ntdfi + 1);
    dfi_wts(ntdfi, w.data());
    std::vector<cplx> av(vrt.size()), ad(div.size()), at(tv.size()), aq(trc.size()), al(lnps.size());
    auto acc = [&](double wk, bool first) {
      for (size_t q = 0; q < vrt.size(); ++q) {
        av[q] = first ? wk * vrt[q] : av[q] + wk * vrt[q];
        ad[q] = first ? wk * div[q] : ad[q] + wk * div[q];
        at[q] = first ? wk * tv[q] : at[q] + wk * tv[q];
      }
      for (size_t q = 0; q < trc.size(); ++q) aq[q] = first ? wk * trc[q] : aq[q] + wk * trc[q];
      for (size_t q = 0; q < lnps.size(); ++q) al[q] = first ? wk * lnps[q] : al[q] + wk * lnps[q];
    };
    acc(w[0], true);
    for (int k = 1; k <= 2 * ntdfi; ++k) {
      advance(t);
      t += c.dt;
      acc(w[k], false);
    }
    vrt = av, div = ad, tv = at, trc = aq, lnps = al;
    std::fill(apcp.begin(), apcp.end(), 0.0);
  }

  // run.f90:194-565 (the stochastic branches but SPPT are out of scope)
  void advance(double t) {
    if (sppt) sppt_step();
    if (iau_nf) getiauforcing(t);
    const long NS = (long)L * nlm, NT = (long)nt * L * nlm;
    const double dt = c.dt;
    std::vector<cplx> vrt0 = vrt, div0 = div, tv0 = tv, trc0 = trc, lnps0 = lnps;
    std::vector<cplx> dvrt0(NS), ddiv0(NS), dtv0(NS), dtrc0(NT), dlnps0(nlm);
    std::vector<cplx> dvrt1(NS), ddiv1(NS), dtv1(NS), dtrc1(NT), dlnps1(nlm);
    std::vector<cplx> dvrt2(NS), ddiv2(NS), dtv2(NS), dtrc2(NT), dlnps2(nlm);
    std::vector<cplx> ddl0(NS), dtl0(NS), dpl0(nlm), ddl1(NS), dtl1(NS), dpl1(nlm), ddl2(NS), dtl2(NS), dpl2(nlm);
    const int T = c.ntrunc;
    auto dmat = [&](int s, int n) { return &dhyb[((long)s * (T + 1) + n) * L * L]; };
    // A x for a level vector of coefficient q of a [lev][nlm] array
    auto matvec = [&](const double* A, const cplx* x, long q, cplx* y) {
      for (int k = 0; k < L; ++k) {
        cplx s = 0;
        for (int j = 0; j < L; ++j) s += A[(long)k * L + j] * x[(long)j * nlm + q];
        y[k] = s;
      }
    };
    // remove linear terms (run.f90:329-335) for coefficient q
    auto linterms = [&](long q, const cplx* tvx, const cplx* lnpsx, const cplx* divx, cplx* ddl, cplx* dtl, cplx* dpl,
                        cplx* ddivt, cplx* dtvt, cplx* dlnpst) {
      std::vector<cplx> y(L);
      matvec(amhyb.data(), tvx, q, y.data());
      for (int k = 0; k < L; ++k) {
        ddl[(long)k * nlm + q] = -lapv[q] * (y[k] + tor[k] * lnpsx[q]);
        ddivt[(long)k * nlm + q] -= ddl[(long)k * nlm + q];
      }
      matvec(bmhyb.data(), divx, q, y.data());
      for (int k = 0; k < L; ++k) {
        dtl[(long)k * nlm + q] = -y[k];
        dtvt[(long)k * nlm + q] -= dtl[(long)k * nlm + q];
      }
      cplx s = 0;
      for (int k = 0; k < L; ++k) s += svhyb[k] * divx[(long)k * nlm + q];
      dpl[q] = -s;
      dlnpst[q] -= dpl[q];
    };
    // implicit solve (run.f90:344-349) with coefficient cc and matrix set s
    auto implicit = [&](long q, double cc, int s) {
      std::vector<cplx> y(L), rhs(L);
      matvec(amhyb.data(), tv.data(), q, y.data());
      for (int k = 0; k < L; ++k) rhs[k] = div[(long)k * nlm + q] - cc * lapv[q] * dt * (y[k] + tor[k] * lnps[q]);
      const double* D = dmat(s, degree[q]);
      for (int k = 0; k < L; ++k) {
        cplx a = 0;
        for (int j = 0; j < L; ++j) a += D[(long)k * L + j] * rhs[j];
        div[(long)k * nlm + q] = a;
      }
      matvec(bmhyb.data(), div.data(), q, y.data());
      for (int k = 0; k < L; ++k) tv[(long)k * nlm + q] -= cc * dt * y[k];
      cplx sd = 0;
      for (int k = 0; k < L; ++k) sd += svhyb[k] * div[(long)k * nlm + q];
      lnps[q] -= cc * dt * sd;
    };

    // stage 1 (run.f90:294-352)
    getdyntend(dvrt0.data(), ddiv0.data(), dtv0.data(), dtrc0.data(), dlnps0.data(), 1, false);
    add_iau(dvrt0.data(), ddiv0.data(), dtv0.data(), dtrc0.data(), dlnps0.data());
    for (long q = 0; q < NS; ++q) vrt[q] = vrt0[q] + A21 * dt * dvrt0[q];
    for (long q = 0; q < NT; ++q) trc[q] = trc0[q] + A21 * dt * dtrc0[q];
    if (c.explicit_) {
      for (long q = 0; q < NS; ++q) {
        div[q] = div0[q] + A21 * dt * ddiv0[q];
        tv[q] = tv0[q] + A21 * dt * dtv0[q];
      }
      for (long q = 0; q < nlm; ++q) lnps[q] = lnps0[q] + A21 * dt * dlnps0[q];
    } else {
#pragma omp parallel for
      for (long q = 0; q < nlm; ++q) {
        linterms(q, tv0.data(), lnps0.data(), div0.data(), ddl0.data(), dtl0.data(), dpl0.data(), ddiv0.data(),
                 dtv0.data(), dlnps0.data());
        for (int k = 0; k < L; ++k) {
          long o = (long)k * nlm + q;
          div[o] = div0[o] + dt * (A21 * ddiv0[o] + AA21 * ddl0[o]);
          tv[o] = tv0[o] + dt * (A21 * dtv0[o] + AA21 * dtl0[o]);
        }
        lnps[q] = lnps0[q] + dt * (A21 * dlnps0[q] + AA21 * dpl0[q]);
        implicit(q, AA22, 0);
      }
    }
    // stage 2 (run.f90:354-418)
    getdyntend(dvrt1.data(), ddiv1.data(), dtv1.data(), dtrc1.data(), dlnps1.data(), 2, false);
    add_iau(dvrt1.data(), ddiv1.data(), dtv1.data(), dtrc1.data(), dlnps1.data());
    for (long q = 0; q < NS; ++q) vrt[q] = vrt0[q] + dt * (A31 * dvrt0[q] + A32 * dvrt1[q]);
    for (long q = 0; q < NT; ++q) trc[q] = trc0[q] + dt * (A31 * dtrc0[q] + A32 * dtrc1[q]);
    if (c.explicit_) {
      for (long q = 0; q < NS; ++q) {
        div[q] = div0[q] + dt * (A31 * ddiv0[q] + A32 * ddiv1[q]);
        tv[q] = tv0[q] + dt * (A31 * dtv0[q] + A32 * dtv1[q]);
      }
      for (long q = 0; q < nlm; ++q) lnps[q] = lnps0[q] + dt * (A31 * dlnps0[q] + A32 * dlnps1[q]);
    } else {
#pragma omp parallel for
      for (long q = 0; q < nlm; ++q) {
        linterms(q, tv.data(), lnps.data(), div.data(), ddl1.data(), dtl1.data(), dpl1.data(), ddiv1.data(),
                 dtv1.data(), dlnps1.data());
        for (int k = 0; k < L; ++k) {
          long o = (long)k * nlm + q;
          div[o] = div0[o] + dt * (A31 * ddiv0[o] + AA31 * ddl0[o] + A32 * ddiv1[o] + AA32 * ddl1[o]);
          tv[o] = tv0[o] + dt * (A31 * dtv0[o] + AA31 * dtl0[o] + A32 * dtv1[o] + AA32 * dtl1[o]);
        }
        lnps[q] = lnps0[q] + dt * (A31 * dlnps0[q] + AA31 * dpl0[q] + A32 * dlnps1[q] + AA32 * dpl1[q]);
        implicit(q, AA33, 1);
      }
    }
    // stage 3 (run.f90:420-490)
    getdyntend(dvrt2.data(), ddiv2.data(), dtv2.data(), dtrc2.data(), dlnps2.data(), 3, false);
    add_iau(dvrt2.data(), ddiv2.data(), dtv2.data(), dtrc2.data(), dlnps2.data());
    for (long q = 0; q < NS; ++q) vrt[q] = vrt0[q] + dt * (B1 * dvrt0[q] + B2 * dvrt1[q] + B3 * dvrt2[q]);
    for (long q = 0; q < NT; ++q) trc[q] = trc0[q] + dt * (B1 * dtrc0[q] + B2 * dtrc1[q] + B3 * dtrc2[q]);
    if (c.explicit_) {
      for (long q = 0; q < NS; ++q) {
        div[q] = div0[q] + dt * (B1 * ddiv0[q] + B2 * ddiv1[q] + B3 * ddiv2[q]);
        tv[q] = tv0[q] + dt * (B1 * dtv0[q] + B2 * dtv1[q] + B3 * dtv2[q]);
      }
      for (long q = 0; q < nlm; ++q) lnps[q] = lnps0[q] + dt * (B1 * dlnps0[q] + B2 * dlnps1[q] + B3 * dlnps2[q]);
    } else {
#pragma omp parallel for
      for (long q = 0; q < nlm; ++q) {
        linterms(q, tv.data(), lnps.data(), div.data(), ddl2.data(), dtl2.data(), dpl2.data(), ddiv2.data(),
                 dtv2.data(), dlnps2.data());
        for (int k = 0; k < L; ++k) {
          long o = (long)k * nlm + q;
          div[o] = div0[o] + dt * (B1 * ddiv0[o] + BB1 * ddl0[o] + B2 * ddiv1[o] + BB2 * ddl1[o] + B3 * ddiv2[o] +
                                   BB3 * ddl2[o]);
          tv[o] = tv0[o] + dt * (B1 * dtv0[o] + BB1 * dtl0[o] + B2 * dtv1[o] + BB2 * dtl1[o] + B3 * dtv2[o] +
                                 BB3 * dtl2[o]);
        }
        lnps[q] = lnps0[q] + dt * (B1 * dlnps0[q] + BB1 * dpl0[q] + B2 * dlnps1[q] + BB2 * dpl1[q] +
                                   B3 * dlnps2[q] + BB3 * dpl2[q]);
        if (fabs(BB4) > 1.e-5) implicit(q, BB4, 2);
      }
    }
    // implicit damping/diffusion (run.f90:493-501)
    for (int k = 0; k < L; ++k)
      for (long q = 0; q < nlm; ++q) {
        long o = (long)k * nlm + q;
        double fd = 1. - (disspec[q] * diff_prof[k] - dmp_prof[k]) * dt;
        double ft = 1. - disspec[q] * diff_prof[k] * dt;
        vrt[o] /= fd;
        div[o] /= fd;
        tv[o] /= ft;
        for (int s = 0; s < nt; ++s) trc[(long)s * NS + o] /= ft;
      }
    // time-split physics (run.f90:509-538)
    if (!c.adiabatic) {
      getdyntend(dvrt1.data(), ddiv1.data(), dtv1.data(), dtrc1.data(), dlnps1.data(), 3, true);
      getphytend(dvrt1.data(), ddiv1.data(), dtv1.data(), dtrc1.data(), dlnps1.data());
      for (long q = 0; q < NS; ++q) {
        vrt[q] += dt * dvrt1[q];
        div[q] += dt * ddiv1[q];
        tv[q] += dt * dtv1[q];
      }
      for (long q = 0; q < NT; ++q) trc[q] += dt * dtrc1[q];
      if (c.massfix) dry_mass_fixer(dlnps1.data(), dt);
      for (long q = 0; q < nlm; ++q) lnps[q] += dt * dlnps1[q];
    }
  }

  // dyn_run.f90:605-634 (pwat is 0 but for the moist simple physics)
  void dry_mass_fixer(cplx* dlnpsdt_, double dtx) {
    double pwatg = 0.0, pmean = 0.0;
    for (long p = 0; p < ng; ++p) pwatg += areawt(p) * pwat[p];
    for (long p = 0; p < ng; ++p) pmean += areawt(p) * psg[p];
    double pcorr = (pdryini + GRAV * pwatg) / pmean;
    std::vector<double> g(ng);
    for (long p = 0; p < ng; ++p) g[p] = log(psg[p] * pcorr);
    std::vector<cplx> ws(nlm);
    sh.grdtospec(g.data(), ws.data());
    for (long q = 0; q < nlm; ++q) dlnpsdt_[q] = (ws[q] - lnps[q]) / dtx;
  }

  // run.f90:159-161
  void diag(double* o) {
    double spd = 0, pmin = 1e300, pmax = -1e300, pt = 0;
    for (long q = 0; q < (long)L * ng; ++q) spd = std::max(spd, sqrt(ug[q] * ug[q] + vg[q] * vg[q]));
    for (long p = 0; p < ng; ++p) {
      pmin = std::min(pmin, psg[p] / 100.);
      pmax = std::max(pmax, psg[p] / 100.);
      double x = 36. * psg[p] * dlnpsdt[p];
      pt += x * x * areawt(p);
    }
    o[0] = spd;
    o[1] = pmin;
    o[2] = pmax;
    o[3] = sqrt(pt);
    o[4] = pdryini;
  }
};

inline Dycore* D(void* h) { return static_cast<Dycore*>(h); }
inline cplx* C(double* p) { return reinterpret_cast<cplx*>(p); }
inline const cplx* C(const double* p) { return reinterpret_cast<const cplx*>(p); }

}  // namespace

extern "C" {

void ora_default_config(ora_config* c) {
  memset(c, 0, sizeof(*c));
  c->ntrunc = 42;
  c->nlon = 128;
  c->nlat = 64;
  c->nlev = 20;
  c->ntrac = 0;
  c->dt = 1200.;
  c->explicit_ = 0;
  c->adiabatic = 0;
  c->heldsuarez = 1;
  c->massfix = 1;
  c->dry = 1;
  c->ndiss = 0;
  c->efold = 0;
  c->hdif_fac = 1.0;
  c->hdif_fac2 = 1.0;
  c->fshk = 0;
  c->taustratdamp = 5. * 86400.;
  c->pdryini = 0;
  c->nthreads = 0;
  c->dcmip = -1;
}

void* ora_create(const ora_config* c, const double* ak, const double* bk) {
  Dycore* d = new Dycore();
  d->init(*c, ak, bk);
  return d;
}
void ora_destroy(void* h) { delete D(h); }
int ora_nlm(void* h) { return D(h)->nlm; }

void ora_set_state(void* h, const double* vrt, const double* div, const double* tv, const double* trc,
                   const double* lnps, const double* topo) {
  Dycore* d = D(h);
  long NS = (long)d->L * d->nlm;
  std::copy(C(vrt), C(vrt) + NS, d->vrt.begin());
  std::copy(C(div), C(div) + NS, d->div.begin());
  std::copy(C(tv), C(tv) + NS, d->tv.begin());
  if (d->nt > 0 && trc) std::copy(C(trc), C(trc) + NS * d->nt, d->trc.begin());
  std::copy(C(lnps), C(lnps) + d->nlm, d->lnps.begin());
  if (topo)
    std::copy(C(topo), C(topo) + d->nlm, d->topo.begin());
  else
    std::fill(d->topo.begin(), d->topo.end(), 0);
  // dyn_init.f90:76-84: phis and its gradient from grav*topospec
  std::vector<cplx> gt(d->nlm);
  for (int q = 0; q < d->nlm; ++q) gt[q] = GRAV * d->topo[q];
  d->sh.spectogrd(gt.data(), d->phis.data());
  d->sh.getgrad(gt.data(), d->dphisdx.data(), d->dphisdy.data(), RERTH);
}
void ora_get_state(void* h, double* vrt, double* div, double* tv, double* trc, double* lnps) {
  Dycore* d = D(h);
  long NS = (long)d->L * d->nlm;
  if (vrt) std::copy(d->vrt.begin(), d->vrt.end(), C(vrt));
  if (div) std::copy(d->div.begin(), d->div.end(), C(div));
  if (tv) std::copy(d->tv.begin(), d->tv.end(), C(tv));
  if (trc && d->nt > 0) std::copy(d->trc.begin(), d->trc.begin() + NS * d->nt, C(trc));
  if (lnps) std::copy(d->lnps.begin(), d->lnps.end(), C(lnps));
}

void ora_spectogrd(void* h, int nb, const double* spec, double* grid) {
  Dycore* d = D(h);
#pragma omp parallel for
  for (int b = 0; b < nb; ++b) d->sh.spectogrd(C(spec) + (long)b * d->nlm, grid + (long)b * d->ng);
}
void ora_grdtospec(void* h, int nb, const double* grid, double* spec) {
  Dycore* d = D(h);
#pragma omp parallel for
  for (int b = 0; b < nb; ++b) d->sh.grdtospec(grid + (long)b * d->ng, C(spec) + (long)b * d->nlm);
}
void ora_getuv(void* h, int nb, const double* vrt, const double* div, double* u, double* v) {
  Dycore* d = D(h);
#pragma omp parallel for
  for (int b = 0; b < nb; ++b)
    d->sh.getuv(C(vrt) + (long)b * d->nlm, C(div) + (long)b * d->nlm, u + (long)b * d->ng, v + (long)b * d->ng,
                RERTH);
}
void ora_getvrtdivspec(void* h, int nb, const double* u, const double* v, double* vrt, double* div) {
  Dycore* d = D(h);
#pragma omp parallel for
  for (int b = 0; b < nb; ++b)
    d->sh.getvrtdivspec(u + (long)b * d->ng, v + (long)b * d->ng, C(vrt) + (long)b * d->nlm,
                        C(div) + (long)b * d->nlm, RERTH);
}
void ora_getgrad(void* h, int nb, const double* spec, double* gx, double* gy) {
  Dycore* d = D(h);
#pragma omp parallel for
  for (int b = 0; b < nb; ++b)
    d->sh.getgrad(C(spec) + (long)b * d->nlm, gx + (long)b * d->ng, gy + (long)b * d->ng, RERTH);
}

void ora_getdyntend(void* h, int rkstage, int inverse_only, double* dvrt, double* ddiv, double* dtv, double* dtrc,
                    double* dlnps) {
  Dycore* d = D(h);
  long NS = (long)d->L * d->nlm;
  std::vector<cplx> a(NS), b(NS), c(NS), e((long)d->nt * NS + 1), f(d->nlm);
  d->getdyntend(a.data(), b.data(), c.data(), e.data(), f.data(), rkstage, inverse_only != 0);
  if (inverse_only) return;
  std::copy(a.begin(), a.end(), C(dvrt));
  std::copy(b.begin(), b.end(), C(ddiv));
  std::copy(c.begin(), c.end(), C(dtv));
  if (dtrc && d->nt > 0) std::copy(e.begin(), e.begin() + (long)d->nt * NS, C(dtrc));
  std::copy(f.begin(), f.end(), C(dlnps));
}

void ora_set_sppt(void* h, void* pattern, double sigtop, double sigbot) {
  static_cast<Dycore*>(h)->set_sppt(pattern, sigtop, sigbot);
}
void ora_advance(void* h, double t, int nsteps) {
  Dycore* d = D(h);
  for (int s = 0; s < nsteps; ++s) {
    d->advance(t);
    t += d->c.dt;
  }
}

int ora_get_grid(void* h, const char* name, double* out) {
  Dycore* d = D(h);
  std::string n(name);
  const std::vector<double>* v = nullptr;
  if (n == "ug") v = &d->ug;
  else if (n == "vg") v = &d->vg;
  else if (n == "vrtg") v = &d->vrtg;
  else if (n == "divg") v = &d->divg;
  else if (n == "tvg") v = &d->tvg;
  else if (n == "trcg") v = &d->trcg;
  else if (n == "dlnpdtg") v = &d->dlnpdtg;
  else if (n == "etadot") v = &d->etadot;
  else if (n == "lnpsg") v = &d->lnpsg;
  else if (n == "psg") v = &d->psg;
  else if (n == "dlnpsdt") v = &d->dlnpsdt;
  else if (n == "prs") v = &d->prs;
  else if (n == "dphisdx") v = &d->dphisdx;
  else if (n == "dphisdy") v = &d->dphisdy;
  else if (n == "precip") v = &d->precip;
  else if (n == "apcp") v = &d->apcp;
  else if (n == "pwat") v = &d->pwat;
  if (!v) return -1;
  std::copy(v->begin(), v->end(), out);
  return 0;
}

void ora_grid_info(void* h, double* lats, double* gauwts, double* areawts, int* degree, int* order, double* lap,
                   double* invlap) {
  Dycore* d = D(h);
  for (int j = 0; j < d->nlat; ++j) {
    if (lats) lats[j] = d->sh.lat[j];
    if (gauwts) gauwts[j] = d->sh.w[j];
    if (areawts) areawts[j] = d->sh.w[j] / (2.0 * d->nlon);
  }
  for (int q = 0; q < d->nlm; ++q) {
    if (degree) degree[q] = d->degree[q];
    if (order) order[q] = d->order[q];
    if (lap) lap[q] = d->lapv[q];
    if (invlap) invlap[q] = d->invlapv[q];
  }
}

void ora_legendre(void* h, int m, double* P, double* H) {
  Dycore* d = D(h);
  long n = (long)(d->c.ntrunc - m + 1) * d->sh.nh;
  std::copy(d->sh.P.begin() + d->sh.toff[m], d->sh.P.begin() + d->sh.toff[m] + n, P);
  std::copy(d->sh.H.begin() + d->sh.toff[m], d->sh.H.begin() + d->sh.toff[m] + n, H);
}

void ora_semimp(void* h, double* amhyb, double* bmhyb, double* svhyb, double* tor, double* dhyb, double* ym) {
  Dycore* d = D(h);
  if (amhyb) std::copy(d->amhyb.begin(), d->amhyb.end(), amhyb);
  if (bmhyb) std::copy(d->bmhyb.begin(), d->bmhyb.end(), bmhyb);
  if (svhyb) std::copy(d->svhyb.begin(), d->svhyb.end(), svhyb);
  if (tor) std::copy(d->tor.begin(), d->tor.end(), tor);
  if (dhyb) std::copy(d->dhyb.begin(), d->dhyb.end(), dhyb);
  if (ym) std::copy(d->ym.begin(), d->ym.end(), ym);
}

void ora_damp(void* h, double* disspec, double* diff_prof, double* dmp_prof) {
  Dycore* d = D(h);
  if (disspec) std::copy(d->disspec.begin(), d->disspec.end(), disspec);
  if (diff_prof) std::copy(d->diff_prof.begin(), d->diff_prof.end(), diff_prof);
  if (dmp_prof) std::copy(d->dmp_prof.begin(), d->dmp_prof.end(), dmp_prof);
}

void ora_diag(void* h, double* out5) { D(h)->diag(out5); }

void ora_set_iau(void* h, int nf, const double* fhrs, double delthrs, const double* vrt, const double* div,
                 const double* tv, const double* trc, const double* lnps) {
  Dycore* d = D(h);
  d->iau_nf = nf;
  if (!nf) return;
  const long NS = (long)d->L * d->nlm, NT = (long)d->nt * NS;
  d->iau_fh.assign(fhrs, fhrs + nf);
  d->iau_delthrs = delthrs;
  d->ivrt.assign(C(vrt), C(vrt) + nf * NS);
  d->idiv.assign(C(div), C(div) + nf * NS);
  d->itv.assign(C(tv), C(tv) + nf * NS);
  d->itrc.assign(NT ? C(trc) : nullptr, NT ? C(trc) + nf * NT : nullptr);
  d->ilnps.assign(C(lnps), C(lnps) + nf * d->nlm);
}
void ora_getiauforcing(void* h, double t, double* dvrt, double* ddiv, double* dtv, double* dtrc, double* dlnps) {
  Dycore* d = D(h);
  d->getiauforcing(t);
  std::copy(d->fvrt.begin(), d->fvrt.end(), C(dvrt));
  std::copy(d->fdiv.begin(), d->fdiv.end(), C(ddiv));
  std::copy(d->ftv.begin(), d->ftv.end(), C(dtv));
  if (dtrc) std::copy(d->ftrc.begin(), d->ftrc.end(), C(dtrc));
  std::copy(d->flnps.begin(), d->flnps.end(), C(dlnps));
}
void ora_dfi(void* h, double t, int ntdfi) { D(h)->dfi(t, ntdfi); }
void ora_dfi_weights(int ntdfi, double* w) { Dycore::dfi_wts(ntdfi, w); }

void ora_simple_columns(int ncol, int n, double dtime, const double* lat, double* t, double* q, double* u, double* v,
                        const double* pmid, const double* pint, const double* ps, double* precl, int test,
                        int turbflux) {
  std::vector<double> pdel(n), rpdel(n), w(12 * (n + 1));
  for (int i = 0; i < ncol; ++i) {
    const double* pi = pint + (long)i * (n + 1);
    for (int k = 0; k < n; ++k) {
      pdel[k] = pi[k + 1] - pi[k];
      rpdel[k] = 1. / pdel[k];
    }
    const long o = (long)i * n;
    simple_column(n, dtime, lat[i], t + o, q + o, u + o, v + o, pmid + o, pi, pdel.data(), rpdel.data(), ps[i],
                  precl + i, test, turbflux != 0, w.data());
  }
}

void ora_getphytend(void* h, double* dvrt, double* ddiv, double* dtv, double* dtrc, double* dlnps) {
  Dycore* d = D(h);
  long NS = (long)d->L * d->nlm;
  std::vector<cplx> e((long)d->nt * NS + 1), f(d->nlm);
  d->getphytend(C(dvrt), C(ddiv), C(dtv), dtrc ? C(dtrc) : e.data(), dlnps ? C(dlnps) : f.data());
}

}  // extern "C"
