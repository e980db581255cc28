// gd_pattern_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle, never the
// product path): CPU restatement of the reference's stochastic pattern
// generator, src/patterngenerator.f90, and of the Mersenne twister it draws
// from, src/w3lib/mersenne_twister.f.
//
// Arithmetic is IEEE single precision throughout, as in the reference's
// default build (kinds.f90:100 default_real = 1 makes r_kind single; w3lib is
// compiled without -r8, so its `real` is single too).  Built with
// -ffp-contract=off: no fused multiply-adds.  The reference's own build uses
// -ffast-math -march=native (Makefile.conf.gfortran:6), whose contractions can
// change the last bit of single-precision intermediates; that binary cannot be
// built here (no Fortran compiler), so those bits are unpinned.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

namespace {

// ---- w3lib Mersenne twister (mersenne_twister.f:160-366) --------------------
struct MtW3 {
  static constexpr int N = 624, M = 397;
  uint32_t mt[N];
  int mti = N + 1;
  int iset = 0;
  float gset = 0.f;

  // random_setseed_t (mersenne_twister.f:282-296): the 1998 sgenrand seeding,
  // mt[i] = 69069 mt[i-1] mod 2^32; seed 0 means 4357
  void setseed(int32_t inseed) {
    const int32_t ii = inseed ? inseed : 4357;
    mti = N;
    mt[0] = (uint32_t)ii;
    for (int i = 1; i < N; ++i) mt[i] = 69069u * mt[i - 1];
    iset = 0;
    gset = 0.f;
  }
  // the MT19937 state transition (mersenne_twister.f:337-351)
  void twist() {
    auto mix = [](uint32_t hi, uint32_t lo, uint32_t far) {
      const uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
      return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    };
    int kk = 0;
    for (; kk < N - M; ++kk) mt[kk] = mix(mt[kk], mt[kk + 1], mt[kk + M]);
    for (; kk < N - 1; ++kk) mt[kk] = mix(mt[kk], mt[kk + 1], mt[kk + (M - N)]);
    mt[N - 1] = mix(mt[N - 1], mt[0], mt[M - 1]);
    mti = 0;
  }
  // tempering (mersenne_twister.f:353-357)
  static uint32_t temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  uint32_t next_word() {
    if (mti >= N) twist();
    return temper(mt[mti++]);
  }
  // the word as a default real (mersenne_twister.f:358-362): the signed word,
  // shifted by 2^32 if negative, over 2^32 - 1, which rounds to 2^32 in single
  static float to_unit(uint32_t y) {
    const int32_t s = (int32_t)y;
    const float two32 = 4294967296.0f;
    if (s < 0) return ((float)s + two32) / two32;
    return (float)s / two32;
  }
  // random_number_t
  void uniform(float* h, int n) {
    for (int j = 0; j < n; ++j) h[j] = to_unit(next_word());
  }
  // Numerical Recipes polar method (mersenne_twister.f:436-448)
  static void rgauss(float r1, float r2, float& r, float& g1, float& g2) {
    const float v1 = 2.f * r1 - 1.f, v2 = 2.f * r2 - 1.f;
    r = v1 * v1 + v2 * v2;
    if (r < 1.f) {
      const float fac = std::sqrt(-2.f * std::log(r) / r);
      g1 = v1 * fac;
      g2 = v2 * fac;
    }
  }
  // random_gauss_t (mersenne_twister.f:397-435): fill with accepted pairs in
  // the order the uniform pairs arrive; an odd count caches the second value
  void gauss(float* h, int mz) {
    if (mz <= 0) return;
    int mx = 0;
    if (iset == 1) {
      mx = 1;
      h[0] = gset;
      iset = 0;
    }
    const int my = (mz - mx) / 2 * 2 + mx;
    for (;;) {
      uniform(h + mx, my - mx);
      const int j1 = my - 2;  // the DO bounds are fixed when the loop starts
      for (int j = mx; j <= j1; j += 2) {
        float r = 1.f, g1 = 0.f, g2 = 0.f;
        rgauss(h[j], h[j + 1], r, g1, g2);
        if (r < 1.f) {
          h[mx] = g1;
          h[mx + 1] = g2;
          mx += 2;
        }
      }
      if (mx == my) break;
    }
    if (my < mz) {
      float r2[2], r = 1.f, g1 = 0.f, g2 = 0.f;
      for (;;) {
        uniform(r2, 2);
        rgauss(r2[0], r2[1], r, g1, g2);
        if (r < 1.f) break;
      }
      h[mz - 1] = g1;
      gset = g2;
      iset = 1;
    }
  }
};

typedef std::complex<float> cf;

// ---- patterngenerator.f90 ---------------------------------------------------
struct Pattern {
  int ntrunc = 0, nlm = 0, nfields = 1;
  float lengthscale = 0, tau = 0, dt = 0, phi = 0, stdev = 0, normfact = 0;
  std::vector<int> degree, order;
  std::vector<float> lap, varspectrum, varspectrum1d;
  std::vector<cf> spec;  // [nfields][nlm]
  MtW3 rs;

  // patterngenerator_init (patterngenerator.f90:33-65)
  void init(float lscale, float delt, float tscale, float sd, int iseed, int jcap, float normalization, int nf) {
    ntrunc = jcap;
    nlm = (jcap + 1) * (jcap + 2) / 2;
    nfields = nf;
    normfact = normalization;
    degree.resize(nlm);
    order.resize(nlm);
    lap.resize(nlm);
    int i = 0;
    for (int m = 0; m <= jcap; ++m)
      for (int n = m; n <= jcap; ++n, ++i) {
        degree[i] = n;
        order[i] = m;
        lap[i] = (float)(-n) * ((float)n + 1.0f);
      }
    tau = tscale;
    lengthscale = lscale;
    dt = delt;
    phi = std::exp(-delt / tscale);
    stdev = sd;
    rs.setseed(iseed);
    gaussian_spect();
    spec.assign((size_t)nfields * nlm, cf(0.f, 0.f));
  }

  // computevarspec (patterngenerator.f90:73-88)
  float computevarspec(const cf* d) const {
    float var = 0.f;
    for (int n = 0; n < nlm; ++n) {
      const cf p = d[n] * std::conj(d[n]);
      if (order[n] != 0)
        var = var + p.real();
      else
        var = var + (0.5f * d[n] * std::conj(d[n])).real();
    }
    return var / normfact;
  }

  // getvarspectrum (patterngenerator.f90:97-113)
  void getvarspectrum(const cf* d, float* vs) const {
    for (int n = 0; n <= ntrunc; ++n) vs[n] = 0.f;
    for (int n = 0; n < nlm; ++n) {
      if (order[n] != 0)
        vs[degree[n]] = vs[degree[n]] + (d[n] * std::conj(d[n])).real();
      else
        vs[degree[n]] = vs[degree[n]] + (0.5f * d[n] * std::conj(d[n])).real();
    }
    for (int n = 0; n <= ntrunc; ++n) vs[n] = vs[n] / normfact;
  }

  // gaussian_spect (patterngenerator.f90:145-177)
  void gaussian_spect() {
    const float rerth = 6.3712e+6f;  // physcons.f90:23
    varspectrum1d.resize(ntrunc + 1);
    varspectrum.resize(nlm);
    for (int n = 0; n <= ntrunc; ++n)
      varspectrum1d[n] =
          std::exp(-(lengthscale * lengthscale * ((float)n * ((float)n + 1.f)) / (4.f * (rerth * rerth))));
    for (int i = 0; i < nlm; ++i)
      varspectrum[i] = std::sqrt((float)ntrunc * std::exp(lengthscale * lengthscale * lap[i] / (4.f * (rerth * rerth))));
    std::vector<cf> noise(nlm);
    for (int n = 0; n < nlm; ++n) {
      if (order[n] != 0)
        noise[n] = cf(1.f, 1.f) / std::sqrt(2.f * (float)degree[n] + 1.f);
      else
        noise[n] = std::sqrt(2.f) / std::sqrt(2.f * (float)degree[n] + 1.f);
    }
    noise[0] = 0.f;  // no global mean
    const float nf = std::sqrt(normfact / (float)ntrunc);
    for (int n = 0; n < nlm; ++n) noise[n] = noise[n] * nf;
    for (int n = 0; n < nlm; ++n) noise[n] = varspectrum[n] * noise[n];
    const float var = computevarspec(noise.data());
    const float sv = std::sqrt(var);
    for (int n = 0; n < nlm; ++n) varspectrum[n] = varspectrum[n] / sv;
    for (int n = 0; n <= ntrunc; ++n) varspectrum1d[n] = varspectrum1d[n] / var;
  }

  // getnoise (patterngenerator.f90:115-132): white noise with unit variance
  void getnoise(cf* noise) {
    std::vector<float> noiser(2 * (size_t)nlm);
    rs.gauss(noiser.data(), 2 * nlm);
    noiser[0] = 0.f;
    noiser[nlm] = 0.f;
    for (int n = 0; n < nlm; ++n) {
      if (order[n] != 0)
        noise[n] = cf(noiser[n], noiser[n + nlm]) / std::sqrt(2.f * (float)degree[n] + 1.f);
      else
        noise[n] = std::sqrt(2.f) * noiser[n] / std::sqrt(2.f * (float)degree[n] + 1.f);
    }
    const float nf = std::sqrt(normfact / (float)ntrunc);
    for (int n = 0; n < nlm; ++n) noise[n] = noise[n] * nf;
  }

  // patterngenerator_advance (patterngenerator.f90:134-143)
  void advance_field(cf* d) {
    std::vector<cf> noise(nlm);
    getnoise(noise.data());
    const float a = stdev * std::sqrt(1.f - phi * phi);
    for (int n = 0; n < nlm; ++n) d[n] = phi * d[n] + (a * varspectrum[n]) * noise[n];
  }

  // the start of a pattern (stoch_data.f90:58, 81, 104, 124-127):
  // spec = stdev * getnoise * varspectrum, field after field
  void start() {
    for (int f = 0; f < nfields; ++f) {
      cf* d = spec.data() + (size_t)f * nlm;
      getnoise(d);
      for (int n = 0; n < nlm; ++n) d[n] = (stdev * d[n]) * varspectrum[n];
    }
  }
  // nsteps AR(1) steps, each advancing every field in turn (stoch_data.f90:138-142)
  void advance(int nsteps) {
    for (int s = 0; s < nsteps; ++s)
      for (int f = 0; f < nfields; ++f) advance_field(spec.data() + (size_t)f * nlm);
  }
};

void put(const cf* src, long n, double* out) {
  for (long i = 0; i < n; ++i) {
    out[2 * i] = src[i].real();
    out[2 * i + 1] = src[i].imag();
  }
}

}  // namespace

extern "C" {

// uniforms and Gaussians of a freshly seeded stream (random_setseed then
// random_number / random_gauss calls with the given counts, in order)
void ora_mt_uniform(int seed, int n, float* out) {
  MtW3 s;
  s.setseed(seed);
  s.uniform(out, n);
}
void ora_mt_gauss(int seed, int ncalls, const int* counts, float* out) {
  MtW3 s;
  s.setseed(seed);
  long o = 0;
  for (int c = 0; c < ncalls; ++c) {
    s.gauss(out + o, counts[c]);
    o += counts[c];
  }
}
// known answer: the twist and tempering above, seeded the standard way
// (init_genrand(5489)), must give the 10000th output the C++ standard fixes for
// std::mt19937 ([rand.predef]: 4123659995); also returns the library's value
uint32_t ora_mt_kat(uint32_t* std_value) {
  MtW3 s;
  s.mt[0] = 5489u;
  for (int i = 1; i < MtW3::N; ++i) s.mt[i] = 1812433253u * (s.mt[i - 1] ^ (s.mt[i - 1] >> 30)) + (uint32_t)i;
  s.mti = MtW3::N;
  uint32_t y = 0;
  for (int i = 0; i < 10000; ++i) y = s.next_word();
  std::mt19937 ref;
  uint32_t z = 0;
  for (int i = 0; i < 10000; ++i) z = (uint32_t)ref();
  if (std_value) *std_value = z;
  return y;
}

void* ora_pattern_create(double lscale, double delt, double tscale, double stdev, int iseed, int jcap,
                         double normalization, int nfields) {
  Pattern* p = new Pattern();
  p->init((float)lscale, (float)delt, (float)tscale, (float)stdev, iseed, jcap, (float)normalization, nfields);
  return p;
}
void ora_pattern_destroy(void* h) { delete static_cast<Pattern*>(h); }
void ora_pattern_start(void* h) { static_cast<Pattern*>(h)->start(); }
void ora_pattern_advance(void* h, int nsteps) { static_cast<Pattern*>(h)->advance(nsteps); }
void ora_pattern_get(void* h, double* out) {
  Pattern* p = static_cast<Pattern*>(h);
  put(p->spec.data(), (long)p->spec.size(), out);
}
void ora_pattern_getnoise(void* h, double* out) {
  Pattern* p = static_cast<Pattern*>(h);
  std::vector<cf> noise(p->nlm);
  p->getnoise(noise.data());
  put(noise.data(), p->nlm, out);
}
void ora_pattern_spectra(void* h, double* varspectrum, double* varspectrum1d, double* phi) {
  Pattern* p = static_cast<Pattern*>(h);
  for (int i = 0; i < p->nlm; ++i) varspectrum[i] = p->varspectrum[i];
  for (int n = 0; n <= p->ntrunc; ++n) varspectrum1d[n] = p->varspectrum1d[n];
  *phi = p->phi;
}
int ora_pattern_jcap(void* h) { return static_cast<Pattern*>(h)->ntrunc; }
double ora_pattern_varspec(void* h, int field) {
  Pattern* p = static_cast<Pattern*>(h);
  return p->computevarspec(p->spec.data() + (size_t)field * p->nlm);
}
void ora_pattern_getvarspectrum(void* h, int field, double* vs) {
  Pattern* p = static_cast<Pattern*>(h);
  std::vector<float> v(p->ntrunc + 1);
  p->getvarspectrum(p->spec.data() + (size_t)field * p->nlm, v.data());
  for (int n = 0; n <= p->ntrunc; ++n) vs[n] = v[n];
}

}  // extern "C"
