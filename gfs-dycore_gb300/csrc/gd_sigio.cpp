// gd_sigio.cpp -- GFS spectral sigma-file reader and writer (host code).
//
// The file format is the one src/sigio_module.f90 reads and writes: Fortran
// unformatted sequential records, big-endian, each framed by a 4-byte length
// before and after it (sigio_sropen / sigio_swopen open with
// convert='big_endian', sigio_module.f90:430-456).  Header versions 200509
// and 198410 (sigio_srhead / sigio_swhead, :470-676); data records in the
// order of sigio_srdata / sigio_swdata (:755-915); record-length tables of
// sigio_adhead (:1323-1382).  On top of the format, readin_sig / wrtout_sig
// (src/dyn_init.f90:93-191) renormalise the coefficients between the NCEP
// spectral normalisation and the model's orthonormal harmonics.
//
// Byte order is assembled byte by byte (no host-endianness assumption); the
// file is read record by record with stdio.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gd_api.h"

namespace {

thread_local std::string t_err;

struct IoFail {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw IoFail{code, msg}; }

// ------------------------------------------------------------ byte order
uint32_t get_u32(const unsigned char* p) {
  return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | (uint32_t)p[3];
}
uint64_t get_u64(const unsigned char* p) { return (uint64_t)get_u32(p) << 32 | get_u32(p + 4); }
void put_u32(unsigned char* p, uint32_t v) {
  p[0] = (unsigned char)(v >> 24);
  p[1] = (unsigned char)(v >> 16);
  p[2] = (unsigned char)(v >> 8);
  p[3] = (unsigned char)v;
}
void put_u64(unsigned char* p, uint64_t v) {
  put_u32(p, (uint32_t)(v >> 32));
  put_u32(p + 4, (uint32_t)v);
}
int32_t get_i32(const unsigned char* p) {
  const uint32_t u = get_u32(p);
  int32_t i;
  memcpy(&i, &u, 4);
  return i;
}
float get_f32(const unsigned char* p) {
  const uint32_t u = get_u32(p);
  float f;
  memcpy(&f, &u, 4);
  return f;
}
double get_f64(const unsigned char* p) {
  const uint64_t u = get_u64(p);
  double d;
  memcpy(&d, &u, 8);
  return d;
}
void put_i32(unsigned char* p, int32_t i) {
  uint32_t u;
  memcpy(&u, &i, 4);
  put_u32(p, u);
}
void put_f32(unsigned char* p, float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  put_u32(p, u);
}
void put_f64(unsigned char* p, double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  put_u64(p, u);
}

// Record builder: words appended in order, big-endian.
struct Rec {
  std::vector<unsigned char> b;
  void i32(int32_t v) {
    b.resize(b.size() + 4);
    put_i32(&b[b.size() - 4], v);
  }
  void f32(float v) {
    b.resize(b.size() + 4);
    put_f32(&b[b.size() - 4], v);
  }
  void chars(const char* s, size_t n) { b.insert(b.end(), s, s + n); }
};

// ------------------------------------------- Fortran sequential records
class SeqFile {
 public:
  SeqFile(const char* path, bool write) : path_(path) {
    f_ = fopen(path, write ? "wb" : "rb");
    if (!f_) fail(GD_ERR_IO, std::string("cannot open ") + path + (write ? " for writing" : ""));
  }
  ~SeqFile() {
    if (f_) fclose(f_);
  }
  // The next record's payload.  A Fortran read of fewer items than the
  // record holds skips the rest, so callers check a minimum length only.
  const std::vector<unsigned char>& next(const char* what, size_t need = 0) {
    unsigned char m[4];
    if (fread(m, 1, 4, f_) != 4) fail(GD_ERR_IO, path_ + ": end of file before the " + what + " record");
    const int32_t n = get_i32(m);
    if (n < 0)
      fail(GD_ERR_IO, path_ + ": the " + what + " record is split into subrecords (2^31 bytes or more)");
    buf_.resize((size_t)n);
    if (n > 0 && fread(buf_.data(), 1, (size_t)n, f_) != (size_t)n)
      fail(GD_ERR_IO, path_ + ": the " + what + " record is truncated");
    unsigned char t[4];
    if (fread(t, 1, 4, f_) != 4 || get_i32(t) != n)
      fail(GD_ERR_IO, path_ + ": the " + what + " record's trailing length marker is missing or differs");
    if (buf_.size() < need)
      fail(GD_ERR_IO, path_ + ": the " + what + " record holds " + std::to_string(buf_.size()) +
                          " bytes, fewer than the " + std::to_string(need) + " read from it");
    return buf_;
  }
  void put(const unsigned char* p, size_t n, const char* what) {
    if (n > 0x7FFFFFFFu) fail(GD_ERR_IO, path_ + ": the " + what + " record is 2^31 bytes or more");
    unsigned char m[4];
    put_u32(m, (uint32_t)n);
    if (fwrite(m, 1, 4, f_) != 4 || (n && fwrite(p, 1, n, f_) != n) || fwrite(m, 1, 4, f_) != 4)
      fail(GD_ERR_IO, path_ + ": writing the " + what + " record failed");
  }
  void put(const Rec& r, const char* what) { put(r.b.data(), r.b.size(), what); }
  void close() {
    FILE* f = f_;
    f_ = nullptr;
    if (fclose(f) != 0) fail(GD_ERR_IO, path_ + ": closing failed");
  }

 private:
  FILE* f_ = nullptr;
  std::string path_;
  std::vector<unsigned char> buf_;
};

// ------------------------------------------------------------ the header
constexpr int kIntFill = -9999;  // sigio_intfill
constexpr float kFill = GD_SIG_FILL;

bool thermo3(const gd_sighead& h) { return (h.idvm / 10) % 10 == 3; }  // Fortran mod: sign of the dividend
long nc_words(const gd_sighead& h) { return (long)(h.jcap + 1) * (h.jcap + 2); }

struct Layout {
  std::vector<int32_t> lhead, ldata;
};

// sigio_adhead (sigio_module.f90:1323-1382).
Layout adhead(gd_sighead& h) {
  h.nxgr = 0;
  h.nxss = 0;
  switch (h.ixgr) {
    case 1: h.nxgr = 2 * h.levs + 1; break;
    case 2: h.nxgr = 4 * h.levs + 3; break;
    case 3: h.nxgr = 3 * h.levs + 1; break;
    case 4: h.nxgr = 4 * h.levs + 3, h.nxss = 1; break;
    case 5: h.nxgr = 3 * h.levs + 1, h.nxss = 1; break;
    default: break;
  }
  const int nspec = 2 + (3 + h.ntrac) * h.levs;
  const int32_t lspec = (int32_t)(4L * h.irealf * nc_words(h));
  const int32_t lgrid = (int32_t)(4L * h.irealf * h.lonb * h.latb);
  Layout L;
  if (h.ivs == 200509) {
    const int jxss = h.nxss > 0 ? 1 : 0;
    h.nhead = thermo3(h) ? 7 : 5;
    h.ndata = nspec + h.nxgr + jxss;
    L.lhead = {32, 4 * (h.nhead + h.ndata), 4 * 50, 4 * ((h.levs + 1) * h.nvcoord), 8 * (5 + h.ntrac)};
    if (thermo3(h)) {
      L.lhead.push_back(4 * (h.ntrac + 1));
      L.lhead.push_back(4 * (h.ntrac + 1));
    }
    L.ldata.assign((size_t)h.ndata, lspec);
    for (int i = nspec; i < nspec + h.nxgr; ++i) L.ldata[(size_t)i] = lgrid;
    for (int i = nspec + h.nxgr; i < h.ndata; ++i) L.ldata[(size_t)i] = 4 * h.irealf * h.nxss;
  } else {
    h.nhead = 2;
    h.ndata = nspec + h.nxgr;
    L.lhead = {32, 4 * 250};
    L.ldata.assign((size_t)h.ndata, lspec);
    for (int i = nspec; i < h.ndata; ++i) L.ldata[(size_t)i] = lgrid;
  }
  return L;
}

void head_init(gd_sighead& h) {
  memset(&h, 0, sizeof(h));
  memset(h.clabsig, ' ', sizeof(h.clabsig));
  h.fhour = kFill;
  for (int& v : h.idate) v = kIntFill;
  for (float& v : h.si) v = kFill;
  for (float& v : h.sl) v = kFill;
  for (float& v : h.ak) v = kFill;
  for (float& v : h.bk) v = kFill;
  int* ints[] = {&h.jcap, &h.levs, &h.itrun, &h.iorder, &h.irealf, &h.igen, &h.latf, &h.lonf, &h.latb,
                 &h.lonb, &h.latr, &h.lonr, &h.ntrac, &h.icen2, &h.iens[0], &h.iens[1], &h.idpp, &h.idsl,
                 &h.idvc, &h.idvm, &h.idvt, &h.idrun, &h.idusr, &h.ncldt, &h.ixgr, &h.ivs, &h.nvcoord,
                 &h.nxgr, &h.nxss, &h.nhead, &h.ndata};
  for (int* p : ints) *p = kIntFill;
  h.pdryini = kFill;
  for (auto& row : h.vcoord)
    for (float& v : row) v = kFill;
  memset(h.cfvars, ' ', sizeof(h.cfvars));
  for (float& v : h.cpi) v = kFill;
  for (float& v : h.ri) v = kFill;
}

// sigio_alhead's effect on a header being read (sigio_module.f90:678-719):
// vcoord to the fill value, cfvars blank.
void alhead(gd_sighead& h) {
  for (auto& row : h.vcoord)
    for (float& v : row) v = kFill;
  memset(h.cfvars, ' ', sizeof(h.cfvars));
}

void check_dims(const gd_sighead& h, const std::string& where, int code) {
  if (h.jcap < 0 || h.levs < 1 || h.ntrac < 0)
    fail(code, where + ": header has jcap " + std::to_string(h.jcap) + ", levs " + std::to_string(h.levs) +
                   ", ntrac " + std::to_string(h.ntrac));
  if (h.levs > GD_SIG_MAXLEVS || h.ntrac > GD_SIG_MAXTRAC)
    fail(GD_ERR_UNSUPPORTED, where + ": header has levs " + std::to_string(h.levs) + " or ntrac " +
                                 std::to_string(h.ntrac) + " beyond GD_SIG_MAXLEVS / GD_SIG_MAXTRAC");
  if ((long)h.jcap + 1 > 46000) fail(code, where + ": jcap " + std::to_string(h.jcap) + " out of range");
}

// Fortran INT of a real ext word (truncation toward zero), for a finite word.
int ext_int(float v, const std::string& path) {
  if (!std::isfinite(v) || std::fabs(v) >= 2147483648.0f)
    fail(GD_ERR_IO, path + ": 198410 header word out of the integer range");
  return (int)v;
}

// sigio_srhead (sigio_module.f90:470-576) on an open file.
void read_head(SeqFile& f, const std::string& path, gd_sighead& h) {
  head_init(h);
  const auto& r1 = f.next("label");
  if (r1.size() >= 8 && memcmp(r1.data(), "GFS SIG ", 8) == 0) {  // modern sigma file
    if (r1.size() < 32) fail(GD_ERR_IO, path + ": label record shorter than 32 bytes");
    h.ivs = get_i32(&r1[8]);
    if (h.ivs != 200509) fail(GD_ERR_IO, path + ": sigma file version " + std::to_string(h.ivs) + " is not 200509");
    f.next("record-length");
    const auto& r3 = f.next("header", 32 * 4);
    const unsigned char* p = r3.data();
    int w = 0;
    auto I = [&] { return get_i32(p + 4 * w++); };
    auto F = [&] { return get_f32(p + 4 * w++); };
    h.fhour = F();
    for (int& v : h.idate) v = I();
    h.jcap = I(), h.levs = I(), h.itrun = I(), h.iorder = I(), h.irealf = I(), h.igen = I();
    h.latf = I(), h.lonf = I(), h.latb = I(), h.lonb = I(), h.latr = I(), h.lonr = I();
    h.ntrac = I(), h.nvcoord = I(), h.icen2 = I(), h.iens[0] = I(), h.iens[1] = I();
    h.idpp = I(), h.idsl = I(), h.idvc = I(), h.idvm = I(), h.idvt = I(), h.idrun = I(), h.idusr = I();
    h.pdryini = F();
    h.ncldt = I(), h.ixgr = I();
    check_dims(h, path, GD_ERR_IO);
    if (h.nvcoord < 0 || h.nvcoord > 3)
      fail(GD_ERR_UNSUPPORTED, path + ": nvcoord " + std::to_string(h.nvcoord) + " outside 0..3");
    alhead(h);
    const int nv = h.levs + 1;
    const auto& rv = f.next("vcoord", (size_t)4 * nv * h.nvcoord);
    for (int j = 0; j < h.nvcoord; ++j)
      for (int k = 0; k < nv; ++k) h.vcoord[j][k] = get_f32(&rv[(size_t)4 * (j * nv + k)]);
    const auto& rc = f.next("cfvars", (size_t)8 * (5 + h.ntrac));
    memcpy(h.cfvars, rc.data(), (size_t)8 * (5 + h.ntrac));
    if (thermo3(h)) {
      const auto& rp = f.next("cpi", (size_t)4 * (h.ntrac + 1));
      for (int i = 0; i <= h.ntrac; ++i) h.cpi[i] = get_f32(&rp[(size_t)4 * i]);
      const auto& rr = f.next("ri", (size_t)4 * (h.ntrac + 1));
      for (int i = 0; i <= h.ntrac; ++i) h.ri[i] = get_f32(&rr[(size_t)4 * i]);
    }
    // the reference sets these after reading a 200509 header
    memset(h.clabsig, ' ', sizeof(h.clabsig));
    for (float& v : h.si) v = kFill;
    for (float& v : h.sl) v = kFill;
    for (float& v : h.ak) v = kFill;
    for (float& v : h.bk) v = kFill;
    h.pdryini = kFill;
  } else {  // 198410: ON85 label, then fhour, idate(4), sisl(201), ext(44)
    if (r1.size() < 32) fail(GD_ERR_IO, path + ": not a sigma file (first record shorter than 32 bytes)");
    memcpy(h.clabsig, r1.data(), 32);
    const auto& r2 = f.next("header", 250 * 4);
    const unsigned char* p = r2.data();
    h.fhour = get_f32(p);
    for (int i = 0; i < 4; ++i) h.idate[i] = get_i32(p + 4 * (1 + i));
    float sisl[201], ext[44];
    for (int i = 0; i < 201; ++i) sisl[i] = get_f32(p + 4 * (5 + i));
    for (int i = 0; i < 44; ++i) ext[i] = get_f32(p + 4 * (206 + i));
    int* dst[] = {&h.jcap, &h.levs, &h.itrun, &h.iorder, &h.irealf, &h.igen, &h.lonf, &h.latf, &h.lonb,
                  &h.latb, &h.lonr, &h.latr};
    for (int i = 0; i < 12; ++i) *dst[i] = ext_int(ext[i], path);
    h.ntrac = ext_int(std::fmax(ext[12], 1.0f), path);
    h.icen2 = ext_int(ext[13], path);
    h.iens[0] = ext_int(ext[14], path), h.iens[1] = ext_int(ext[15], path);
    int* dst2[] = {&h.idpp, &h.idsl, &h.idvc, &h.idvm, &h.idvt, &h.idrun, &h.idusr};
    for (int i = 0; i < 7; ++i) *dst2[i] = ext_int(ext[16 + i], path);
    h.pdryini = ext[23];
    h.ncldt = ext_int(ext[24], path);
    h.ixgr = ext_int(ext[25], path);
    check_dims(h, path, GD_ERR_IO);
    const int L = h.levs;
    if (h.idvc == 0 || h.idvc == 1) {
      if (L > 100) fail(GD_ERR_IO, path + ": 198410 sigma header with more than 100 levels");
      for (int k = 0; k <= L; ++k) h.si[k] = sisl[k];
      for (int k = 0; k < L; ++k) h.sl[k] = sisl[L + 1 + k];
      h.nvcoord = 1;
      alhead(h);
      for (int k = 0; k <= L; ++k) h.vcoord[0][k] = sisl[k];
    } else if (h.idvc == 2 || h.idvc == 3) {
      if (L > 99) fail(GD_ERR_IO, path + ": 198410 hybrid header with more than 99 levels");
      if (h.idvc == 2) {
        for (int k = 0; k <= L; ++k) h.ak[k] = sisl[k];
        for (int k = 0; k <= L; ++k) h.bk[k] = sisl[L + 1 + k];
      }
      h.nvcoord = 2;
      alhead(h);
      for (int k = 0; k <= L; ++k) h.vcoord[0][k] = sisl[k], h.vcoord[1][k] = sisl[L + 1 + k];
    }
    h.ivs = 198410;
  }
  adhead(h);
}

// sigio_modpr's layer values for one column (sigio_module.f90:1207-1321),
// the cases sigio_swhead uses: sigma interfaces vcoord(:,1) at ps = 1,
// idsl 0/1 (Phillips) or 2 (mean).  Returns false for another idsl.
bool modpr_sigma_layers(const gd_sighead& h, float* pm) {
  int id2 = 0;
  if (h.idsl == 0 || h.idsl == 1) id2 = 1;
  else if (h.idsl == 2) id2 = 2;
  if (id2 == 0) return false;
  const double rocp = (double)(287.05f / 1004.6f);  // single-precision literals
  const double rocpr = 1 / rocp;
  const float ps = 1.0f;
  double pid = ps, pidk = id2 == 1 ? std::pow(pid, rocp) : 0.0;
  for (int k = 0; k < h.levs; ++k) {
    const double piu = (double)(h.vcoord[0][k + 1] * ps);
    double pmm, piuk = 0.0;
    if (id2 == 1) {
      piuk = std::pow(piu, rocp);
      const double pmk = (pid * pidk - piu * piuk) / ((rocp + 1) * (pid - piu));
      pmm = std::pow(pmk, rocpr);
    } else {
      pmm = (pid + piu) / 2;
    }
    pm[k] = (float)pmm;
    pid = piu;
    pidk = piuk;
  }
  return true;
}

// sigio_swhead (sigio_module.f90:578-676).
void write_head(SeqFile& f, gd_sighead& h, const Layout& L) {
  if (h.ivs >= 200509) {
    Rec r1;
    r1.chars("GFS SIG ", 8);
    for (int v : {h.ivs, h.nhead, h.ndata, 0, 0, 0}) r1.i32(v);
    f.put(r1, "label");
    Rec r2;
    for (int32_t v : L.lhead) r2.i32(v);
    for (int32_t v : L.ldata) r2.i32(v);
    f.put(r2, "record-length");
    Rec r3;
    r3.f32(h.fhour);
    for (int v : h.idate) r3.i32(v);
    for (int v : {h.jcap, h.levs, h.itrun, h.iorder, h.irealf, h.igen, h.latf, h.lonf, h.latb, h.lonb, h.latr,
                  h.lonr, h.ntrac, h.nvcoord, h.icen2, h.iens[0], h.iens[1], h.idpp, h.idsl, h.idvc, h.idvm,
                  h.idvt, h.idrun, h.idusr})
      r3.i32(v);
    r3.f32(h.pdryini);
    r3.i32(h.ncldt);
    r3.i32(h.ixgr);
    for (int i = 0; i < 18; ++i) r3.i32(0);
    f.put(r3, "header");
    Rec rv;
    for (int j = 0; j < h.nvcoord; ++j)
      for (int k = 0; k <= h.levs; ++k) rv.f32(h.vcoord[j][k]);
    f.put(rv, "vcoord");
    Rec rc;
    rc.chars(&h.cfvars[0][0], (size_t)8 * (5 + h.ntrac));
    f.put(rc, "cfvars");
    if (thermo3(h)) {
      Rec rp, rr;
      for (int i = 0; i <= h.ntrac; ++i) rp.f32(h.cpi[i]), rr.f32(h.ri[i]);
      f.put(rp, "cpi");
      f.put(rr, "ri");
    }
    return;
  }
  const int Lv = h.levs;
  float sisl[201] = {0};
  if (h.idvc == 0 || h.idvc == 1) {
    if (Lv > 100) fail(GD_ERR_ARG, "198410 sigma header with more than 100 levels");
    if (h.nvcoord == 1 && h.vcoord[0][0] == 1.0f) {
      for (int k = 0; k <= Lv; ++k) sisl[k] = h.vcoord[0][k];
      modpr_sigma_layers(h, sisl + Lv + 1);
    } else {
      for (int k = 0; k <= Lv; ++k) sisl[k] = h.si[k];
      for (int k = 0; k < Lv; ++k) sisl[Lv + 1 + k] = h.sl[k];
    }
  } else if (h.idvc == 2 || h.idvc == 3) {
    if (Lv > 99) fail(GD_ERR_ARG, "198410 hybrid header with more than 99 levels");
    if (h.nvcoord == 2 && h.vcoord[1][0] == 1.0f) {
      for (int k = 0; k <= Lv; ++k) sisl[k] = h.vcoord[0][k], sisl[Lv + 1 + k] = h.vcoord[1][k];
    } else if (h.idvc == 2) {
      for (int k = 0; k <= Lv; ++k) sisl[k] = h.ak[k], sisl[Lv + 1 + k] = h.bk[k];
    }
  }
  float ext[44] = {0};
  const int src[] = {h.jcap, h.levs, h.itrun, h.iorder, h.irealf, h.igen, h.lonf, h.latf, h.lonb, h.latb, h.lonr,
                     h.latr, h.ntrac, h.icen2, h.iens[0], h.iens[1], h.idpp, h.idsl, h.idvc, h.idvm, h.idvt,
                     h.idrun, h.idusr};
  for (int i = 0; i < 23; ++i) ext[i] = (float)src[i];
  ext[23] = h.pdryini;
  ext[24] = (float)h.ncldt;
  ext[25] = (float)h.ixgr;
  f.put(reinterpret_cast<const unsigned char*>(h.clabsig), 32, "label");
  Rec r2;
  r2.f32(h.fhour);
  for (int v : h.idate) r2.i32(v);
  for (float v : sisl) r2.f32(v);
  for (float v : ext) r2.f32(v);
  f.put(r2, "header");
}

// ------------------------------------------------------------- the data
// sqrt(2 pi) of copyspecin / copyspecout (dyn_init.f90:97-99): pi is the
// reference's con_pi, a literal without a kind suffix (single-rounded).
const double kRenorm = std::sqrt(2.0 * (double)(float)3.1415926535897931);

// One data record into nc/2 complex coefficients (interleaved doubles):
// sigio_srdata's values (rounded to float from 8-byte data) times sqrt(2 pi).
void spec_in(const std::vector<unsigned char>& r, long nc, bool dbl, double* out) {
  if (!out) return;
  if (dbl)
    for (long i = 0; i < nc; ++i) out[i] = kRenorm * (double)(float)get_f64(&r[(size_t)8 * i]);
  else
    for (long i = 0; i < nc; ++i) out[i] = kRenorm * (double)get_f32(&r[(size_t)4 * i]);
}

// copyspecout into one data record: re / sqrt(2 pi) rounded to float, then
// widened for 8-byte data (sigio_swdata copies the float buffer).  NULL
// writes zeros.
void spec_out(const double* in, long nc, bool dbl, std::vector<unsigned char>& r) {
  const size_t w = dbl ? 8 : 4;
  r.assign(w * (size_t)nc, 0);
  if (!in) return;
  for (long i = 0; i < nc; ++i) {
    const float v = (float)(in[i] / kRenorm);
    if (dbl) put_f64(&r[8 * (size_t)i], (double)v);
    else put_f32(&r[4 * (size_t)i], v);
  }
}

template <typename F>
int guarded(F f) {
  try {
    f();
    return GD_OK;
  } catch (const IoFail& e) {
    t_err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    t_err = "host allocation failed";
    return GD_ERR_NOMEM;
  } catch (const std::exception& e) {
    t_err = e.what();
    return GD_ERR_IO;
  }
}

}  // namespace

extern "C" {

int gd_sigio_head_init(gd_sighead* head) {
  if (!head) return GD_ERR_ARG;
  head_init(*head);
  return GD_OK;
}

int gd_sigio_read_head(const char* path, gd_sighead* head) {
  if (!path || !head) {
    t_err = "gd_sigio_read_head: null argument";
    return GD_ERR_ARG;
  }
  return guarded([&] {
    SeqFile f(path, false);
    read_head(f, path, *head);
  });
}

int gd_sigio_read(const char* path, int jcap, int levs, int ntrac, gd_sighead* head, double* vrt, double* div,
                  double* tv, double* trc, double* lnps, double* topo) {
  if (!path || !head || jcap < 0 || levs < 1 || ntrac < 0) {
    t_err = "gd_sigio_read: null path/header or negative size";
    return GD_ERR_ARG;
  }
  return guarded([&] {
    SeqFile f(path, false);
    gd_sighead h;
    read_head(f, path, h);
    if (h.jcap != jcap || h.levs != levs || h.ntrac < ntrac)
      fail(GD_ERR_ARG, std::string(path) + ": file has jcap " + std::to_string(h.jcap) + ", levs " +
                           std::to_string(h.levs) + ", ntrac " + std::to_string(h.ntrac) + "; the caller expects " +
                           std::to_string(jcap) + ", " + std::to_string(levs) + ", >= " + std::to_string(ntrac));
    const long nc = nc_words(h), nlm2 = nc;  // nc reals = nlm complex
    const bool dbl = h.irealf == 2;
    const size_t w = dbl ? 8 : 4, need = w * (size_t)nc;
    spec_in(f.next("orography", need), nc, dbl, topo);
    spec_in(f.next("ln(ps)", need), nc, dbl, lnps);
    for (int k = 0; k < levs; ++k) spec_in(f.next("temperature", need), nc, dbl, tv ? tv + nlm2 * k : nullptr);
    for (int k = 0; k < levs; ++k) {
      spec_in(f.next("divergence", need), nc, dbl, div ? div + nlm2 * k : nullptr);
      spec_in(f.next("vorticity", need), nc, dbl, vrt ? vrt + nlm2 * k : nullptr);
    }
    for (int n = 0; n < h.ntrac; ++n)
      for (int k = 0; k < levs; ++k) {
        const auto& r = f.next("tracer", need);
        if (n < ntrac && trc) spec_in(r, nc, dbl, trc + nlm2 * ((long)n * levs + k));
      }
    for (int n = 0; n < h.nxgr; ++n) f.next("extra grid", w * (size_t)h.lonb * (size_t)h.latb);
    if (h.nxss > 0) f.next("extra scalar", w * (size_t)h.nxss);
    *head = h;
  });
}

int gd_sigio_write(const char* path, gd_sighead* head, int ntrac, const double* vrt, const double* div,
                   const double* tv, const double* trc, const double* lnps, const double* topo) {
  if (!path || !head) {
    t_err = "gd_sigio_write: null path or header";
    return GD_ERR_ARG;
  }
  return guarded([&] {
    gd_sighead& h = *head;
    check_dims(h, "gd_sigio_write", GD_ERR_ARG);
    if (ntrac < 0 || ntrac > h.ntrac)
      fail(GD_ERR_ARG, "gd_sigio_write: " + std::to_string(ntrac) + " tracers given, header has " +
                           std::to_string(h.ntrac));
    if (h.ivs >= 200509 && (h.nvcoord < 0 || h.nvcoord > 3))
      fail(GD_ERR_ARG, "gd_sigio_write: nvcoord " + std::to_string(h.nvcoord) + " outside 0..3");
    const Layout L = adhead(h);
    if (h.nxgr > 0 && (h.lonb < 0 || h.latb < 0))
      fail(GD_ERR_ARG, "gd_sigio_write: extra grid records need lonb, latb >= 0");
    SeqFile f(path, true);
    write_head(f, h, L);
    const long nc = nc_words(h), nlm2 = nc;
    const bool dbl = h.irealf == 2;
    std::vector<unsigned char> r;
    auto put = [&](const double* p, const char* what) {
      spec_out(p, nc, dbl, r);
      f.put(r.data(), r.size(), what);
    };
    put(topo, "orography");
    put(lnps, "ln(ps)");
    for (int k = 0; k < h.levs; ++k) put(tv ? tv + nlm2 * k : nullptr, "temperature");
    for (int k = 0; k < h.levs; ++k) {
      put(div ? div + nlm2 * k : nullptr, "divergence");
      put(vrt ? vrt + nlm2 * k : nullptr, "vorticity");
    }
    for (int n = 0; n < h.ntrac; ++n)
      for (int k = 0; k < h.levs; ++k)
        put(n < ntrac && trc ? trc + nlm2 * ((long)n * h.levs + k) : nullptr, "tracer");
    const size_t w = dbl ? 8 : 4;
    r.assign(w * (size_t)h.lonb * (size_t)(h.latb > 0 ? h.latb : 0), 0);
    for (int n = 0; n < h.nxgr; ++n) f.put(r.data(), r.size(), "extra grid");
    if (h.nxss > 0) {
      r.assign(w * (size_t)h.nxss, 0);
      f.put(r.data(), r.size(), "extra scalar");
    }
    f.close();
  });
}

int gd_sigio_config(const gd_sighead* head, gd_config* cfg, double* ak, double* bk) {
  if (!head || !cfg) {
    t_err = "gd_sigio_config: null argument";
    return GD_ERR_ARG;
  }
  return guarded([&] {
    const gd_sighead& h = *head;
    check_dims(h, "gd_sigio_config", GD_ERR_ARG);
    if (h.idvc != 2 || h.nvcoord < 2)
      fail(GD_ERR_UNSUPPORTED, "gd_sigio_config: unknown vertical coordinate type " + std::to_string(h.idvc) +
                                   " (hybrid, idvc 2 with nvcoord >= 2, is required)");
    cfg->ntrunc = h.jcap;
    cfg->nlon = h.lonb;
    cfg->nlat = h.latb;
    cfg->nlev = h.levs;
    // params.f90:259-264: single-precision product, reset when above 1e5 Pa
    double p = h.pdryini == kFill ? 0.0 : (double)(h.pdryini * 1000.0f);
    if (p > 1.e5) p = 0.0;
    cfg->pdryini = p;
    for (int k = 0; k <= h.levs; ++k) {
      if (ak) ak[k] = h.vcoord[0][h.levs - k];
      if (bk) bk[k] = h.vcoord[1][h.levs - k];
    }
  });
}

const char* gd_sigio_last_error(void) { return t_err.c_str(); }

}  // extern "C"
