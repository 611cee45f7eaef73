// Text writers of the exciton path's output files, byte for byte in the reference's formatted records, so that
// PP_ONLY runs (bsedielraw and friends read bse_opt_diel.dat back) and the downstream steps that read these files
// keep working.  Host code: the files are written from host arrays the C ABI returned.
//
// Formatted records follow the Fortran edit descriptors the reference uses:
//   Fw.d  the value rounded to d decimals (correctly rounded from the binary value), right-justified in w
//         characters, the optional leading zero dropped when it does not fit, w asterisks when the number
//         does not fit at all;
//   Ew.d  0.d1...dd E+xx (E dropped for a three-digit exponent), same justification rules;
//   Iw, Iw.m  right-justified integers, Iw.0 of zero is all blanks; the reference's width-less I is read as
//         I12, the default width of a 4-byte integer.
// List-directed records (the '#' header lines, and the whole of bse_diel_*.dat, sp_diel*.dat, bands_bse.dat,
// bz_act_*.dat and dichroism.dat) are written as gfortran's runtime writes them (the reference's README names the
// GNU compiler): a blank before the first item, one blank between items except between two character items,
// 4-byte integers as I11, REAL(8) as 1PG25.17E3 and REAL(4) as 1PG16.9E2.
//   bse_opt_diel.dat / -pol   src/module_bse.F90:2132-2133, :2556-2567 (7F15.4 / 6F15.4)
//   sp_optics.dat / -pol      :2296-2297, :2366-2367 (7F15.4 / 6F15.4)
//   tm_coef.dat / -pol        :2300-2311, :2370-2377 (3F10.4,3I10.0,7F10.4 / ...,6F10.4)
//   exc_wf_<n>.dat            excwf2, :374-408 ((I,3F15.4,2I,2E15.4)); exc_wf_<n>_<q>.dat excwfi2, :412-448
//   exciton_lifetime.dat      lifetime, :3271-3349 ((1F15.4,4E15.4)); -pol: lifetimepol, :3353-3432 ((1F15.4,6E15.4))
//   bse_diel_*.dat            bsedielraw, :926-931, :1004-1009; bsedielrawpol :1130-1134, :1174-1178;
//   sp_diel_*.dat             spdielraw / spdielrawpol (same records): REAL(8) energy, two REAL(4)
//   bands_bse.dat             bsebnds, :1536-1543 / bsebndstemp :1981-1990: REAL(4) path coordinate, REAL(8)
//                             energy, an empty record after each band
//   bz_act_*.dat, dichroism   spoptpolbz, :4754-4759: three REAL(4) k coordinates, one REAL(8)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#include "ctx.h"

namespace wtb {

// IEEE specials under F and E editing: Infinity / -Infinity (Inf when narrower than 8), NaN
static std::string fortran_special(double x, int w) {
  std::string s = std::isnan(x) ? "NaN" : (w >= 8 + (x < 0) ? "Infinity" : "Inf");
  if (std::isinf(x) && x < 0) s = "-" + s;
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string fortran_F(double x, int w, int d) {
  if (std::isnan(x) || std::isinf(x)) return fortran_special(x, w);
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%.*f", d, x);
  std::string s(buf);
  if ((int)s.size() > w) {
    // the leading zero of |x| < 1 is optional
    if (s.rfind("0.", 0) == 0)
      s.erase(0, 1);
    else if (s.rfind("-0.", 0) == 0)
      s.erase(1, 1);
  }
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string fortran_E(double x, int w, int d) {
  if (std::isnan(x) || std::isinf(x)) return fortran_special(x, w);
  std::string digits;
  int e10 = 0;
  bool neg = std::signbit(x);
  if (x == 0.0) {
    digits.assign((size_t)d, '0');
  } else {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.*e", d - 1, std::fabs(x));  // d significant digits: "D.DDDe+XX"
    const char* p = buf;
    digits.push_back(*p++);
    if (*p == '.') ++p;
    while (*p && *p != 'e') digits.push_back(*p++);
    e10 = std::atoi(p + 1) + 1;
  }
  std::string exp;
  char eb[16];
  if (std::abs(e10) <= 99)
    std::snprintf(eb, sizeof(eb), "E%c%02d", e10 < 0 ? '-' : '+', std::abs(e10));
  else
    std::snprintf(eb, sizeof(eb), "%c%03d", e10 < 0 ? '-' : '+', std::abs(e10));
  exp = eb;
  std::string s = std::string(neg ? "-" : "") + "0." + digits + exp;
  if ((int)s.size() > w) s = std::string(neg ? "-" : "") + "." + digits + exp;
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string fortran_I(long v, int w, int m) {
  if (m == 0 && v == 0) return std::string((size_t)w, ' ');
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%ld", std::labs(v));
  std::string s(buf);
  if ((int)s.size() < m) s = std::string((size_t)(m - (int)s.size()), '0') + s;
  if (v < 0) s = "-" + s;
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

namespace {

// Radiative lifetimes of exclft (src/module_bse.F90:326-370) for the rows of bse_opt_diel.dat as lifetime reads
// them (src/module_bse.F90:3271-3349): fosc(dim, 7) = energy, xx, yy, zz, ...; lft(dim, 4) = for xx+yy+zz, xx,
// yy, zz.  pol: the rows of bse_opt_diel-pol.dat as lifetimepol reads them (:3353-3432), fosc(dim, 6) = energy,
// xx, yy, zz, sp, sm and lft(dim, 6) adding sp, sm.  The constants are the reference's single-precision
// literals; sysdim 3 / 2 / 1.
__global__ void lifetime_kernel(const double* __restrict__ fosc, int dim, int pol, int sysdim, double ng,
                                double vc2d, double a11, double* __restrict__ lft) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dim) return;
  const double cfe = (double)7.297E-3f, lspd = (double)299.792E16f, hbar = (double)6.582E-16f;
  const double pi = (double)3.14159274101257324f;
  const size_t n = (size_t)dim;
  const double e = fosc[i];
  const int nout = pol ? 6 : 4;
  double f[6] = {fosc[n + i] + fosc[2 * n + i] + fosc[3 * n + i], fosc[n + i], fosc[2 * n + i], fosc[3 * n + i],
                 0.0, 0.0};
  if (pol) {
    f[4] = fosc[4 * n + i];
    f[5] = fosc[5 * n + i];
  }
  for (int c = 0; c < nout; ++c) {
    double l;
    if (sysdim == 3) {
      const double aux1 = (4.0 * cfe) * (e * e * e);
      const double aux2 = f[c] / ng;
      const double aux3 = 3.0 * (lspd * lspd) * (hbar * hbar * hbar);
      l = 1.0 / ((aux1 * aux2) / aux3);
    } else if (sysdim == 2) {
      const double aux1 = ng * vc2d * hbar;
      const double aux2 = (8.0 * pi * cfe * e) * f[c];
      l = aux1 / aux2;
    } else {
      const double aux2 = (2.0 * pi * cfe * e * e) * f[c];
      const double aux1 = ng * a11 * hbar * hbar * lspd;
      l = aux1 / aux2;
    }
    lft[c * n + i] = l;
  }
}

}  // namespace

}  // namespace wtb

namespace {

using wtb::fortran_E;
using wtb::fortran_F;
using wtb::fortran_I;
using wtb::fortran_special;

// One real item of a list-directed WRITE as gfortran's runtime edits it: G editing with scale factor 1P,
// 1PG25.17E3 for REAL(8) (kind 8) and 1PG16.9E2 for REAL(4) (kind 4, of the value rounded to single precision).
// With r the value rounded to d significant digits and 10^(k-1) <= |r| < 10^k: F(w-n).(d-k) followed by n = e+2
// blanks when 0 <= k <= d, else one digit, the point, d-1 digits and E+-e digits; zero as F(w-n).(d-1).
// The C library's conversions round the exact binary value to nearest, ties to even.
std::string ld_real(double x, int kind) {
  const int w = kind == 8 ? 25 : 16, d = kind == 8 ? 17 : 9, e = kind == 8 ? 3 : 2, n = e + 2;
  if (kind != 8) x = (double)(float)x;
  if (std::isnan(x) || std::isinf(x)) return fortran_special(x, w);
  const std::string sign = std::signbit(x) ? "-" : "";
  auto pad = [](const std::string& t, int width) {
    return (int)t.size() >= width ? t : std::string((size_t)(width - (int)t.size()), ' ') + t;
  };
  char buf[128];
  if (x == 0.0) return pad(sign + "0." + std::string((size_t)(d - 1), '0'), w - n) + std::string((size_t)n, ' ');
  std::snprintf(buf, sizeof(buf), "%.*e", d - 1, std::fabs(x));  // "D.DDDe+XX", rounded to d digits
  const char* ep = std::strchr(buf, 'e');
  const int ex = std::atoi(ep + 1), k = ex + 1;
  if (k >= 0 && k <= d) {
    char fb[128];
    std::snprintf(fb, sizeof(fb), "%#.*f", d - k, std::fabs(x));  // '#': the point also with no decimals
    return pad(sign + fb, w - n) + std::string((size_t)n, ' ');
  }
  char xb[16];
  std::snprintf(xb, sizeof(xb), "E%c%0*d", ex < 0 ? '-' : '+', e, std::abs(ex));
  return pad(sign + std::string(buf, (size_t)(ep - buf)) + xb, w);
}

// One list-directed output record as gfortran writes it: a blank before the first item, one blank before
// every later item except a character item that follows a character item; character items as they are,
// 4-byte integers as I11, reals by ld_real.  A WRITE with no items is an empty record.
struct LdRecord {
  std::string s;
  bool first = true, prev_char = false;
  void sep(bool is_char) {
    if (first || !(is_char && prev_char)) s += ' ';
    first = false;
    prev_char = is_char;
  }
  LdRecord& c(const char* t) {
    sep(true);
    s += t;
    return *this;
  }
  LdRecord& i(long v) {
    sep(false);
    s += fortran_I(v, 11, 1);
    return *this;
  }
  LdRecord& r8(double v) {
    sep(false);
    s += ld_real(v, 8);
    return *this;
  }
  LdRecord& r4(double v) {
    sep(false);
    s += ld_real(v, 4);
    return *this;
  }
};

// a record of character items only
LdRecord ld_chars(std::initializer_list<const char*> items) {
  LdRecord r;
  for (const char* it : items) r.c(it);
  return r;
}

struct File {
  FILE* f = nullptr;
  explicit File(const char* path) : f(path ? std::fopen(path, "w") : nullptr) {}
  ~File() {
    if (f) std::fclose(f);
  }
  void line(const std::string& s) { std::fputs((s + "\n").c_str(), f); }
  void line(const LdRecord& r) { line(r.s); }
};

}  // namespace

extern "C" {

int wtb_fortran_format(char kind, double x, int w, int d, char* out, int outlen) {
  if (!out || outlen < w + 1 || w < 1 || d < 0) return WTB_EBADARG;
  std::string s;
  if (kind == 'F')
    s = fortran_F(x, w, d);
  else if (kind == 'E')
    s = fortran_E(x, w, d);
  else if (kind == 'I')
    s = fortran_I((long)x, w, d);
  else if (kind == 'G' && w == 25 && d == 17)
    s = ld_real(x, 8);
  else if (kind == 'G' && w == 16 && d == 9)
    s = ld_real(x, 4);
  else
    return WTB_EBADARG;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return WTB_OK;
}

int wtb_write_bse_opt_diel(const char* path, int dim, const double* Ws, const double* acts, int pol) {
  if (!path || dim < 1 || !Ws || !acts) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t n = (size_t)dim;
  if (!pol) {
    f.line(ld_chars({"#", "  ", "exciton energy", "  ", "xx", "  ", "yy", "  ", "zz", " ", "xy", "  ", "xz", "  ", "yz"}));
    for (size_t i = 0; i < n; ++i) {
      std::string s = fortran_F(Ws[i], 15, 4);
      for (int c = 0; c < 6; ++c) s += fortran_F(acts[c * n + i], 15, 4);
      f.line(s);
    }
  } else {
    f.line(ld_chars({"#", "  ", "exciton energy", "  ", "xx", "  ", "yy", "  ", "zz", " ", "sp", "  ", "sm"}));
    const int cols[5] = {0, 1, 2, 6, 7};
    for (size_t i = 0; i < n; ++i) {
      std::string s = fortran_F(Ws[i], 15, 4);
      for (int c : cols) s += fortran_F(acts[c * n + i], 15, 4);
      f.line(s);
    }
  }
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_sp_optics(const char* path, int dimsp, const float* rec, int pol) {
  if (!path || dimsp < 1 || !rec) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t n = (size_t)dimsp;
  if (!pol)
    f.line(ld_chars({"#", "  ", "energy", "  ", "xx", "  ", "yy", "  ", "zz", "  ", "xy", "  ", "xz", "  ", "yz"}));
  else
    f.line(ld_chars({"#", "  ", "energy", "  ", "xx", "  ", "yy", "  ", "zz", "  ", "sp", "  ", "sm"}));
  const int c7[7] = {6, 7, 8, 9, 10, 11, 12}, c6[6] = {6, 7, 8, 9, 13, 14};
  for (size_t i = 0; i < n; ++i) {
    std::string s;
    if (!pol)
      for (int c : c7) s += fortran_F((double)rec[c * n + i], 15, 4);
    else
      for (int c : c6) s += fortran_F((double)rec[c * n + i], 15, 4);
    f.line(s);
  }
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_tm_coef(const char* path, int nk, int nc, int nv, const float* rec, int pol) {
  if (!path || nk < 1 || nc < 1 || nv < 1 || !rec) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t n = (size_t)nk * nc * nv;
  f.line(ld_chars({"number of kpoints:"}).i(nk));
  f.line(ld_chars({"number of conduction states"}).i(nc));
  f.line(ld_chars({"number of valence states"}).i(nv));
  if (!pol)
    f.line(ld_chars({"#", " ", "kx", " ", "ky", " ", "kz", " ", "nocp", " ", "nc", " ", "nv", "  ", "energy", "  ",
                     "xx", "  ", "yy", "  ", "zz", "  ", "xy", "  ", "xz", "  ", "yz"}));
  else
    f.line(ld_chars({"#", " ", "kx", " ", "ky", " ", "kz", " ", "nocp", " ", "nc", " ", "nv", "  ", "energy", "  ",
                     "xx", "  ", "yy", "  ", "zz", "  ", "sp", "  ", "sm"}));
  const int c7[7] = {6, 7, 8, 9, 10, 11, 12}, c6[6] = {6, 7, 8, 9, 13, 14};
  for (size_t i = 0; i < n; ++i) {
    std::string s;
    for (int c = 0; c < 3; ++c) s += fortran_F((double)rec[c * n + i], 10, 4);
    for (int c = 3; c < 6; ++c) s += fortran_I((long)rec[c * n + i], 10, 0);  // int() truncates
    if (!pol)
      for (int c : c7) s += fortran_F((double)rec[c * n + i], 10, 4);
    else
      for (int c : c6) s += fortran_F((double)rec[c * n + i], 10, 4);
    f.line(s);
  }
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_exc_wf(const char* path, int nk, int nc, int nv, const int* nocpk, const double* kpt, const double* q4,
                     int excnum, double energy, const double* ewf) {
  if (!path || nk < 1 || nc < 1 || nv < 1 || !nocpk || !kpt || !ewf) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t nkk = (size_t)nk;
  if (q4)  // excwfi2's momentum line: three REAL(4) list-directed items
    f.line(ld_chars({"#", " ", "excitonic momentum"}).r4(q4[1]).r4(q4[2]).r4(q4[3]));
  f.line(ld_chars({"#", " ", "excitonic state"}).i(excnum));
  f.line(ld_chars({"#", " ", "exciton energy:"}).r8(energy));
  f.line(ld_chars({"#", " ", "number occupied states"}).i(nocpk[0]).c("(not valid for metallic systems)"));
  f.line(ld_chars({"#", " ", "Number of conduction states", ""}).i(nc));
  f.line(ld_chars({"#", " ", "Number of valence states", ""}).i(nv));
  f.line(ld_chars({"#", " ", "Number of kpoints", ""}).i(nk));
  f.line(ld_chars({"#", " ", "nocpk", " ", "kx", " ", "ky", " ", "kz", " ", "nc", " ", "nv", " ", "re_wf", " ",
                   "imag_wf"}));
  size_t I = 0;
  for (int k = 0; k < nk; ++k)
    for (int c = 0; c < nc; ++c)
      for (int v = 0; v < nv; ++v, ++I) {
        const int no = nocpk[k];
        std::string s = fortran_I(no, 12, 1);
        for (int d = 0; d < 3; ++d) s += fortran_F(kpt[k + d * nkk], 15, 4);
        s += fortran_I(no + (nv + c + 1) - nv, 12, 1);  // nocp + stt(i,3) - nv
        s += fortran_I(no - nv + (v + 1), 12, 1);       // nocp - nv + stt(i,2)
        s += fortran_E(ewf[2 * I], 15, 4);
        s += fortran_E(ewf[2 * I + 1], 15, 4);
        f.line(s);
      }
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_exciton_lifetime(const char* path, int dim, const double* energy, const double* lft, int pol) {
  if (!path || dim < 1 || !energy || !lft) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t n = (size_t)dim;
  const int nout = pol ? 6 : 4;
  f.line(pol ? ld_chars({"#energy(eV) sum-lft(s)  x-lft(s) y-lft(s) z-lft(s) sp-lft(s) sm-lft(s)"})
             : ld_chars({"#energy(eV) sum-lft(s)  x-lft(s) y-lft(s) z-lft(s)"}));
  for (size_t i = 0; i < n; ++i) {
    std::string s = fortran_F(energy[i], 15, 4);
    for (int c = 0; c < nout; ++c) s += fortran_E(lft[c * n + i], 15, 4);
    f.line(s);
  }
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_diel(const char* path, int numbse, const double* dielf) {
  if (!path || numbse < 1 || !dielf) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t n = (size_t)numbse;
  f.line(ld_chars({"#", "  ", "energy", "  ", "real", "  ", "imag"}));
  for (size_t i = 0; i < n; ++i) f.line(LdRecord().r8(dielf[i]).r4(dielf[n + i]).r4(dielf[2 * n + i]));
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_bands_bse(const char* path, int nq, int dim, const double* qpath, const double* exk) {
  if (!path || nq < 1 || dim < 1 || !qpath || !exk) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  for (size_t b = 0; b < (size_t)dim; ++b) {
    for (size_t i = 0; i < (size_t)nq; ++i) f.line(LdRecord().r4(qpath[i]).r8(exk[i * (size_t)dim + b]));
    f.line(LdRecord());
  }
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_write_bz_act(const char* path, int nk, const double* kpt, const double* value) {
  if (!path || nk < 1 || !kpt || !value) return WTB_EBADARG;
  File f(path);
  if (!f.f) return WTB_EBADARG;
  const size_t n = (size_t)nk;
  for (size_t k = 0; k < n; ++k) f.line(LdRecord().r4(kpt[k]).r4(kpt[n + k]).r4(kpt[2 * n + k]).r8(value[k]));
  return std::ferror(f.f) ? WTB_EBADARG : WTB_OK;
}

int wtb_exciton_lifetime(wtb_ctx* c, const char* sysdim, const int* ngrid, int dim, const double* fosc, int pol,
                         double* lft) {
  if (!c) return WTB_EBADARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return WTB_ENODEV;
  if (!sysdim || !ngrid || dim < 1 || !fosc || !lft) return wtb::ctx_set_err(c, WTB_EBADARG, "bad arguments");
  int sd = 0;
  if (!std::strcmp(sysdim, "3D")) sd = 3;
  else if (!std::strcmp(sysdim, "2D")) sd = 2;
  else if (!std::strcmp(sysdim, "1D")) sd = 1;
  else return wtb::ctx_set_err(c, WTB_EBADARG, "Wrong System dimension");
  if (!c->have_hr) return wtb::ctx_set_err(c, WTB_ESTATE, "lattice not set (call wtb_set_hr first)");
  const double* r = c->rlat_rm;  // rows a1, a2, a3
  const double vx = r[1] * r[5] - r[2] * r[4], vy = r[2] * r[3] - r[0] * r[5], vz = r[0] * r[4] - r[1] * r[3];
  const double vc2d = std::sqrt(vx * vx + vy * vy + vz * vz);  // vcell2D
  const double ng = (double)(ngrid[0] * ngrid[1] * ngrid[2]);
  cudaError_t err = cudaSuccess;
  const int nin = pol ? 6 : 7, nout = pol ? 6 : 4;
  double* df = c->ws.get<double>("lft_in", (size_t)nin * dim, &err);
  double* dl = c->ws.get<double>("lft_out", (size_t)nout * dim, &err);
  if (err == cudaSuccess) err = cudaMemcpyAsync(df, fosc, sizeof(double) * nin * dim, cudaMemcpyHostToDevice, c->s);
  if (err == cudaSuccess) {
    wtb::lifetime_kernel<<<(dim + 255) / 256, 256, 0, c->s>>>(df, dim, pol ? 1 : 0, sd, ng, vc2d, r[0], dl);
    ++wtb::g_launch_count;
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpyAsync(lft, dl, sizeof(double) * nout * dim, cudaMemcpyDeviceToHost, c->s);
  if (err != cudaSuccess) return wtb::ctx_set_err(c, WTB_ECUDA, std::string("lifetime: ") + cudaGetErrorString(err));
  return wtb::ctx_check_status(c);
}

}  // extern "C"
