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
// List-directed records (the '#' header lines) are written as a blank followed by the character items with no
// separators, and integers in 12-character fields.
//   bse_opt_diel.dat / -pol   src/module_bse.F90:2132-2133, :2556-2567 (7F15.4 / 6F15.4)
//   sp_optics.dat / -pol      :2296-2297, :2366-2367 (7F15.4 / 6F15.4)
//   tm_coef.dat / -pol        :2300-2311, :2370-2377 (3F10.4,3I10.0,7F10.4 / ...,6F10.4)
//   exc_wf_<n>.dat            excwf2, :374-408 ((I,3F15.4,2I,2E15.4)); exc_wf_<n>_<q>.dat excwfi2, :412-448
//   exciton_lifetime.dat      lifetime, :3271-3349 ((1F15.4,4E15.4)); -pol: lifetimepol, :3353-3432 ((1F15.4,6E15.4))
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

// a list-directed record of character items: a leading blank, the items without separators
std::string ld_chars(std::initializer_list<const char*> items) {
  std::string s = " ";
  for (const char* it : items) s += it;
  return s;
}

// a list-directed 4-byte integer item
std::string ld_int(long v) { return fortran_I(v, 12, 1); }

// a list-directed REAL(8) item: 15 significant digits in a 25-character field
std::string ld_real8(double v) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%25.15G", v);
  return buf;
}

// a list-directed REAL(4) item: 7 significant digits in a 15-character field
std::string ld_real4(double v) {
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%15.7G", (double)(float)v);
  return buf;
}

struct File {
  FILE* f = nullptr;
  explicit File(const char* path) : f(path ? std::fopen(path, "w") : nullptr) {}
  ~File() {
    if (f) std::fclose(f);
  }
  void line(const std::string& s) { std::fputs((s + "\n").c_str(), f); }
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
  f.line(ld_chars({"number of kpoints:"}) + ld_int(nk));
  f.line(ld_chars({"number of conduction states"}) + ld_int(nc));
  f.line(ld_chars({"number of valence states"}) + ld_int(nv));
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
    f.line(ld_chars({"#", " ", "excitonic momentum"}) + ld_real4(q4[1]) + ld_real4(q4[2]) + ld_real4(q4[3]));
  f.line(ld_chars({"#", " ", "excitonic state"}) + ld_int(excnum));
  f.line(ld_chars({"#", " ", "exciton energy:"}) + ld_real8(energy));
  f.line(ld_chars({"#", " ", "number occupied states"}) + ld_int(nocpk[0]) + "(not valid for metallic systems)");
  f.line(ld_chars({"#", " ", "Number of conduction states", ""}) + ld_int(nc));
  f.line(ld_chars({"#", " ", "Number of valence states", ""}) + ld_int(nv));
  f.line(ld_chars({"#", " ", "Number of kpoints", ""}) + ld_int(nk));
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
